"""CPU oracle for the 3DMatch registration hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module.  It is the checker, never the thing measured or shipped.

* ``oracle.c`` (built into ``oracle/_build/liboracle.so`` by ``build()``) holds
  the C restatement of the reference's loops; this module binds it with ctypes.
* The numpy functions below restate the parts the reference writes in MATLAB
  or in its file formats:
    - PLY reader ............ core/demo.cu:69-93
    - keypts/desc writers ... core/demo.cu:236-255
    - .marvin tensor files .. core/marvin.hpp:2515-2530 (type ids),
                              2581-2612 (read), 2764-2790 (write)
    - Forsyth-Ponce rigid fit core/external/estimateRigidTransform/
                              estimateRigidTransform.m:23-72, quat2rot.m:10-25
    - registration metric ... evaluation/geometric-registration/external/
                              ElasticReconstruction/mrEvaluateRegistration.m
"""
from __future__ import annotations

import ctypes
import os
import platform
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.%s.so" % platform.machine())

NET_LAYERS = ["conv1", "conv2", "conv3", "conv4", "conv5", "conv6", "conv7", "conv8", "feat"]
NET_COUT = [64, 64, 128, 128, 256, 256, 512, 512, 512]
NET_CIN = [1, 64, 64, 128, 128, 256, 256, 512, 512]
NET_KS = [3, 3, 3, 3, 3, 3, 3, 3, 1]


def build(force: bool = False) -> str:
    """Compile oracle.c with gcc/OpenMP (no fused multiply-add contraction)."""
    src = os.path.join(HERE, "oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               src, "-o", tmp, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i32, i64, f32, u64 = ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_uint64
        sig = {
            "orc_num_threads": (i32, []),
            "orc_set_threads": (None, [i32]),
            "orc_keypoint_indices": (None, [u64, i32, i32, P]),
            "orc_ransac_sample": (None, [u64, ctypes.c_uint32, i32, P]),
            "orc_grid_setup": (None, [P, i32, f32, i32, P, P]),
            "orc_occupancy": (None, [P, i32, P, P, f32, P]),
            "orc_count_misdecoded": (i64, [P, i32]),
            "orc_tdf_range": (None, [P, P, f32, f32, i32, i64, i64, P]),
            "orc_tdf": (None, [P, P, f32, f32, i32, P]),
            "orc_keypoints": (None, [P, P, i32, P, f32, P, P]),
            "orc_gather": (None, [P, P, P, i32, P]),
            "orc_conv3d_f32": (None, [P, i32, i32, i32, P, P, i32, i32, i32, P]),
            "orc_conv3d_f64": (None, [P, i32, i32, i32, P, P, i32, i32, i32, P]),
            "orc_pool_f32": (None, [P, i32, i32, i32, P]),
            "orc_pool_f64": (None, [P, i32, i32, i32, P]),
            "orc_net_forward_f32": (None, [P, i32, P, P, i32, P]),
            "orc_net_forward_f64": (None, [P, i32, P, P, i32, P]),
            "orc_nn": (None, [P, i32, P, i32, i32, P]),
            "orc_mutual_nn": (i32, [P, i32, P, i32, i32, P, P, P]),
            "orc_kabsch": (i32, [P, P, P, i32, P, P]),
            "orc_kabsch3f": (i32, [P, P, P, P, P]),
            "orc_ransac_trial": (i32, [P, P, i32, u64, ctypes.c_uint32, f32, P, P]),
            "orc_ransac": (i32, [P, P, i32, u64, i32, f32, P, P, P, P]),
            "orc_ransac_adaptive_stop": (i32, [P, i32, i32, i32, P]),
            "orc_tsdf_integrate": (None, [P, P, P, i32, i32, P, P, f32, f32, P, P]),
            "orc_tsdf_integrate_z": (None, [P, P, P, i32, i32, P, P, f32, f32, i32, i32, P, P]),
            "orc_extract_surface": (i64, [P, P, P, P, f32, f32, f32, P]),
            "orc_overlap": (None, [P, i32, P, i32, P, f32, P]),
            "orc_tdf_exact": (None, [P, i32, P, P, f32, f32, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def num_threads() -> int:
    return lib().orc_num_threads()


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


# --------------------------------------------------------------------------
# File formats
# --------------------------------------------------------------------------
def read_ply(path: str) -> np.ndarray:
    """core/demo.cu:69-93: skip 7 text lines, vertex count is the third token
    of line 3, then N*3 little-endian float32."""
    with open(path, "rb") as f:
        n = 0
        for i in range(7):
            line = f.readline()
            if i == 2:
                tok = line.split()
                n = int(tok[2]) if len(tok) >= 3 else 0
        if n == 0:
            raise ValueError("third line of the .ply does not give the vertex count")
        data = np.frombuffer(f.read(12 * n), dtype="<f4")
    if data.size != 3 * n:
        raise ValueError("truncated .ply: %d of %d floats" % (data.size, 3 * n))
    return data.reshape(n, 3).copy()


def write_ply(path: str, pts: np.ndarray) -> None:
    """Binary PLY with the 7-line header core/utils.hpp:36-43 writes."""
    pts = np.ascontiguousarray(pts, dtype="<f4")
    hdr = ("ply\nformat binary_little_endian 1.0\nelement vertex %d\nproperty float x\n"
           "property float y\nproperty float z\nend_header\n" % pts.shape[0])
    with open(path, "wb") as f:
        f.write(hdr.encode())
        f.write(pts.tobytes())


def read_keypts_bin(path: str) -> np.ndarray:
    """core/demo.cu:236-244: float K, then K*3 float."""
    d = np.fromfile(path, dtype="<f4")
    k = int(d[0])
    return d[1:1 + 3 * k].reshape(k, 3)


def read_desc_bin(path: str) -> np.ndarray:
    """core/demo.cu:246-255: float K, float 512, then K*512 float."""
    d = np.fromfile(path, dtype="<f4")
    k, n = int(d[0]), int(d[1])
    return d[2:2 + k * n].reshape(k, n)


_TYPE_IDS = {0: np.float16, 1: np.float32, 2: np.float64, 3: np.uint8, 4: np.uint16, 5: np.uint32,
             6: np.uint64, 7: np.int8, 8: np.int16, 9: np.int32, 10: np.int64}


def read_marvin(path: str) -> dict:
    """Repeated {u8 typeid; u32 sizeof; i32 nameLen; name; i32 nDims; i32 dims[];
    data} records (core/marvin.hpp:2581-2612).  Returns name -> float32 array."""
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0
    while pos < len(buf):
        tid, tsz = struct.unpack_from("<BI", buf, pos)
        pos += 5
        if tid not in _TYPE_IDS or np.dtype(_TYPE_IDS[tid]).itemsize != tsz:
            raise ValueError("unsupported tensor type id %d / sizeof %d" % (tid, tsz))
        (ln,) = struct.unpack_from("<i", buf, pos)
        pos += 4
        name = buf[pos:pos + ln].decode()
        pos += ln
        (nd,) = struct.unpack_from("<i", buf, pos)
        pos += 4
        dims = struct.unpack_from("<%di" % nd, buf, pos)
        pos += 4 * nd
        count = int(np.prod(dims)) if nd else 0
        arr = np.frombuffer(buf, dtype=np.dtype(_TYPE_IDS[tid]).newbyteorder("<"), count=count, offset=pos)
        pos += count * tsz
        out[name] = arr.astype(np.float32).reshape(dims)
    return out


def write_marvin(path: str, tensors: dict, dtype=np.float32) -> None:
    """Write tensors in the record format of core/marvin.hpp:2764-2790."""
    tid = {np.float16: 0, np.float32: 1, np.float64: 2}[dtype]
    with open(path, "wb") as f:
        for name, a in tensors.items():
            a = np.ascontiguousarray(a, dtype=dtype)
            nb = name.encode()
            f.write(struct.pack("<BIi", tid, np.dtype(dtype).itemsize, len(nb)))
            f.write(nb)
            f.write(struct.pack("<i", a.ndim))
            f.write(struct.pack("<%di" % a.ndim, *a.shape))
            f.write(a.astype(np.dtype(dtype).newbyteorder("<")).tobytes())


def he_normal_weights(seed: int, bias_scale: float = 0.05) -> dict:
    """Seeded He-normal weights in Marvin's names and shapes
    ([K,C,3,3,3] weights, [1,K,1,1,1] biases), small uniform biases."""
    rng = np.random.default_rng(seed)
    w = {}
    for name, k, c, ks in zip(NET_LAYERS, NET_COUT, NET_CIN, NET_KS):
        fan_in = c * ks ** 3
        w[name + ".weight"] = (rng.standard_normal((k, c, ks, ks, ks)) * np.sqrt(2.0 / fan_in)).astype(np.float32)
        w[name + ".bias"] = rng.uniform(-bias_scale, bias_scale, (1, k, 1, 1, 1)).astype(np.float32)
    return w


# --------------------------------------------------------------------------
# TDF / keypoints / gather
# --------------------------------------------------------------------------
def grid_setup(pts: np.ndarray, voxel_size: float = 0.01, pad: int = 15):
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    dim = np.zeros(3, np.int32)
    origin = np.zeros(3, np.float32)
    lib().orc_grid_setup(_p(pts), pts.shape[0], voxel_size, pad, _p(dim), _p(origin))
    return dim, origin


def occupancy(pts, dim, origin, voxel_size):
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    occ = np.zeros(int(np.prod(dim.astype(np.int64))), np.uint8)
    lib().orc_occupancy(_p(pts), pts.shape[0], _p(dim), _p(origin), voxel_size, _p(occ))
    return occ


def count_misdecoded(dim, mode: int) -> int:
    dim = np.ascontiguousarray(dim, dtype=np.int32)
    return int(lib().orc_count_misdecoded(_p(dim), mode))


def tdf(occ, dim, voxel_size, trunc, mode=0, v0=0, v1=None):
    dim = np.ascontiguousarray(dim, dtype=np.int32)
    V = int(np.prod(dim.astype(np.int64)))
    v1 = V if v1 is None else v1
    out = np.zeros(v1 - v0, np.float32)
    lib().orc_tdf_range(_p(occ), _p(dim), voxel_size, trunc, mode, v0, v1, _p(out))
    return out


def keypoint_indices(seed: int, n_pts: int, k: int) -> np.ndarray:
    idx = np.zeros(k, np.int32)
    lib().orc_keypoint_indices(seed, n_pts, k, _p(idx))
    return idx


def keypoints(pts, idx, origin, voxel_size):
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    kp = np.zeros((idx.size, 3), np.float32)
    kg = np.zeros((idx.size, 3), np.int32)
    lib().orc_keypoints(_p(pts), _p(idx), idx.size, _p(origin), voxel_size, _p(kp), _p(kg))
    return kp, kg


def gather(tdf_grid, dim, kp_grid):
    kp_grid = np.ascontiguousarray(kp_grid, dtype=np.int32)
    out = np.zeros((kp_grid.shape[0], 27000), np.float32)
    lib().orc_gather(_p(tdf_grid), _p(np.ascontiguousarray(dim, np.int32)), _p(kp_grid), kp_grid.shape[0], _p(out))
    return out


# --------------------------------------------------------------------------
# Net
# --------------------------------------------------------------------------
def _weight_ptrs(weights: dict):
    ws = [np.ascontiguousarray(weights[n + ".weight"], np.float32).reshape(-1) for n in NET_LAYERS]
    bs = [np.ascontiguousarray(weights[n + ".bias"], np.float32).reshape(-1) for n in NET_LAYERS]
    wp = (ctypes.c_void_p * 9)(*[w.ctypes.data for w in ws])
    bp = (ctypes.c_void_p * 9)(*[b.ctypes.data for b in bs])
    return ws, bs, wp, bp


def net_forward(patches: np.ndarray, weights: dict, use_feat: bool = True, f64: bool = False) -> np.ndarray:
    """Direct-loop forward of core/3dmatch-net-test.json on B patches [B,27000]."""
    patches = np.ascontiguousarray(patches, dtype=np.float32).reshape(-1, 27000)
    keep = _weight_ptrs(weights)
    B = patches.shape[0]
    out = np.zeros((B, 512), np.float64 if f64 else np.float32)
    fn = lib().orc_net_forward_f64 if f64 else lib().orc_net_forward_f32
    fn(_p(patches), B, ctypes.cast(keep[2], ctypes.c_void_p), ctypes.cast(keep[3], ctypes.c_void_p),
       1 if use_feat else 0, _p(out))
    return out


def round_bf16(x) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x, np.float32))
    return t.to(torch.bfloat16).to(torch.float64).numpy()


def round_e4m3(x) -> np.ndarray:
    """Round to FP8 E4M3 (nearest, ties to even, saturating at +-448, as the
    cvt.rn.satfinite conversion), returned as float64."""
    import torch
    t = torch.from_numpy(np.clip(np.asarray(x, np.float32), -448.0, 448.0))
    return t.to(torch.float8_e4m3fn).to(torch.float64).numpy()


def net_layer_quantized(x: np.ndarray, weights: dict, l: int, fp8_in: bool = False, in_scale: float = 1.0,
                        out: str = "bf16", out_scale: float = 1.0) -> np.ndarray:
    """One layer (index l: 0..8 = conv1..conv8, feat) of the tensor-core forms
    restated in float64, on stored input values x ([B, D, D, D, C] channels-
    last: BF16 values, or E4M3 codes times in_scale when fp8_in).

    BF16 layer: BF16 weights.  E4M3 layer: weights are the E4M3 codes of
    w / s_k with s_k = max|w_k| / 448 per output channel (float32), inputs
    the E4M3 codes of x / in_scale, and the sum is scaled by in_scale * s_k.
    Then bias, ReLU (not for feat), and the stored output: "bf16" (rounded to
    BF16), "e4m3" (E4M3 codes of y / out_scale, returned times out_scale), or
    "f32" (feat's float output).  Sums are exact in float64; the GPU adds in
    FP32, so the two differ by at most one rounding step of the stored output
    on a few elements."""
    name = NET_LAYERS[l]
    K, ks = NET_COUT[l], NET_KS[l]
    B, D, C = x.shape[0], x.shape[1], x.shape[4]
    Do = D - ks + 1
    w = np.ascontiguousarray(weights[name + ".weight"], np.float32).reshape(K, -1)
    bias = np.ascontiguousarray(weights[name + ".bias"], np.float32).reshape(-1).astype(np.float64)
    if fp8_in:
        s_w = (np.abs(w).max(axis=1) / np.float32(448.0)).astype(np.float32)
        s_w[s_w == 0] = 1.0
        wq = round_e4m3(w / s_w[:, None]).astype(np.float32)
        scale = (np.float32(in_scale) * s_w).astype(np.float32).astype(np.float64)
        xin = round_e4m3(np.asarray(x, np.float64) / in_scale)
    else:
        wq = round_bf16(w).astype(np.float32)
        scale = np.ones(K)
        xin = round_bf16(x) if l == 0 else np.asarray(x, np.float64)
    y = np.zeros((B, Do, Do, Do, K))
    zb = np.zeros(K, np.float32)
    lib().orc_conv3d_f64(_p(np.ascontiguousarray(xin)), B, D, C, _p(np.ascontiguousarray(wq)), _p(zb), K, ks, 0,
                         _p(y))
    v = y * scale + bias
    if l < 8:
        v = np.maximum(v, 0.0)
    if out == "f32":
        return v
    if out == "e4m3":
        qinv = np.float32(1.0) / np.float32(out_scale)
        return round_e4m3(v.astype(np.float32) * qinv) * out_scale
    return round_bf16(v)


def pool_max(x: np.ndarray) -> np.ndarray:
    """2^3 max-pool, stride 2, of [B, D, D, D, C] values (core/marvin.hpp:5577)."""
    B, D, C = x.shape[0], x.shape[1], x.shape[4]
    z = np.zeros((B, D // 2, D // 2, D // 2, C))
    lib().orc_pool_f64(_p(np.ascontiguousarray(x, np.float64)), B, D, C, _p(z))
    return z


def net_forward_quantized(patches: np.ndarray, weights: dict, fp8_layers=(), act_scales=None, want=None):
    """The whole net through net_layer_quantized: BF16 everywhere, E4M3
    operands for the layers in `fp8_layers` (2..7 = conv3..conv8) with
    act_scales[l] the scale of layer l's E4M3 input.  Returns the descriptors,
    or (descriptors, {name: stored response values}) for the names in `want`.
    Because every stored rounding turns a tiny difference of the sums into a
    whole rounding step now and then, and later layers spread it, this whole-
    net restatement and the GPU drift apart by about one rounding step (BF16
    ~3e-3, E4M3 ~5e-2) over the nine layers: kernels are checked layer by
    layer on the GPU's own inputs, the whole forward against FP64."""
    fp8 = set(int(l) for l in fp8_layers)
    assert fp8 <= set(range(2, 8)), "E4M3 layers are conv3..conv8 (2..7)"
    x = np.ascontiguousarray(patches, np.float32).reshape(-1, 30, 30, 30, 1).astype(np.float64)
    resp = {}
    for l, name in enumerate(NET_LAYERS):
        nxt = l + 1
        out = "f32" if l == 8 else ("e4m3" if nxt in fp8 else "bf16")
        x = net_layer_quantized(x, weights, l, l in fp8, act_scales[l] if l in fp8 else 1.0, out,
                                act_scales[nxt] if nxt in fp8 else 1.0)
        if want and name in want:
            resp[name] = x.copy()
        if l == 1:
            x = pool_max(x)
            if want and "pool1" in want:
                resp["pool1"] = x.copy()
    desc = x.reshape(x.shape[0], 512)
    return (desc, resp) if want else desc


def fp8_act_scales(patches: np.ndarray, weights: dict) -> np.ndarray:
    """The E4M3 activation scales the FP8 form calibrates: for l = 2..7 the
    largest value of layer l-1's BF16-form response (conv2..conv7) over the
    calibration patches, divided by 448; index l = the layer that reads it."""
    _, r = net_forward_quantized(patches, weights, want=["conv2", "conv3", "conv4", "conv5", "conv6", "conv7"])
    sc = np.ones(9, np.float32)
    for l, name in zip(range(2, 8), ["conv2", "conv3", "conv4", "conv5", "conv6", "conv7"]):
        m = np.float32(r[name].max())
        sc[l] = (m if m > 0 else np.float32(1.0)) / np.float32(448.0)
    return sc


# --------------------------------------------------------------------------
# Matching and registration
# --------------------------------------------------------------------------
def tdf_exact(pts: np.ndarray, dim, origin, vs, trunc):
    """pointCloud2TDF.m restated (double distances), x fastest."""
    pts = np.ascontiguousarray(pts, np.float32)
    d = np.ascontiguousarray(dim, np.int32)
    o = np.ascontiguousarray(origin, np.float32)
    out = np.zeros(int(d[0]) * int(d[1]) * int(d[2]), np.float32)
    lib().orc_tdf_exact(_p(pts), pts.shape[0], _p(d), _p(o), vs, trunc, _p(out))
    return out


def overlap(a: np.ndarray, b: np.ndarray, rt, radius=0.05):
    """(points of a near Rt*b, points of Rt*b near a): register2Fragments.m:90-97."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    r = np.ascontiguousarray(np.asarray(rt, np.float64).reshape(-1)[:12])
    c = np.zeros(2, np.int32)
    lib().orc_overlap(_p(a), a.shape[0], _p(b), b.shape[0], _p(r), radius, _p(c))
    return int(c[0]), int(c[1])


def mutual_nn(da: np.ndarray, db: np.ndarray):
    da = np.ascontiguousarray(da, np.float32)
    db = np.ascontiguousarray(db, np.float32)
    na, nb, dim = da.shape[0], db.shape[0], da.shape[1]
    nn_ab = np.zeros(na, np.int32)
    nn_ba = np.zeros(nb, np.int32)
    pairs = np.zeros((min(na, nb), 2), np.int32)
    m = lib().orc_mutual_nn(_p(da), na, _p(db), nb, dim, _p(nn_ab), _p(nn_ba), _p(pairs))
    return pairs[:m].copy(), nn_ab, nn_ba


def ransac_sample(seed: int, h: int, m: int):
    out = np.zeros(3, np.int32)
    lib().orc_ransac_sample(seed, h, m, _p(out))
    return out


def kabsch3f(x: np.ndarray, y: np.ndarray, idx):
    """RANSAC's FP32 three-point fit (x = R y + t) on correspondences idx[0..2]."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    idx = np.ascontiguousarray(idx, np.int32)
    R = np.zeros(9, np.float32)
    t = np.zeros(3, np.float32)
    if lib().orc_kabsch3f(_p(x), _p(y), _p(idx), _p(R), _p(t)) != 0:
        raise ValueError("degenerate fit")
    return R.reshape(3, 3), t


def kabsch(x: np.ndarray, y: np.ndarray, idx=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    R = np.zeros(9)
    t = np.zeros(3)
    if idx is None:
        rc = lib().orc_kabsch(_p(x), _p(y), None, x.shape[0], _p(R), _p(t))
    else:
        idx = np.ascontiguousarray(idx, np.int32)
        rc = lib().orc_kabsch(_p(x), _p(y), _p(idx), idx.size, _p(R), _p(t))
    if rc != 0:
        raise ValueError("degenerate fit")
    return R.reshape(3, 3), t


def ransac(x, y, seed: int, iters: int, thr: float = 0.05, want_counts: bool = False):
    """Fixed-trial RANSAC with the product's sampling stream.  x = R y + t."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    m = x.shape[0]
    counts = np.zeros(iters, np.int32) if want_counts else None
    best = np.zeros(1, np.int32)
    inl = np.zeros(m, np.int32)
    Rt = np.zeros(12)
    n = lib().orc_ransac(_p(x), _p(y), m, seed, iters, thr, _p(counts) if want_counts else None, _p(best),
                         _p(inl), _p(Rt))
    res = {"Rt": Rt.reshape(3, 4), "inliers": inl[:n].copy(), "best_trial": int(best[0])}
    if want_counts:
        res["counts"] = counts
    return res


def ransac_adaptive_stop(counts: np.ndarray, m: int, max_trials: int = 50000):
    counts = np.ascontiguousarray(counts, np.int32)
    best = np.zeros(1, np.int32)
    n = lib().orc_ransac_adaptive_stop(_p(counts), counts.size, m, max_trials, _p(best))
    return n, int(best[0])


def estimate_rigid_transform_fp(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Forsyth-Ponce quaternion fit of estimateRigidTransform.m:23-72: x = T y.
    x, y: 3xN.  Returns the 4x4 T."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n = x.shape[1]
    xc = x.sum(axis=1) / n
    yc = y.sum(axis=1) / n
    xz = x - xc[:, None]
    yz = y - yc[:, None]
    B = np.zeros((4, 4))
    for i in range(n):
        d = yz[:, i] - xz[:, i]
        s = yz[:, i] + xz[:, i]
        A = np.zeros((4, 4))
        A[0, 1:] = d
        A[1:, 0] = -d
        A[1:, 1:] = np.array([[0, -s[2], s[1]], [s[2], 0, -s[0]], [-s[1], s[0], 0]])
        B += A.T @ A
    _, _, vt = np.linalg.svd(B)
    q = vt[-1]
    q0, q1, q2, q3 = q
    R = np.array([
        [q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3, 2 * (q1 * q2 - q0 * q3), 2 * (q1 * q3 + q0 * q2)],
        [2 * (q1 * q2 + q0 * q3), q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3, 2 * (q2 * q3 - q0 * q1)],
        [2 * (q1 * q3 - q0 * q2), 2 * (q2 * q3 + q0 * q1), q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3]])
    T1 = np.eye(4); T1[:3, 3] = -yc
    T2 = np.eye(4); T2[:3, :3] = R
    T3 = np.eye(4); T3[:3, 3] = xc
    return T3 @ T2 @ T1


# --------------------------------------------------------------------------
# TSDF
# --------------------------------------------------------------------------
def tsdf_integrate(K, cam2base, depth, dim, origin, vs, trunc, tsdf_grid, weight, z0=0, z1=0):
    """One frame of depth-fusion/demo.cu:18-68 into the full grids (voxel
    slices z0 <= z < z1 only, when z1 > 0)."""
    K = np.ascontiguousarray(K, np.float32).reshape(9)
    c2b = np.ascontiguousarray(cam2base, np.float32).reshape(16)
    depth = np.ascontiguousarray(depth, np.float32)
    H, W = depth.shape
    lib().orc_tsdf_integrate_z(_p(K), _p(c2b), _p(depth), H, W, _p(np.ascontiguousarray(dim, np.int32)),
                               _p(np.ascontiguousarray(origin, np.float32)), vs, trunc, z0, z1, _p(tsdf_grid),
                               _p(weight))


def extract_surface(tsdf_grid, weight, dim, origin, vs, tsdf_thr=0.2, w_thr=1.0):
    dim = np.ascontiguousarray(dim, np.int32)
    origin = np.ascontiguousarray(origin, np.float32)
    n = lib().orc_extract_surface(_p(tsdf_grid), _p(weight), _p(dim), _p(origin), vs, tsdf_thr, w_thr, None)
    pts = np.zeros((max(n, 1), 3), np.float32)
    lib().orc_extract_surface(_p(tsdf_grid), _p(weight), _p(dim), _p(origin), vs, tsdf_thr, w_thr, _p(pts))
    return pts[:n]


# --------------------------------------------------------------------------
# Registration metric (mrEvaluateRegistration.m)
# --------------------------------------------------------------------------
def read_log(path: str):
    """.log trajectory: records of 'i j n' followed by a 4x4 matrix."""
    recs = []
    with open(path) as f:
        lines = [l for l in f.read().split("\n") if l.strip()]
    for k in range(0, len(lines) - 4, 5):
        info = [int(v) for v in lines[k].split()[:3]]
        mat = np.array([[float(v) for v in lines[k + r].split()] for r in range(1, 5)])
        recs.append((info, mat))
    return recs


def read_info(path: str):
    """.info: records of 'i j n' followed by a 6x6 matrix."""
    recs = []
    with open(path) as f:
        lines = [l for l in f.read().split("\n") if l.strip()]
    for k in range(0, len(lines) - 6, 7):
        info = [int(v) for v in lines[k].split()[:3]]
        mat = np.array([[float(v) for v in lines[k + r].split()] for r in range(1, 7)])
        recs.append((info, mat))
    return recs


def _dcm2quat(R):
    q0 = 0.5 * np.sqrt(1 + R[0, 0] + R[1, 1] + R[2, 2])
    return np.array([q0, -(R[2, 1] - R[1, 2]) / (4 * q0), -(R[0, 2] - R[2, 0]) / (4 * q0),
                     -(R[1, 0] - R[0, 1]) / (4 * q0)])


def evaluate_registration(result, gt, gt_info, err2=0.04):
    """Recall / precision of mrEvaluateRegistration.m:1-43."""
    num = gt[0][0][2]
    mask = {}
    gt_num = 0
    for i, (info, _) in enumerate(gt):
        if info[1] - info[0] > 1:
            mask[info[0] + info[1] * num] = i
            gt_num += 1
    rs_num = good = 0
    for info, trans in result:
        if info[1] - info[0] > 1:
            rs_num += 1
            idx = mask.get(info[0] + info[1] * num)
            if idx is not None:
                T = np.linalg.solve(gt[idx][1], trans)
                q = _dcm2quat(T[:3, :3])
                er = np.concatenate([T[:3, 3], -q[1:]])
                M = gt_info[idx][1]
                p = er @ M @ er / M[0, 0]
                if p <= err2:
                    good += 1
    return good / gt_num, (good / rs_num if rs_num else 0.0)


# --------------------------------------------------------------------------
# ICP (the register2Fragments.m:70-78 refinement): numpy FP64 restatement of
# the library's algorithm, for parity tests.
# --------------------------------------------------------------------------
def _grid_average(p, cell):
    k = np.floor(p.astype(np.float32) / np.float32(cell)).astype(np.int64)
    _, inv, n = np.unique(k, axis=0, return_inverse=True, return_counts=True)
    s = np.zeros((n.size, 3))
    np.add.at(s, inv.ravel(), p.astype(np.float64))
    return (s / n[:, None]).astype(np.float32)


def icp(fixed, moving, init, grid=0.01, max_dist=0.10, inlier_ratio=0.30, iterations=1):
    """Grid-average both clouds; per iteration: nearest fixed point within
    max_dist of each moved point, the pairs in the 4,096-bin d^2 histogram
    up to the bin reaching ceil(ratio * pairs), Kabsch (SVD) of those."""
    from scipy.spatial import cKDTree
    A, B = _grid_average(fixed, grid), _grid_average(moving, grid)
    tree = cKDTree(A.astype(np.float64))
    T = np.asarray(init, np.float64).reshape(-1)[:12].reshape(3, 4).copy()
    md2 = np.float32(max_dist) * np.float32(max_dist)
    for _ in range(iterations):
        # moved points and squared distances in float32 with the library's
        # operation order, so the histogram bins agree
        Tf = T.astype(np.float32)
        m = np.stack([((Tf[r, 0] * B[:, 0] + Tf[r, 1] * B[:, 1]) + Tf[r, 2] * B[:, 2]) + Tf[r, 3] for r in range(3)],
                     1).astype(np.float32)
        _, j = tree.query(m.astype(np.float64), distance_upper_bound=float(max_dist) * 1.001)
        found = j < A.shape[0]
        jj = np.where(found, j, 0)
        e = m - A[jj]
        d2 = (e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1]) + e[:, 2] * e[:, 2]
        ok = found & (d2 < md2)
        if ok.sum() < 3:
            break
        b = np.minimum(4095, ((d2[ok] / md2) * np.float32(4096)).astype(np.int64))
        hist = np.bincount(b, minlength=4096)
        want = max(3, int(np.ceil(inlier_ratio * ok.sum())))
        bmax = int(np.searchsorted(np.cumsum(hist), want))
        sel = np.flatnonzero(ok)[b <= bmax]
        x, y = A[jj[sel]].astype(np.float64), m[sel].astype(np.float64)
        cx, cy = x.mean(0), y.mean(0)
        U, _, Vt = np.linalg.svd((y - cy).T @ (x - cx))
        D = np.diag([1.0, 1.0, np.sign(np.linalg.det(Vt.T @ U.T))])
        R = Vt.T @ D @ U.T
        t = cx - R @ cy
        T = np.concatenate([R @ T[:, :3], (R @ T[:, 3] + t)[:, None]], 1)
    out = np.eye(4)
    out[:3] = T
    return out
