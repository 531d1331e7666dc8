"""Python host binding of libtdm (the GB300 3DMatch registration hot path).

Mirrors the reference's demo interface (core/demo.cu) and Marvin's net calls
over the C ABI of include/tdm.h.  Device buffers are torch CUDA tensors (torch
is used only for device memory and streams).  There is no CPU fallback: if the
compiled library is missing, loading fails loudly.

The directory name is not a Python identifier; load it with
``importlib.util.spec_from_file_location`` (see ``load()`` in
``__graft_entry__.py``).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libtdm.so")

TDM_FP32, TDM_BF16, TDM_FP8 = 0, 1, 2
PRECISIONS = {"fp32": TDM_FP32, "bf16": TDM_BF16, "fp8": TDM_FP8}
TDF_EXACT, TDF_REFCOMPAT_FLOAT, TDF_REFCOMPAT_FMA = 0, 1, 2
STATUS = {0: "OK", 1: "INVALID_ARG", 2: "IO", 3: "FORMAT", 4: "OOM", 5: "DEVICE", 6: "TIMEOUT", 7: "CANCELLED",
          8: "UNSUPPORTED"}

# Every symbol include/tdm.h declares (checked by the CPU tests).
EXPORTS = [
    "tdm_version", "tdm_last_error", "tdm_device_status", "tdm_launch_count", "tdm_selftest_wait_timeout",
    "tdm_grid_from_points_host", "tdm_grid_workspace_bytes", "tdm_grid_from_points",
    "tdm_tdf_workspace_bytes", "tdm_tdf",
    "tdm_keypoint_indices", "tdm_keypoints", "tdm_gather",
    "tdm_net_create", "tdm_net_create_from_host", "tdm_net_forward", "tdm_net_response", "tdm_net_set_max_batch",
    "tdm_net_set_timing", "tdm_net_layer_times", "tdm_net_calibrate", "tdm_net_act_scales", "tdm_net_destroy",
    "tdm_write_seeded_weights",
    "tdm_mnn_workspace_bytes", "tdm_match_mnn",
    "tdm_ransac_workspace_bytes", "tdm_ransac", "tdm_ransac_noalloc", "tdm_pairs_to_points",
    "tdm_tsdf_init", "tdm_depth_from_mm", "tdm_tsdf_integrate", "tdm_extract_workspace_bytes", "tdm_tsdf_extract",
    "tdm_pipeline_create", "tdm_pipeline_destroy", "tdm_describe_fragment", "tdm_register_pair",
    "tdm_register_pair_host", "tdm_net_clone", "tdm_net_workspace_bytes",
    "tdm_server_create", "tdm_server_slots", "tdm_server_submit", "tdm_server_wait", "tdm_server_destroy",
    "tdm_server_submit_pair", "tdm_server_cancel", "tdm_server_get_stats",
    "tdm_store_create", "tdm_store_destroy", "tdm_store_describe", "tdm_store_put", "tdm_store_get",
    "tdm_store_remove", "tdm_store_get_stats", "tdm_register_stored",
    "tdm_net_autotune", "tdm_net_tiles", "tdm_net_set_tile", "tdm_net_tile_forms", "tdm_net_set_tile_form",
    "tdm_batch_create", "tdm_batch_destroy", "tdm_batch_device_bytes", "tdm_describe_batch", "tdm_batch_stats",
    "tdm_overlap_workspace_bytes", "tdm_overlap", "tdm_tdf_exact", "tdm_icp_workspace_bytes", "tdm_icp",
]


class TdmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Grid(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32 * 3), ("origin", ctypes.c_float * 3), ("voxel_size", ctypes.c_float),
                ("trunc_margin", ctypes.c_float)]

    @property
    def voxels(self) -> int:
        return int(self.dim[0]) * int(self.dim[1]) * int(self.dim[2])

    def as_tuple(self):
        return (tuple(self.dim), tuple(self.origin), self.voxel_size, self.trunc_margin)


class RansacParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("iterations", ctypes.c_int32), ("threshold", ctypes.c_float),
                ("adaptive", ctypes.c_int32), ("max_trials", ctypes.c_int32)]


class PipelineConfig(ctypes.Structure):
    _fields_ = [("voxel_size", ctypes.c_float), ("trunc_voxels", ctypes.c_float), ("pad", ctypes.c_int32),
                ("max_points", ctypes.c_int32), ("max_keypoints", ctypes.c_int32), ("max_voxels", ctypes.c_int64),
                ("match_precision", ctypes.c_int32), ("ransac", RansacParams)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("max_fragments", ctypes.c_int32), ("max_points", ctypes.c_int64), ("max_keypoints", ctypes.c_int64),
                ("max_voxels", ctypes.c_int64), ("trunc_voxels", ctypes.c_float), ("pad", ctypes.c_int32),
                ("use_graph", ctypes.c_int32)]


class IcpParams(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_float), ("max_dist", ctypes.c_float), ("inlier_ratio", ctypes.c_float),
                ("max_iterations", ctypes.c_int32), ("tol_translation", ctypes.c_float),
                ("tol_rotation_deg", ctypes.c_float)]


class IcpResult(ctypes.Structure):
    _fields_ = [("rt", ctypes.c_double * 12), ("iterations", ctypes.c_int32), ("correspondences", ctypes.c_int32),
                ("rmse", ctypes.c_float), ("converged", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("pipeline", PipelineConfig), ("slots", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("store_bytes", ctypes.c_int64)]


class Fragment(ctypes.Structure):
    _fields_ = [("key", ctypes.c_uint64), ("pts", ctypes.c_void_p), ("n", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("k", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("requests_done", ctypes.c_int64), ("requests_cancelled", ctypes.c_int64), ("waves", ctypes.c_int64),
                ("fragments_described", ctypes.c_int64), ("store_hits", ctypes.c_int64),
                ("store_entries", ctypes.c_int64), ("max_wave_requests", ctypes.c_int64),
                ("device_bytes", ctypes.c_int64), ("describe_ms", ctypes.c_double), ("match_ms", ctypes.c_double),
                ("overlap_ms", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class StoreStats(ctypes.Structure):
    _fields_ = [("entries", ctypes.c_int64), ("bytes_used", ctypes.c_int64), ("capacity", ctypes.c_int64),
                ("hits", ctypes.c_int64), ("misses", ctypes.c_int64), ("evictions", ctypes.c_int64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class PairResult(ctypes.Structure):
    _fields_ = [("rt", ctypes.c_double * 16), ("n_matches", ctypes.c_int32), ("n_inliers", ctypes.c_int32),
                ("best_trial", ctypes.c_int32), ("keypoints", ctypes.c_int32 * 2),
                ("grid_dim", (ctypes.c_int32 * 3) * 2)]


_lib = None


def lib():
    """The loaded libtdm.so with argument types set.  Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libtdm.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P, i32, i64, f32, u64, sz = (ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_uint64,
                                 ctypes.c_size_t)
    G = ctypes.POINTER(Grid)
    sig = {
        "tdm_version": (ctypes.c_char_p, []),
        "tdm_last_error": (ctypes.c_char_p, []),
        "tdm_device_status": (i32, [P]),
        "tdm_launch_count": (i64, []),
        "tdm_selftest_wait_timeout": (i32, [ctypes.c_uint32, P, P]),
        "tdm_grid_from_points_host": (i32, [P, i32, f32, f32, i32, G]),
        "tdm_grid_workspace_bytes": (sz, []),
        "tdm_grid_from_points": (i32, [P, i32, f32, f32, i32, G, P, P]),
        "tdm_tdf_workspace_bytes": (sz, [G]),
        "tdm_tdf": (i32, [P, i32, G, i32, P, P, sz, P]),
        "tdm_keypoint_indices": (i32, [u64, i32, i32, P, P]),
        "tdm_keypoints": (i32, [P, i32, P, i32, G, P, P, P]),
        "tdm_gather": (i32, [P, G, P, i32, P, P]),
        "tdm_net_create": (i32, [ctypes.c_char_p, i32, i32, ctypes.POINTER(P)]),
        "tdm_net_create_from_host": (i32, [P, P, i32, i32, ctypes.POINTER(P)]),
        "tdm_net_forward": (i32, [P, P, i32, P, P]),
        "tdm_net_response": (i32, [P, ctypes.c_char_p, P, i32, P, P]),
        "tdm_net_set_max_batch": (i32, [P, i32]),
        "tdm_net_set_timing": (i32, [P, i32]),
        "tdm_net_calibrate": (i32, [P, P, i32, P]),
        "tdm_net_act_scales": (i32, [P, P]),
        "tdm_net_layer_times": (i32, [P, P, P, i32]),
        "tdm_net_destroy": (i32, [P]),
        "tdm_write_seeded_weights": (i32, [ctypes.c_char_p, u64]),
        "tdm_mnn_workspace_bytes": (sz, [i32, i32, i32]),
        "tdm_match_mnn": (i32, [P, i32, P, i32, i32, i32, P, P, P, P, P, sz, P]),
        "tdm_ransac_workspace_bytes": (sz, [i32, i32]),
        "tdm_ransac": (i32, [P, P, P, i32, ctypes.POINTER(RansacParams), P, P, P, P, sz, P]),
        "tdm_ransac_noalloc": (i32, [P, P, P, i32, ctypes.POINTER(RansacParams), P, P, P, P]),
        "tdm_pairs_to_points": (i32, [P, P, P, P, i32, P, P, P]),
        "tdm_tsdf_init": (i32, [P, P, P, P]),
        "tdm_depth_from_mm": (i32, [P, i64, P, P]),
        "tdm_tsdf_integrate": (i32, [P, P, P, P, f32, f32, P, i32, i32, i32, P, P, P]),
        "tdm_extract_workspace_bytes": (sz, [P]),
        "tdm_tsdf_extract": (i32, [P, P, P, P, f32, f32, f32, P, i64, P, P, sz, P]),
        "tdm_pipeline_create": (i32, [ctypes.POINTER(PipelineConfig), P, ctypes.POINTER(P)]),
        "tdm_pipeline_destroy": (i32, [P]),
        "tdm_describe_fragment": (i32, [P, P, i32, u64, i32, P, P, G, P]),
        "tdm_register_pair": (i32, [P, P, i32, P, i32, u64, i32, ctypes.POINTER(PairResult), P]),
        "tdm_register_pair_host": (i32, [P, P, i32, P, i32, u64, i32, ctypes.POINTER(PairResult), P]),
        "tdm_net_clone": (i32, [P, ctypes.POINTER(P)]),
        "tdm_net_workspace_bytes": (sz, [P, i32]),
        "tdm_server_create": (i32, [ctypes.POINTER(ServerConfig), P, ctypes.POINTER(P)]),
        "tdm_server_slots": (i32, [P]),
        "tdm_server_submit": (i32, [P, P, i32, P, i32, u64, i32, ctypes.POINTER(ctypes.c_int64)]),
        "tdm_server_wait": (i32, [P, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(PairResult),
                                  ctypes.POINTER(ctypes.c_double)]),
        "tdm_server_submit_pair": (i32, [P, ctypes.POINTER(Fragment), ctypes.POINTER(Fragment),
                                         ctypes.POINTER(ctypes.c_int64)]),
        "tdm_server_cancel": (i32, [P, ctypes.c_int64]),
        "tdm_server_get_stats": (i32, [P, ctypes.POINTER(ServerStats)]),
        "tdm_store_create": (i32, [i64, ctypes.POINTER(P)]),
        "tdm_store_destroy": (i32, [P]),
        "tdm_store_describe": (i32, [P, P, u64, P, i32, u64, i32, ctypes.POINTER(i32), P]),
        "tdm_store_put": (i32, [P, u64, u64, P, P, i32, G, P]),
        "tdm_store_get": (i32, [P, u64, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(i32), G]),
        "tdm_store_remove": (i32, [P, u64]),
        "tdm_store_get_stats": (i32, [P, ctypes.POINTER(StoreStats)]),
        "tdm_register_stored": (i32, [P, P, u64, u64, ctypes.POINTER(PairResult), P]),
        "tdm_server_destroy": (i32, [P]),
        "tdm_net_autotune": (i32, [P, P, i32, i32, P]),
        "tdm_net_tiles": (i32, [P, P, P]),
        "tdm_net_set_tile": (i32, [P, i32, i32, i32]),
        "tdm_net_tile_forms": (i32, [P, P]),
        "tdm_net_set_tile_form": (i32, [P, i32, i32, i32, i32]),
        "tdm_batch_create": (i32, [ctypes.POINTER(BatchConfig), P, ctypes.POINTER(P)]),
        "tdm_batch_destroy": (i32, [P]),
        "tdm_batch_device_bytes": (sz, [P]),
        "tdm_describe_batch": (i32, [P, P, i32, P, P, P, P, P, P, P, P]),
        "tdm_batch_stats": (i32, [P, P, P]),
        "tdm_overlap_workspace_bytes": (sz, [i32, i32]),
        "tdm_overlap": (i32, [P, i32, P, i32, P, f32, P, P, sz, P]),
        "tdm_tdf_exact": (i32, [P, i32, G, P, P]),
        "tdm_icp_workspace_bytes": (sz, [i32, i32]),
        "tdm_icp": (i32, [P, i32, P, i32, P, ctypes.POINTER(IcpParams), ctypes.POINTER(IcpResult), P, sz, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != 0:
        raise TdmError(status, lib().tdm_last_error().decode())


def version() -> str:
    return lib().tdm_version().decode()


def _ptr(t) -> int:
    """Device (torch) or host (numpy) buffer address."""
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def _stream(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def device_status(stream=None) -> None:
    check(lib().tdm_device_status(_stream(stream)))


def selftest_wait_timeout(budget_us: int, device="cuda", stream=None):
    """Runs the bounded-wait self-test kernel (a wait that nothing satisfies,
    given up after budget_us); returns its 3 result words.  The device error
    word is raised: the next device_status() raises TdmError(TIMEOUT)."""
    import torch
    out = torch.zeros(3, dtype=torch.int32, device=device)
    check(lib().tdm_selftest_wait_timeout(budget_us, _ptr(out), _stream(stream)))
    return out.cpu().tolist()


def launch_count() -> int:
    """Kernels launched by libtdm so far in this process."""
    return int(lib().tdm_launch_count())


# --------------------------------------------------------------------------
# Stage calls (core/demo.cu)
# --------------------------------------------------------------------------
def grid_from_points_host(pts: np.ndarray, voxel_size=0.01, trunc_voxels=5.0, pad=15) -> Grid:
    pts = np.ascontiguousarray(pts, np.float32)
    g = Grid()
    check(lib().tdm_grid_from_points_host(_ptr(pts), pts.shape[0], voxel_size, np.float32(voxel_size) *
                                          np.float32(trunc_voxels), pad, ctypes.byref(g)))
    return g


def grid_from_points(pts_dev, voxel_size=0.01, trunc_voxels=5.0, pad=15, stream=None) -> Grid:
    import torch
    ws = torch.empty(lib().tdm_grid_workspace_bytes(), dtype=torch.uint8, device=pts_dev.device)
    g = Grid()
    check(lib().tdm_grid_from_points(_ptr(pts_dev), pts_dev.shape[0], voxel_size,
                                     float(np.float32(voxel_size) * np.float32(trunc_voxels)), pad, ctypes.byref(g),
                                     _ptr(ws), _stream(stream)))
    return g


def tdf(pts_dev, grid: Grid, mode: int = TDF_EXACT, stream=None):
    import torch
    out = torch.empty(grid.voxels, dtype=torch.float32, device=pts_dev.device)
    nws = lib().tdm_tdf_workspace_bytes(ctypes.byref(grid))
    ws = torch.empty(nws, dtype=torch.uint8, device=pts_dev.device)
    check(lib().tdm_tdf(_ptr(pts_dev), pts_dev.shape[0], ctypes.byref(grid), mode, _ptr(out), _ptr(ws), nws,
                        _stream(stream)))
    return out


def keypoint_indices(seed: int, n_pts: int, k: int, device="cuda", stream=None):
    import torch
    idx = torch.empty(k, dtype=torch.int32, device=device)
    check(lib().tdm_keypoint_indices(seed, n_pts, k, _ptr(idx), _stream(stream)))
    return idx


def keypoints(pts_dev, idx_dev, grid: Grid, stream=None):
    import torch
    k = idx_dev.shape[0]
    kp = torch.empty((k, 3), dtype=torch.float32, device=pts_dev.device)
    kg = torch.empty((k, 3), dtype=torch.int32, device=pts_dev.device)
    check(lib().tdm_keypoints(_ptr(pts_dev), pts_dev.shape[0], _ptr(idx_dev), k, ctypes.byref(grid), _ptr(kp),
                              _ptr(kg), _stream(stream)))
    return kp, kg


def gather(tdf_dev, grid: Grid, kp_grid_dev, stream=None):
    import torch
    k = kp_grid_dev.shape[0]
    out = torch.empty((k, 27000), dtype=torch.float32, device=tdf_dev.device)
    check(lib().tdm_gather(_ptr(tdf_dev), ctypes.byref(grid), _ptr(kp_grid_dev), k, _ptr(out), _stream(stream)))
    return out


# --------------------------------------------------------------------------
# Net (marvin::Net replacement)
# --------------------------------------------------------------------------
class Net:
    """Descriptor net of core/3dmatch-net-test.json on the GPU."""

    def __init__(self, weights=None, precision="fp32", use_feat=True, marvin_path=None):
        self.precision = precision
        h = ctypes.c_void_p()
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        if marvin_path is not None:
            check(lib().tdm_net_create(marvin_path.encode(), prec, 1 if use_feat else 0, ctypes.byref(h)))
        else:
            names = ["conv1", "conv2", "conv3", "conv4", "conv5", "conv6", "conv7", "conv8", "feat"]
            ws = [np.ascontiguousarray(weights[n + ".weight"], np.float32).reshape(-1) for n in names]
            bs = [np.ascontiguousarray(weights[n + ".bias"], np.float32).reshape(-1) for n in names]
            wp = (ctypes.c_void_p * 9)(*[w.ctypes.data for w in ws])
            bp = (ctypes.c_void_p * 9)(*[b.ctypes.data for b in bs])
            check(lib().tdm_net_create_from_host(ctypes.cast(wp, ctypes.c_void_p), ctypes.cast(bp, ctypes.c_void_p),
                                                 prec, 1 if use_feat else 0, ctypes.byref(h)))
        self.handle = h

    def forward(self, patches_dev, out=None, stream=None):
        import torch
        b = patches_dev.shape[0]
        if out is None:
            out = torch.empty((b, 512), dtype=torch.float32, device=patches_dev.device)
        check(lib().tdm_net_forward(self.handle, _ptr(patches_dev), b, _ptr(out), _stream(stream)))
        return out

    def response(self, name: str, patches_dev, stream=None):
        """Named intermediate response, float channels-last [b, D, D, D, C]."""
        import torch
        shapes = {"conv1": (28, 64), "conv2": (26, 64), "pool1": (13, 64), "conv3": (11, 128), "conv4": (9, 128),
                  "conv5": (7, 256), "conv6": (5, 256), "conv7": (3, 512), "conv8": (1, 512), "feat": (1, 512)}
        D, C = shapes[name]
        b = patches_dev.shape[0]
        out = torch.empty((b, D, D, D, C), dtype=torch.float32, device=patches_dev.device)
        check(lib().tdm_net_response(self.handle, name.encode(), _ptr(patches_dev), b, _ptr(out), _stream(stream)))
        return out

    def calibrate(self, patches_dev, stream=None) -> None:
        """FP8 form: activation scales from these calibration patches."""
        check(lib().tdm_net_calibrate(self.handle, _ptr(patches_dev), patches_dev.shape[0], _stream(stream)))

    def act_scales(self):
        out = np.zeros(9, np.float32)
        check(lib().tdm_net_act_scales(self.handle, _ptr(out)))
        return out

    def set_max_batch(self, n: int) -> None:
        check(lib().tdm_net_set_max_batch(self.handle, n))

    LAYER_SLOTS = ["conv1", "conv2", "conv3", "conv4", "conv5", "conv6", "conv7", "conv8", "feat", "pool1"]

    def set_timing(self, enable: bool) -> None:
        check(lib().tdm_net_set_timing(self.handle, 1 if enable else 0))

    def layer_times(self, reset: bool = False) -> dict:
        """{layer: (total ms, launches)} from the CUDA events of set_timing(True)."""
        ms = np.zeros(10, np.float64)
        n = np.zeros(10, np.int64)
        check(lib().tdm_net_layer_times(self.handle, _ptr(ms), _ptr(n), 1 if reset else 0))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.LAYER_SLOTS)}

    def autotune(self, patches_dev, reps: int = 3, stream=None) -> dict:
        """Per-layer tcgen05 tile chosen by timing every shape on these patches."""
        check(lib().tdm_net_autotune(self.handle, _ptr(patches_dev), patches_dev.shape[0], reps, _stream(stream)))
        return self.tiles()

    def tiles(self) -> dict:
        """{layer: (N tile, M sub-tiles)} of the tensor-core forms."""
        nt = np.zeros(9, np.int32)
        ms = np.zeros(9, np.int32)
        check(lib().tdm_net_tiles(self.handle, _ptr(nt), _ptr(ms)))
        return {k: (int(nt[i]), int(ms[i])) for i, k in enumerate(self.LAYER_SLOTS[:9])}

    CONV_FORMS = ("grid", "dxf", "gather", "xrun", "gather_wt", "xrun_wt", "dxf_pair")

    def forms(self) -> dict:
        """{layer: kernel form}: "grid" (implicit GEMM over every input
        position), "dxf" (conv2's dx-fused form) or "gather" (GEMM over the
        valid output positions, A rows gathered per tap) or "xrun" (gathered
        (b, z, y) rows with whole input x runs, the dx taps sharing one operand);
        "gather_wt" / "xrun_wt" put the weights in the MMA's A operand (conv3,
        conv4); "dxf_pair" runs conv2's dx-fused form on CTA pairs sharing each
        MMA (M = 256, N = 192)."""
        f = np.zeros(9, np.int32)
        check(lib().tdm_net_tile_forms(self.handle, _ptr(f)))
        return {k: self.CONV_FORMS[int(f[i])] for i, k in enumerate(self.LAYER_SLOTS[:9])}

    def set_tile(self, layer: str, nt: int, msub: int, form: str = None) -> None:
        """Tile (and optionally kernel form) of one layer; without a form the
        layer keeps its current form when that form has the tile."""
        code = -1 if form is None else self.CONV_FORMS.index(form)
        check(lib().tdm_net_set_tile_form(self.handle, self.LAYER_SLOTS.index(layer), nt, msub, code))

    def close(self):
        if self.handle:
            lib().tdm_net_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_seeded_weights(path: str, seed: int) -> None:
    check(lib().tdm_write_seeded_weights(path.encode(), seed))


# --------------------------------------------------------------------------
# Matching / registration
# --------------------------------------------------------------------------
def match_mnn(da_dev, db_dev, precision="fp32", stream=None):
    import torch
    na, dim = da_dev.shape
    nb = db_dev.shape[0]
    dev = da_dev.device
    nn_ab = torch.empty(na, dtype=torch.int32, device=dev)
    nn_ba = torch.empty(nb, dtype=torch.int32, device=dev)
    pairs = torch.empty((max(1, min(na, nb)), 2), dtype=torch.int32, device=dev)
    npairs = torch.zeros(1, dtype=torch.int32, device=dev)
    nws = lib().tdm_mnn_workspace_bytes(na, nb, dim)
    ws = torch.empty(max(nws, 16), dtype=torch.uint8, device=dev)
    prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    check(lib().tdm_match_mnn(_ptr(da_dev), na, _ptr(db_dev), nb, dim, prec, _ptr(nn_ab), _ptr(nn_ba), _ptr(pairs),
                              _ptr(npairs), _ptr(ws), nws, _stream(stream)))
    return pairs, npairs, nn_ab, nn_ba


def ransac(x_dev, y_dev, m_dev, seed: int, iterations: int, threshold=0.05, adaptive=False, max_trials=50000,
           stream=None):
    import torch
    m_max = x_dev.shape[0]
    dev = x_dev.device
    prm = RansacParams(seed, iterations, threshold, 1 if adaptive else 0, max_trials)
    rt = torch.zeros(12, dtype=torch.float64, device=dev)
    inl = torch.zeros(max(m_max, 1), dtype=torch.int32, device=dev)
    info = torch.zeros(4, dtype=torch.int32, device=dev)
    nws = lib().tdm_ransac_workspace_bytes(m_max, iterations)
    ws = torch.empty(max(nws, 16), dtype=torch.uint8, device=dev)
    check(lib().tdm_ransac(_ptr(x_dev), _ptr(y_dev), _ptr(m_dev), m_max, ctypes.byref(prm), _ptr(rt), _ptr(inl),
                           _ptr(info), _ptr(ws), nws, _stream(stream)))
    return rt, inl, info


def tdf_exact(pts_dev, grid: Grid, stream=None):
    """pointCloud2TDF.m on the grid's voxel centres (float [V], x fastest)."""
    import torch
    out = torch.empty(grid.voxels, dtype=torch.float32, device=pts_dev.device)
    check(lib().tdm_tdf_exact(_ptr(pts_dev), pts_dev.shape[0], ctypes.byref(grid), _ptr(out), _stream(stream)))
    return out


def icp(fixed_dev, moving_dev, init_rt, grid=0.01, max_dist=0.10, inlier_ratio=0.30, max_iterations=50,
        tol_translation=1e-4, tol_rotation_deg=9e-5, stream=None):
    """ICP of moving onto fixed from init_rt (3x4 or 4x4, moving -> fixed):
    (4x4 float64, IcpResult)."""
    import torch
    nf, nm = fixed_dev.shape[0], moving_dev.shape[0]
    r = np.ascontiguousarray(np.asarray(init_rt, np.float64).reshape(-1)[:12])
    prm = IcpParams(grid, max_dist, inlier_ratio, max_iterations, tol_translation, tol_rotation_deg)
    res = IcpResult()
    nws = lib().tdm_icp_workspace_bytes(nf, nm)
    ws = torch.empty(max(nws, 16), dtype=torch.uint8, device=fixed_dev.device)
    check(lib().tdm_icp(_ptr(fixed_dev), nf, _ptr(moving_dev), nm, _ptr(r), ctypes.byref(prm), ctypes.byref(res),
                        _ptr(ws), nws, _stream(stream)))
    T = np.eye(4)
    T[:3] = np.array(list(res.rt)).reshape(3, 4)
    return T, res


def overlap(a_dev, b_dev, rt, radius=0.05, stream=None):
    """(points of a near Rt*b, points of Rt*b near a) within radius: the
    reference's ratioAligned numerators (register2Fragments.m:90-97)."""
    import torch
    na, nb = a_dev.shape[0], b_dev.shape[0]
    r = np.ascontiguousarray(np.asarray(rt, np.float64).reshape(-1)[:12])
    counts = torch.zeros(2, dtype=torch.int32, device=a_dev.device)
    nws = lib().tdm_overlap_workspace_bytes(na, nb)
    ws = torch.empty(max(nws, 16), dtype=torch.uint8, device=a_dev.device)
    check(lib().tdm_overlap(_ptr(a_dev), na, _ptr(b_dev), nb, _ptr(r), radius, _ptr(counts), _ptr(ws), nws,
                            _stream(stream)))
    c = counts.cpu().numpy()
    return int(c[0]), int(c[1])


def pairs_to_points(kp_a, kp_b, pairs, n_pairs_dev, stream=None):
    import torch
    mx = pairs.shape[0]
    x = torch.zeros((mx, 3), dtype=torch.float32, device=kp_a.device)
    y = torch.zeros((mx, 3), dtype=torch.float32, device=kp_a.device)
    check(lib().tdm_pairs_to_points(_ptr(kp_a), _ptr(kp_b), _ptr(pairs), _ptr(n_pairs_dev), mx, _ptr(x), _ptr(y),
                                    _stream(stream)))
    return x, y


# --------------------------------------------------------------------------
# TSDF fusion
# --------------------------------------------------------------------------
def tsdf_init(tsdf_dev, weight_dev, dim, stream=None):
    d = (ctypes.c_int32 * 3)(*dim)
    check(lib().tdm_tsdf_init(_ptr(tsdf_dev), _ptr(weight_dev), d, _stream(stream)))


def depth_from_mm(mm_dev, out_dev, stream=None):
    check(lib().tdm_depth_from_mm(_ptr(mm_dev), mm_dev.numel(), _ptr(out_dev), _stream(stream)))


def tsdf_integrate(tsdf_dev, weight_dev, dim, origin, voxel_size, trunc, depth_dev, K, cam2base, stream=None):
    nf, H, W = depth_dev.shape
    d = (ctypes.c_int32 * 3)(*dim)
    o = (ctypes.c_float * 3)(*origin)
    Kc = (ctypes.c_float * 9)(*np.asarray(K, np.float32).reshape(9))
    c2b = np.ascontiguousarray(cam2base, np.float32).reshape(nf, 16)
    check(lib().tdm_tsdf_integrate(_ptr(tsdf_dev), _ptr(weight_dev), d, o, voxel_size, trunc, _ptr(depth_dev), nf, H,
                                   W, Kc, _ptr(c2b), _stream(stream)))


def tsdf_extract(tsdf_dev, weight_dev, dim, origin, voxel_size, tsdf_thr=0.2, w_thr=1.0, max_pts=None, stream=None):
    import torch
    d = (ctypes.c_int32 * 3)(*dim)
    o = (ctypes.c_float * 3)(*origin)
    V = int(dim[0]) * int(dim[1]) * int(dim[2])
    max_pts = V if max_pts is None else max_pts
    pts = torch.empty((max(max_pts, 1), 3), dtype=torch.float32, device=tsdf_dev.device)
    n = torch.zeros(1, dtype=torch.int64, device=tsdf_dev.device)
    nws = lib().tdm_extract_workspace_bytes(d)
    ws = torch.empty(max(nws, 16), dtype=torch.uint8, device=tsdf_dev.device)
    check(lib().tdm_tsdf_extract(_ptr(tsdf_dev), _ptr(weight_dev), d, o, voxel_size, tsdf_thr, w_thr, _ptr(pts),
                                 max_pts, _ptr(n), _ptr(ws), nws, _stream(stream)))
    return pts, n


# --------------------------------------------------------------------------
# Whole path
# --------------------------------------------------------------------------
def pipeline_config(voxel_size=0.01, trunc_voxels=5.0, pad=15, max_points=400000, max_keypoints=5000,
                    max_voxels=120_000_000, match_precision="fp32", ransac_seed=7, ransac_iters=100000, threshold=0.05,
                    adaptive=False, max_trials=50000) -> PipelineConfig:
    return PipelineConfig(voxel_size, trunc_voxels, pad, max_points, max_keypoints, max_voxels,
                          PRECISIONS[match_precision],
                          RansacParams(ransac_seed, ransac_iters, threshold, 1 if adaptive else 0, max_trials))


class Pipeline:
    def __init__(self, net: Net, **kw):
        cfg = pipeline_config(**kw)
        h = ctypes.c_void_p()
        check(lib().tdm_pipeline_create(ctypes.byref(cfg), net.handle, ctypes.byref(h)))
        self.handle = h
        self.net = net

    def register(self, pts_a, pts_b, seed: int, k: int, stream=None) -> PairResult:
        r = PairResult()
        if isinstance(pts_a, np.ndarray):
            a = np.ascontiguousarray(pts_a, np.float32)
            b = np.ascontiguousarray(pts_b, np.float32)
            check(lib().tdm_register_pair_host(self.handle, _ptr(a), a.shape[0], _ptr(b), b.shape[0], seed, k,
                                               ctypes.byref(r), _stream(stream)))
        else:
            check(lib().tdm_register_pair(self.handle, _ptr(pts_a), pts_a.shape[0], _ptr(pts_b), pts_b.shape[0],
                                          seed, k, ctypes.byref(r), _stream(stream)))
        return r

    def describe(self, pts_dev, seed: int, k: int, stream=None):
        import torch
        kp = torch.empty((k, 3), dtype=torch.float32, device=pts_dev.device)
        desc = torch.empty((k, 512), dtype=torch.float32, device=pts_dev.device)
        g = Grid()
        check(lib().tdm_describe_fragment(self.handle, _ptr(pts_dev), pts_dev.shape[0], seed, k, _ptr(kp), _ptr(desc),
                                          ctypes.byref(g), _stream(stream)))
        return kp, desc, g

    def close(self):
        if self.handle:
            lib().tdm_pipeline_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Store:
    """Device-resident fragment store (tdm_store): describe once, register many."""

    def __init__(self, budget_bytes: int):
        h = ctypes.c_void_p()
        check(lib().tdm_store_create(budget_bytes, ctypes.byref(h)))
        self.handle = h

    def describe(self, pipe: "Pipeline", key: int, pts_dev, seed: int, k: int, stream=None) -> bool:
        """Describes the fragment under `key` unless stored; returns whether it was a hit."""
        hit = ctypes.c_int32()
        check(lib().tdm_store_describe(self.handle, pipe.handle, key, _ptr(pts_dev), pts_dev.shape[0], seed, k,
                                       ctypes.byref(hit), _stream(stream)))
        return bool(hit.value)

    def put(self, key: int, seed: int, keypts_dev, desc_dev, grid: Grid = None, stream=None) -> None:
        check(lib().tdm_store_put(self.handle, key, seed, _ptr(keypts_dev), _ptr(desc_dev), keypts_dev.shape[0],
                                  ctypes.byref(grid) if grid is not None else None, _stream(stream)))

    def get(self, key: int, device="cuda"):
        """Copies of the stored keypoints and descriptors (torch tensors) and the grid."""
        import torch
        kp, desc, k, g = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_int32(), Grid()
        check(lib().tdm_store_get(self.handle, key, ctypes.byref(kp), ctypes.byref(desc), ctypes.byref(k),
                                  ctypes.byref(g)))
        n = k.value
        torch.cuda.synchronize()
        return (_device_view(kp.value, (n, 3), device).clone(), _device_view(desc.value, (n, 512), device).clone(), g)

    def remove(self, key: int) -> None:
        check(lib().tdm_store_remove(self.handle, key))

    def stats(self) -> dict:
        st = StoreStats()
        check(lib().tdm_store_get_stats(self.handle, ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        if self.handle:
            lib().tdm_store_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _CudaArray:
    """A float32 device buffer described by __cuda_array_interface__."""

    def __init__(self, ptr: int, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (ptr, False),
                                         "version": 2, "strides": None}


def _device_view(ptr: int, shape, device="cuda"):
    import torch
    return torch.as_tensor(_CudaArray(ptr, shape), device=device)


def register_stored(pipe: "Pipeline", store: Store, key_a: int, key_b: int, stream=None) -> PairResult:
    r = PairResult()
    check(lib().tdm_register_stored(pipe.handle, store.handle, key_a, key_b, ctypes.byref(r), _stream(stream)))
    return r


class Batch:
    """Many fragments of uneven size through one persistent launch per stage
    (tdm_describe_batch); with use_graph the sequence is replayed as a CUDA graph."""

    def __init__(self, net: Net, max_fragments=64, max_points=20_000_000, max_keypoints=330_000,
                 max_voxels=1_500_000_000, trunc_voxels=5.0, pad=15, use_graph=True):
        self.net = net
        cfg = BatchConfig(max_fragments, max_points, max_keypoints, max_voxels, trunc_voxels, pad,
                          1 if use_graph else 0)
        h = ctypes.c_void_p()
        check(lib().tdm_batch_create(ctypes.byref(cfg), net.handle, ctypes.byref(h)))
        self.handle = h

    @property
    def device_bytes(self) -> int:
        return int(lib().tdm_batch_device_bytes(self.handle))

    def describe(self, pts_dev, point_offsets, voxel_sizes, keypoints, seeds, keypts=None, desc=None, stream=None):
        """pts_dev: (sum n, 3) float32 on the device; per-fragment host lists.
        Returns (keypts (sum k, 3), desc (sum k, 512), [Grid per fragment])."""
        import torch
        F = len(keypoints)
        off = np.ascontiguousarray(point_offsets, np.int64)
        vs = np.ascontiguousarray(voxel_sizes, np.float32)
        ks = np.ascontiguousarray(keypoints, np.int32)
        sd = np.ascontiguousarray(seeds, np.uint64)
        assert off.shape == (F + 1,) and vs.shape == (F,) and sd.shape == (F,)
        K = int(ks.sum())
        dev = pts_dev.device
        if keypts is None:
            keypts = torch.empty((max(K, 1), 3), dtype=torch.float32, device=dev)
        if desc is None:
            desc = torch.empty((max(K, 1), 512), dtype=torch.float32, device=dev)
        grids = (Grid * F)()
        check(lib().tdm_describe_batch(self.handle, _ptr(pts_dev), F, _ptr(off), _ptr(vs), _ptr(ks), _ptr(sd),
                                       _ptr(keypts), _ptr(desc), ctypes.cast(grids, ctypes.c_void_p),
                                       _stream(stream)))
        return keypts[:K], desc[:K], list(grids)

    def stats(self):
        n = ctypes.c_int64()
        r = ctypes.c_int32()
        check(lib().tdm_batch_stats(self.handle, ctypes.byref(n), ctypes.byref(r)))
        return {"launches_per_call": n.value, "replayed": bool(r.value)}

    def close(self):
        if self.handle:
            lib().tdm_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """tdm_server: continuous batching of pair registrations over the batched
    description kernels and a device-resident fragment store."""

    def __init__(self, net: Net, slots=4, hbm_budget_bytes=120 << 30, store_bytes=0, **pipeline_kw):
        cfg = ServerConfig(pipeline_config(**pipeline_kw), slots, hbm_budget_bytes, store_bytes)
        h = ctypes.c_void_p()
        check(lib().tdm_server_create(ctypes.byref(cfg), net.handle, ctypes.byref(h)))
        self.handle = h

    @property
    def slots(self) -> int:
        return int(lib().tdm_server_slots(self.handle))

    def submit(self, pts_a: np.ndarray, pts_b: np.ndarray, seed: int, k: int) -> int:
        a = np.ascontiguousarray(pts_a, np.float32)
        b = np.ascontiguousarray(pts_b, np.float32)
        t = ctypes.c_int64()
        check(lib().tdm_server_submit(self.handle, _ptr(a), a.shape[0], _ptr(b), b.shape[0], seed, k, ctypes.byref(t)))
        return t.value

    def submit_pair(self, a: dict, b: dict) -> int:
        """a, b: {"key": int (0 = anonymous), "pts": array or None, "seed": int, "k": int}."""
        frags, keep = [], []
        for f in (a, b):
            pts = f.get("pts")
            if pts is not None:
                pts = np.ascontiguousarray(pts, np.float32)
                keep.append(pts)
            frags.append(Fragment(f.get("key", 0), _ptr(pts) if pts is not None else None,
                                  pts.shape[0] if pts is not None else 0, f["seed"], f["k"]))
        t = ctypes.c_int64()
        check(lib().tdm_server_submit_pair(self.handle, ctypes.byref(frags[0]), ctypes.byref(frags[1]),
                                           ctypes.byref(t)))
        return t.value

    def cancel(self, ticket: int) -> None:
        check(lib().tdm_server_cancel(self.handle, ticket))

    def wait(self, ticket: int, timeout_ms: int = -1):
        r = PairResult()
        lat = ctypes.c_double()
        check(lib().tdm_server_wait(self.handle, ticket, timeout_ms, ctypes.byref(r), ctypes.byref(lat)))
        return r, lat.value

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().tdm_server_get_stats(self.handle, ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        if self.handle:
            lib().tdm_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
