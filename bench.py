#!/usr/bin/env python
"""Pair registrations per second of the GB300 3DMatch registration path.

A step registers one fragment pair shaped like the demo pipeline (two ~150k
point fragments of a seeded synthetic room, 1 cm TDF, 1000 keypoints each,
30^3 patches through the 9-layer net, mutual-NN matching, RANSAC with 100k
trials and Kabsch refit).  The headline form is BF16 (tcgen05) for the net and
the descriptor-distance GEMM; the FP32 CUDA-core form is timed beside it on the
same GPU.  `value` is device-resident throughput (points already in HBM);
`e2e` goes through the host C ABI (tdm_register_pair_host) with the
host->device copy of the points and the device->host copy of the result
inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference's loops (the
C/OpenMP oracle) on the host cores on a bounded sample of the same workload,
extrapolated to one pair.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONV2_FLOP_PER_PATCH = 2.0 * 26 ** 3 * 64 * (27 * 64)  # useful FLOPs of conv2 (algorithmic)
# MMA work the CTA-pair conv2 issues per patch: 78 tiles (3 blocks of 252 plane rows x 26 z)
# x 36 MMAs of 256 x 192 x 16 (1.14x the useful work: rows with y = 26, dx taps of x >= 26)
CONV2_MMA_FLOP_PER_PATCH = 78 * 36 * 2 * 256 * 192 * 16
# the MMA rate measured by the tcgen05 probe: 4,096 MAC/clk/SM
MMA_MAC_PER_CLK_SM = 4096
NET_FLOP_PER_PATCH = 6.452e9


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["bf16", "fp8", "fp32"])
    ap.add_argument("--fp8-steps", type=int, default=5)
    ap.add_argument("--keypoints", type=int, default=1000)
    ap.add_argument("--points", type=int, default=150_000)
    ap.add_argument("--ransac-iters", type=int, default=100_000)
    ap.add_argument("--pairs", type=int, default=4, help="distinct synthetic pairs cycled through")
    ap.add_argument("--fp32-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve", action="store_true", help="serving sweep (Poisson arrivals) instead of the pair bench")
    ap.add_argument("--serve-lambdas", default="10,50,200,2000")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--tsdf", action="store_true", help="TSDF fusion then description workload")
    ap.add_argument("--descriptors", action="store_true", help="descriptor throughput workload (5000 patches)")
    ap.add_argument("--batch", action="store_true", help="batched uneven fragments workload (64 fragments)")
    ap.add_argument("--batch-fragments", type=int, default=64)
    ap.add_argument("--net-chunk", type=int, default=0,
                    help="batched form: patches per net launch (0 = the library default, 2,048)")
    ap.add_argument("--registration", action="store_true",
                    help="registration benchmark scored in the reference's metric (synthetic scene)")
    ap.add_argument("--reg-views", type=int, default=8)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic(name):
    """dram bytes per launch recorded in profiles/<name>.md ('traffic_bytes_per_launch: N')."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the sampler takes a moment to start: the timed region begins after its first row
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[4:8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# --------------------------------------------------------------------------
# CPU baseline: the oracle's restated reference loops on a bounded sample
# --------------------------------------------------------------------------
MARVIN_BATCH = 50  # patches per net forward in core/demo.cu:195 (one Marvin batch)


def cpu_sample(pair, k, ransac_iters, ransac_sample_iters=20_000):
    """Times one bounded sample of the pair workload on all host cores with the
    oracle's restated reference loops (OpenMP C) and extrapolates it linearly
    to a whole pair.  The sample: the whole-grid TDF of fragment A (one of the
    pair's two grids), one Marvin batch of 50 of its 30^3 patches through the
    net (2k per pair), the full k x k mutual NN, and `ransac_sample_iters` of
    the pair's RANSAC trials.  Returns (pairs/s extrapolated, seconds the
    sample took, fraction of a pair's work the sample is, description, parts)."""
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    a, b, _ = pair
    dim, origin = O.grid_setup(a)
    occ = O.occupancy(a, dim, origin, 0.01)
    t0 = time.perf_counter()
    tdf = O.tdf(occ, dim, 0.01, np.float32(0.01) * np.float32(5))
    t_tdf = time.perf_counter() - t0
    idx = O.keypoint_indices(1, a.shape[0], MARVIN_BATCH)
    _, kg = O.keypoints(a, idx, origin, 0.01)
    patches = O.gather(tdf, dim, kg)
    w = O.he_normal_weights(1)
    t0 = time.perf_counter()
    O.net_forward(patches, w)
    t_net = time.perf_counter() - t0
    rng = np.random.default_rng(0)
    da = rng.normal(size=(k, 512)).astype(np.float32)
    db = rng.normal(size=(k, 512)).astype(np.float32)
    t0 = time.perf_counter()
    O.mutual_nn(da, db)
    t_mnn = time.perf_counter() - t0
    m = 300
    x = rng.uniform(-1, 1, (m, 3)).astype(np.float32)
    y = rng.uniform(-1, 1, (m, 3)).astype(np.float32)
    it = min(ransac_iters, ransac_sample_iters)
    t0 = time.perf_counter()
    O.ransac(x, y, 1, it, 0.05)
    t_ransac = time.perf_counter() - t0
    sample_s = t_tdf + t_net + t_mnn + t_ransac
    # whole pair: two grids, 2k patches, one MNN, all RANSAC trials
    parts = {"tdf_s": 2 * t_tdf, "net_s": t_net * (2 * k) / MARVIN_BATCH, "mnn_s": t_mnn,
             "ransac_s": t_ransac * ransac_iters / it}
    t_pair = sum(parts.values())
    sample = ("whole-grid TDF of one fragment (%d voxels; x2 per pair), net on one Marvin batch of %d gathered "
              "patches (x%.0f per pair), MNN %dx%d, RANSAC %d of %d trials (m=%d); extrapolated linearly"
              % (int(np.prod(dim.astype(np.int64))), MARVIN_BATCH, 2 * k / MARVIN_BATCH, k, k, it, ransac_iters, m))
    return 1.0 / t_pair, sample_s, sample_s / t_pair, sample, parts


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    import __graft_entry__ as ge
    ge.load()
    from tdm_gb300 import synth
    pair = synth.fragment_pair(20260000, n_points=args.points)
    for _ in range(args.warmup):
        cpu_sample(pair, args.keypoints, args.ransac_iters)
    rates, secs, fracs = [], [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, sec, frac, sample, parts = cpu_sample(pair, args.keypoints, args.ransac_iters)
        rates.append(v)
        secs.append(sec)
        fracs.append(frac)
    wall = time.perf_counter() - t0
    # a step is one sample: ms_per_step is its measured time, and the rate is
    # the pair fraction the steps covered over the time they took
    value = float(np.sum(fracs) / np.sum(secs))
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": "pair registrations/s", "value": value, "unit": "pairs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean(secs)), "pair_fraction_per_step": float(np.mean(fracs)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "demo pipeline pair: 2 x %d-point synthetic room fragments, 1 cm TDF, %d keypoints "
                               "per fragment, 30^3 patches, 9-layer net, mutual NN, RANSAC %d trials"
                               % (args.points, args.keypoints, args.ransac_iters)},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                         "sample": sample + "; one sample per step, wall %.1fs for %d steps" % (wall, args.steps),
                         "parts_s_per_pair": {kk: round(vv, 3) for kk, vv in parts.items()}},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference loops (oracle/oracle.c, OpenMP); the reference's own "
                "demo.cu needs OpenCV and cuDNN and MATLAB for matching, so it is not built here",
    }
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def stage_breakdown(tdm, torch, dev, pair, net, k, ransac_iters, prec, reps=5):
    """Times each stage of one pair with CUDA events (median of reps) and
    reports its achieved rate against the stage's roofline."""
    peaks, kind = load_peaks()
    hbm = peaks["hbm_gbs"]
    tc_peak = peaks["bf16_tflops"]
    a, b, _ = pair
    stream = torch.cuda.current_stream()

    def timeit(fn):
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts)), out

    pd = torch.from_numpy(a).to(dev)
    g = tdm.grid_from_points_host(a)
    V = g.voxels
    ms_tdf, tdf = timeit(lambda: tdm.tdf(pd, g))
    idx = tdm.keypoint_indices(5, a.shape[0], k, device=dev)
    kp, kg = tdm.keypoints(pd, idx, g)
    ms_gather, patches = timeit(lambda: tdm.gather(tdf, g, kg))
    p2 = torch.cat([patches, patches])
    ms_net, desc = timeit(lambda: net.forward(p2))
    mprec = "bf16" if prec in ("bf16", "fp8") else "fp32"
    ms_mnn, res = timeit(lambda: tdm.match_mnn(desc[:k].contiguous(), desc[k:].contiguous(), mprec))
    # RANSAC on the real matches of a pair
    pb = torch.from_numpy(b).to(dev)
    gb = tdm.grid_from_points_host(b)
    kpb, kgb = tdm.keypoints(pb, tdm.keypoint_indices(6, b.shape[0], k, device=dev), gb)
    descb = net.forward(tdm.gather(tdm.tdf(pb, gb), gb, kgb))
    pairs_, npairs, _, _ = tdm.match_mnn(desc[:k].contiguous(), descb, mprec)
    x, y = tdm.pairs_to_points(kp, kpb, pairs_, npairs)
    m = int(npairs.item())
    ms_ransac, _ = timeit(lambda: tdm.ransac(x, y, npairs, 7, ransac_iters, 0.05))

    def frac(ach, peak):
        return round(ach / peak, 4)

    tdf_bytes = 12 * a.shape[0] + 4 * V
    gather_bytes = k * 27000 * 8
    net_flop = 2 * k * NET_FLOP_PER_PATCH
    mnn_flop = 2.0 * k * k * 512
    ransac_flop = ransac_iters * max(m, 1) * 20.0
    return {
        "tdf": {"ms": ms_tdf, "bound": "hbm", "achieved_gbs": tdf_bytes / ms_tdf / 1e6,
                "frac": frac(tdf_bytes / ms_tdf / 1e6, hbm), "work": "12*N + 4*V = %d bytes (V=%d)" % (tdf_bytes, V)},
        "gather": {"ms": ms_gather, "bound": "hbm", "achieved_gbs": gather_bytes / ms_gather / 1e6,
                   "frac": frac(gather_bytes / ms_gather / 1e6, hbm), "work": "%d patches x 27000 x 8 B" % k},
        "net": {"ms": ms_net, "bound": "tensor", "achieved_tflops": net_flop / ms_net / 1e9,
                "frac": frac(net_flop / ms_net / 1e9, tc_peak), "work": "%d patches x 6.452 GFLOP" % (2 * k)},
        "mnn": {"ms": ms_mnn, "bound": "tensor", "achieved_tflops": mnn_flop / ms_mnn / 1e9,
                "frac": frac(mnn_flop / ms_mnn / 1e9, tc_peak), "work": "2 x %d x %d x 512 FLOP" % (k, k)},
        "ransac": {"ms": ms_ransac, "bound": "fp32 simt", "achieved_tflops": ransac_flop / ms_ransac / 1e9,
                   "work": "%d trials x %d matches x 20 FLOP" % (ransac_iters, m)},
        "peak_source": kind + " (hbm_gbs, bf16_tflops burst: stages timed alone)",
    }


def replica_seeds(rank, n_pairs):
    """Seeds of the synthetic pairs one replica cycles through: every rank
    registers its own pairs (weak scaling, no data-path collective)."""
    return [20260000 + 97 * rank + i for i in range(n_pairs)]


def max_over_ranks(values, dist, device):
    """Element-wise maximum of per-rank timings (the slowest replica sets the
    whole-job time); identity on one process."""
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def job_rate(world, units_per_rank, ms_max):
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / (ms_max / 1000.0)


def run_ours(args, rank, world, local):
    import torch
    import __graft_entry__ as ge
    tdm = ge.load()
    try:
        tdm.lib()
    except ImportError:
        ge.build()
        tdm.lib()
    from tdm_gb300 import synth
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    k = args.keypoints
    pairs = [synth.fragment_pair(sd, n_points=args.points) for sd in replica_seeds(rank, args.pairs)]
    dpairs = [(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)) for a, b, _ in pairs]
    hpairs = [(torch.from_numpy(a).pin_memory().numpy(), torch.from_numpy(b).pin_memory().numpy())
              for a, b, _ in pairs]
    wfile = os.path.join(tempfile.gettempdir(), "tdm_bench_weights_%d.marvin" % os.getpid())
    tdm.write_seeded_weights(wfile, 20260000)

    calib = None

    def calibration_patches():
        # seeded calibration batch: 256 patches of a separate synthetic fragment
        cp = synth.fragment(20269999, n_points=args.points)
        pd = torch.from_numpy(cp).to(dev)
        g = tdm.grid_from_points_host(cp)
        t = tdm.tdf(pd, g)
        _, kg = tdm.keypoints(pd, tdm.keypoint_indices(20269999, cp.shape[0], 256, device=dev), g)
        return tdm.gather(t, g, kg)

    def make(prec):
        nonlocal calib
        net = tdm.Net(marvin_path=wfile, precision=prec)
        if prec == "fp8":
            if calib is None:
                calib = calibration_patches()
            net.calibrate(calib)
        pipe = tdm.Pipeline(net, max_keypoints=k, max_points=max(p[0].shape[0] for p in pairs) + 16,
                            max_voxels=80_000_000, match_precision="bf16" if prec == "fp8" else prec,
                            ransac_seed=20260000,
                            ransac_iters=args.ransac_iters)
        return net, pipe

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(pipe, steps, host=False):
        stream = torch.cuda.current_stream()
        barrier()
        t0 = time.perf_counter()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = None
        for s in range(steps):
            if host:
                a, b = hpairs[s % len(hpairs)]
            else:
                a, b = dpairs[s % len(dpairs)]
            res = pipe.register(a, b, seed=1000 + s, k=k)
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1)
        wall = (time.perf_counter() - t0) * 1000.0
        ms, wall = max_over_ranks([ms, wall], dist, dev)
        return ms, wall, res

    prec = args.precision
    net, pipe = make(prec)
    for s in range(args.warmup):
        a, b = dpairs[s % len(dpairs)]
        pipe.register(a, b, seed=1000 + s, k=k)
    net.layer_times(reset=True)
    net.set_timing(True)
    clocks = Clocks(local)
    clocks.start()
    l0 = tdm.launch_count()
    ms, wall, res = timed(pipe, args.steps)
    launches = tdm.launch_count() - l0
    clk = clocks.stop()
    net.set_timing(False)
    lt = net.layer_times(reset=True)
    ms_step = ms / args.steps
    value = job_rate(world, args.steps, ms)
    # e2e through the host C ABI
    e2e_steps = max(3, args.steps // 2)
    ms_e2e, _, _ = timed(pipe, e2e_steps, host=True)
    e2e = job_rate(world, e2e_steps, ms_e2e)
    h2d = int(np.mean([(a.shape[0] + b.shape[0]) * 12 for a, b in hpairs]))
    d2h = 12 * 8 + 16 + 4
    # FP32 drop-in form on the same GPU
    fp32 = None
    if prec != "fp32" and args.fp32_steps > 0:
        net32, pipe32 = make("fp32")
        pipe32.register(*dpairs[0], seed=1, k=k)
        ms32, _, _ = timed(pipe32, args.fp32_steps)
        fp32 = world * args.fp32_steps / (ms32 / 1000.0)
        pipe32.close()
        net32.close()
    # FP8 form (E4M3 conv3..conv8) on the same GPU
    fp8 = None
    if prec != "fp8" and args.fp8_steps > 0:
        net8, pipe8 = make("fp8")
        pipe8.register(*dpairs[0], seed=1, k=k)
        ms8, _, _ = timed(pipe8, args.fp8_steps)
        fp8 = world * args.fp8_steps / (ms8 / 1000.0)
        pipe8.close()
        net8.close()
    # per-pair latency of the headline form (one pair per call, synchronous)
    lat = []
    for s_ in range(args.steps):
        a, b = dpairs[s_ % len(dpairs)]
        t0 = time.perf_counter()
        pipe.register(a, b, seed=2000 + s_, k=k)
        lat.append((time.perf_counter() - t0) * 1000.0)
    # per-stage breakdown of one pair through the stage calls (CUDA events on
    # the launching stream), each against its roofline
    stages = stage_breakdown(tdm, torch, dev, pairs[0], net, k, args.ransac_iters, prec)
    # roofline of the dominant kernel: conv2 on tcgen05 (useful FLOPs per launch / event time)
    conv2_ms, conv2_n = lt["conv2"]
    peaks, peak_kind = load_peaks()
    roof = None
    if conv2_n > 0:
        flop = CONV2_FLOP_PER_PATCH * 2 * k
        achieved = flop / (conv2_ms / conv2_n / 1000.0) / 1e12
        # burst peak: conv2 runs inside a ~14 ms step at full clocks, not a
        # seconds-long loop under the power cap
        peak = peaks["bf16_tflops"] if prec == "bf16" else None
        roof = {"kernel": "tc_conv_dxf2_kernel<bf16,x-,z-,y-pooled> (conv2 on CTA pairs, %d patches per launch)" % (2 * k),
                "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if peak else None, "peak_source": peak_kind + " bf16 burst",
                "traffic": profile_traffic("conv2_pair_bf16"),
                "ms_per_launch": conv2_ms / conv2_n, "share_of_step": (conv2_ms / args.steps) / ms_step,
                "note": "achieved counts useful FLOPs (valid outputs); the kernel issues %.2fx that in MMAs "
                        "(%.0f TFLOP/s of MMA work), and the measured burst peak is a cuBLAS GEMM, below the "
                        "probe's %d MAC/clk/SM" % (CONV2_MMA_FLOP_PER_PATCH / CONV2_FLOP_PER_PATCH,
                                                  achieved * CONV2_MMA_FLOP_PER_PATCH / CONV2_FLOP_PER_PATCH,
                                                  MMA_MAC_PER_CLK_SM)}
    layer_ms = {name: round(v[0] / max(1, v[1]), 4) for name, v in lt.items() if v[1]}
    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            v, sec, _, sample, parts = cpu_sample(pairs[0], k, args.ransac_iters)
            cpu = {"value": v, "unit": "pairs/s", "cores": os.cpu_count() or 1, "kind": "port",
                   "sample": sample + " (%.1f s)" % sec,
                   "parts_s_per_pair": {kk: round(vv, 3) for kk, vv in parts.items()}}
        out = {
            "metric": "pair registrations/s", "value": value, "unit": "pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": prec, "data": "synthetic",
            "config": {"workload": "demo pipeline pair: 2 x %d-point synthetic room fragments, 1 cm TDF, %d keypoints "
                                   "per fragment, 30^3 patches, 9-layer net (%s), mutual NN (%s), RANSAC %d trials, "
                                   "Kabsch refit" % (args.points, k, prec, prec, args.ransac_iters),
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "working set > L2 (net activations %.1f GB per step)" % (2 * k * 5.1e6 / 1e9),
                       "fp32_pairs_per_s": fp32,
                       "fp8_pairs_per_s": fp8,
                       "fp8_note": "FP8 (E4M3 conv3-8) is outside the 1e-2 descriptor tolerance (~8e-2): "
                                   "reported, not the headline",
                       "bf16_over_fp32": (value / fp32) if fp32 else None,
                       "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                      "n": len(lat)},
                       "net_tflops_useful": 2 * k * NET_FLOP_PER_PATCH / (ms_step / 1000.0) / 1e12,
                       "layer_ms_per_launch": layer_ms,
                       "last_result": {"matches": res.n_matches, "inliers": res.n_inliers} if res else None},
            "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roof,
            "stages": stages,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
        }
        print(json.dumps(out))
    pipe.close()
    net.close()
    try:
        os.unlink(wfile)
    except OSError:
        pass
    if dist is not None:
        dist.destroy_process_group()
    return 0


def rot_err_deg(R1, R2):
    c = (np.trace(R1.T @ R2) - 1.0) / 2.0
    return float(np.degrees(np.arccos(np.clip(c, -1.0, 1.0))))


def run_serve(args, rank, world, local):
    """Serving sweep: requests of demo-shaped pairs with points log-uniform in
    [20k, 300k] and keypoints uniform in [500, 5000] arrive as a Poisson
    process at rate lambda; RANSAC 50k trials.  The BF16 and FP8 forms are
    swept over lambda; the FP32 drop-in form is run at the highest lambda
    (saturated) beside them."""
    import threading
    import torch
    import __graft_entry__ as ge
    tdm = ge.load()
    from tdm_gb300 import synth
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(20260004)
    pool = []
    for i in range(8):
        n = int(np.exp(rng.uniform(np.log(20_000), np.log(300_000))))
        a, b, rt = synth.fragment_pair(20264000 + i, n_points=n)
        pool.append((a, b, rt))
    wfile = os.path.join(tempfile.gettempdir(), "tdm_serve_weights_%d.marvin" % os.getpid())
    tdm.write_seeded_weights(wfile, 20260000)
    cp = synth.fragment(20269999, n_points=150_000)
    cpd = torch.from_numpy(cp).to(dev)
    cg = tdm.grid_from_points_host(cp)
    _, ckg = tdm.keypoints(cpd, tdm.keypoint_indices(20269999, cp.shape[0], 256, device=dev), cg)
    calib = tdm.gather(tdm.tdf(cpd, cg), cg, ckg)
    lambdas = [float(x) for x in args.serve_lambdas.split(",")]
    forms = {}
    for form in ("bf16", "fp8", "fp32"):
        net = tdm.Net(marvin_path=wfile, precision=form)
        if form == "fp8":
            net.calibrate(calib)
        net.set_max_batch(1024)
        srv = tdm.Server(net, slots=args.serve_slots, hbm_budget_bytes=120 << 30, max_points=300_016,
                         max_keypoints=5000, max_voxels=80_000_000, match_precision="fp32" if form == "fp32" else "bf16",
                         ransac_seed=20260000, ransac_iters=50_000)
        for t in [srv.submit(pool[i % 8][0], pool[i % 8][1], 1, 1000) for i in range(srv.slots)]:  # warm-up
            srv.wait(t)
        sweep = []
        for lam in (lambdas if form != "fp32" else lambdas[-1:]):
            nreq = args.serve_requests if form != "fp32" else max(8, args.serve_requests // 2)
            reqs = []
            for r in range(nreq):
                a, b, rt = pool[int(rng.integers(0, len(pool)))]
                reqs.append((a, b, rt, int(rng.integers(500, 5001))))
            gaps = rng.exponential(1.0 / lam, len(reqs))
            tickets = [None] * len(reqs)
            t0 = time.perf_counter()

            def submitter():
                t_next = t0
                for i, (a, b, rt, k) in enumerate(reqs):
                    t_next += gaps[i]
                    d = t_next - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    tickets[i] = srv.submit(a, b, 3000 + i, k)

            th = threading.Thread(target=submitter)
            th.start()
            lat, rerr, terr = [], [], []
            th.join()
            for i, t in enumerate(tickets):
                res, ms = srv.wait(t)
                lat.append(ms)
                est = np.array(res.rt).reshape(4, 4)
                gt = reqs[i][2]
                rerr.append(rot_err_deg(est[:3, :3], gt[:3, :3]))
                terr.append(float(np.linalg.norm(est[:3, 3] - gt[:3, 3])))
            wall = time.perf_counter() - t0
            sweep.append({"lambda": lam, "requests": len(reqs), "pairs_per_s": len(reqs) / wall,
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                          "rot_err_deg_median": float(np.median(rerr)), "trans_err_m_median": float(np.median(terr)),
                          "mean_keypoints": float(np.mean([r[3] for r in reqs]))})
        forms[form] = {"slots": srv.slots, "sweep": sweep, "server": srv.stats(),
                       "saturated_pairs_per_s": max(d["pairs_per_s"] for d in sweep)}
        srv.close()
        net.close()
    os.unlink(wfile)
    best = forms["bf16"]["saturated_pairs_per_s"]
    if rank == 0:
        print(json.dumps({
            "metric": "pair registrations/s (serving, BF16)", "value": best, "unit": "pairs/s",
            "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic",
            "config": {"workload": "serving: Poisson arrivals, pairs with points log-uniform in [20k, 300k] and "
                                   "keypoints uniform in [500, 5000], RANSAC 50k trials, HBM budget 120 GB",
                       "forms": forms,
                       "bf16_over_fp32": best / forms["fp32"]["saturated_pairs_per_s"],
                       "fp8_over_fp32": forms["fp8"]["saturated_pairs_per_s"] / forms["fp32"]["saturated_pairs_per_s"]}}))
    return 0


def _event_ms(torch, fn, reps=3):
    stream = torch.cuda.current_stream()
    ts = []
    out = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts)), out


def run_tsdf(args, rank, world, local):
    """50 synthetic uint16 depth frames (640x480, sigma 2 mm, 1 % dropout) fused
    into a 512^3 TSDF at 6 mm, surface extraction, TDF at 1 cm, 2000 keypoints
    through the BF16 net."""
    import torch
    import __graft_entry__ as ge
    tdm = ge.load()
    from tdm_gb300 import synth
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    peaks, kind = load_peaks()
    frames, poses = synth.depth_sequence(20260003, n_frames=50)
    K = np.array([585.0, 0, 320.0, 0, 585.0, 240.0, 0, 0, 1], np.float32)
    dim = [512, 512, 512]
    origin = [-1.536, -1.536, 0.5]
    vs = 0.006
    trunc = float(np.float32(vs) * np.float32(5))
    V = 512 ** 3
    mm = torch.from_numpy(frames.astype(np.uint16).view(np.int16)).to(dev)
    depth = torch.empty(frames.shape, dtype=torch.float32, device=dev)
    ts = torch.empty(V, dtype=torch.float32, device=dev)
    wt = torch.empty(V, dtype=torch.float32, device=dev)

    def fuse():
        tdm.depth_from_mm(mm, depth)
        tdm.tsdf_init(ts, wt, dim)
        tdm.tsdf_integrate(ts, wt, dim, origin, vs, trunc, depth, K, poses)

    fuse()
    ms_fuse, _ = _event_ms(torch, fuse)
    ms_int, _ = _event_ms(torch, lambda: tdm.tsdf_integrate(ts, wt, dim, origin, vs, trunc, depth, K, poses))
    ms_ext, (pts, n) = _event_ms(torch, lambda: tdm.tsdf_extract(ts, wt, dim, origin, vs, 0.2, 1.0, max_pts=V // 8))
    npts = int(n.item())
    surf = pts[:npts].contiguous()
    wfile = os.path.join(tempfile.gettempdir(), "tdm_tsdf_weights_%d.marvin" % os.getpid())
    tdm.write_seeded_weights(wfile, 20260000)
    net = tdm.Net(marvin_path=wfile, precision="bf16")
    pipe = tdm.Pipeline(net, max_points=max(npts, 1) + 16, max_keypoints=2000, max_voxels=200_000_000)
    pipe.describe(surf, seed=1, k=2000)
    ms_desc, (kp, desc, g) = _event_ms(torch, lambda: pipe.describe(surf, seed=1, k=2000))
    launches = (50 + 31) // 32
    dram_bytes = launches * 16.0 * V + frames.size * 4  # grids read+written once per 32-frame launch
    ref_bytes = 50 * 16.0 * V + frames.size * 4          # the reference's per-frame passes
    total_ms = ms_fuse + ms_ext + ms_desc
    if rank == 0:
        print(json.dumps({
            "metric": "TSDF fragments/s (50 frames fused, extracted and described)", "value": 1000.0 / total_ms,
            "unit": "fragments/s", "n_gpus": world, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (TSDF), bf16 (net)", "data": "synthetic",
            "config": {"workload": "50 frames 640x480 uint16 mm into a 512^3 TSDF at 6 mm, trunc 5 voxels; surface "
                                   "extraction; TDF at 1 cm; 2000 keypoints; BF16 net",
                       "frames_per_s": 50 * 1000.0 / ms_int, "integrate_ms": ms_int, "fuse_ms_incl_init": ms_fuse,
                       "extract_ms": ms_ext, "surface_points": npts, "describe_ms": ms_desc,
                       "grid_dim_1cm": list(g.dim)},
            "roofline": {"kernel": "integrate_kernel (32 frames per launch)", "bound": "hbm",
                         "achieved": dram_bytes / ms_int / 1e6, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": dram_bytes / ms_int / 1e6 / peaks["hbm_gbs"], "traffic": None,
                         "note": "bytes = 16 B/voxel per launch + depth; the reference's per-frame passes would "
                                 "move %.1f GB, this moves %.1f GB" % (ref_bytes / 1e9, dram_bytes / 1e9)}}))
    pipe.close()
    net.close()
    os.unlink(wfile)
    return 0


def run_descriptors(args, rank, world, local):
    """5000 keypoints of one demo-shaped fragment: patches/s of the FP32, BF16
    and FP8 forms on the same 5000 patches, and the BF16/FP8 descriptors and
    5000 x 5000 mutual-NN results against the FP32 form."""
    import torch
    import __graft_entry__ as ge
    tdm = ge.load()
    from tdm_gb300 import synth
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    peaks, kind = load_peaks()
    a, b, _ = synth.fragment_pair(20260000)
    out = {}
    pt = []
    for pts, seed in ((a, 1), (b, 2)):
        pd = torch.from_numpy(pts).to(dev)
        g = tdm.grid_from_points_host(pts)
        _, kg = tdm.keypoints(pd, tdm.keypoint_indices(seed, pts.shape[0], 5000, device=dev), g)
        pt.append(tdm.gather(tdm.tdf(pd, g), g, kg))
    wfile = os.path.join(tempfile.gettempdir(), "tdm_desc_weights_%d.marvin" % os.getpid())
    tdm.write_seeded_weights(wfile, 20260000)
    desc = {}
    for prec in ("fp32", "bf16", "fp8"):
        net = tdm.Net(marvin_path=wfile, precision=prec)
        net.set_max_batch(5000)
        if prec == "fp8":
            net.calibrate(pt[1][:256].contiguous())
        net.forward(pt[0])
        net.set_timing(True)
        ms, d = _event_ms(torch, lambda: net.forward(pt[0]))
        lt = net.layer_times()
        d_b = net.forward(pt[1])
        desc[prec] = (d.clone(), d_b.clone())
        out[prec] = {"patches_per_s": 5000 * 1000.0 / ms, "ms": ms,
                     "tflops_useful": 5000 * NET_FLOP_PER_PATCH / ms / 1e9,
                     "frac_of_bf16_peak": 5000 * NET_FLOP_PER_PATCH / ms / 1e9 / peaks["bf16_tflops"],
                     "layer_ms": {kk: round(v[0] / max(v[1], 1), 3) for kk, v in lt.items() if v[1]}}
        net.close()
    ref_a, ref_b = desc["fp32"]
    _, _, nn_ab32, nn_ba32 = tdm.match_mnn(ref_a, ref_b, "fp32")
    # margin of the FP32 form's nearest neighbour: second-nearest / nearest distance (per row of a)
    d2 = torch.cdist(ref_a.double(), ref_b.double())
    two = torch.topk(d2, 2, dim=1, largest=False).values
    margin = (two[:, 1] / two[:, 0].clamp_min(1e-30)).float()
    p32, n32, _, _ = tdm.match_mnn(ref_a, ref_b, "fp32")
    p32 = set(map(tuple, p32[:int(n32.item())].cpu().numpy().tolist()))
    for prec in ("bf16", "fp8"):
        da, db = desc[prec]
        rel = float(torch.linalg.norm((da - ref_a).double()) / torch.linalg.norm(ref_a.double()))
        pairs, npairs, nn_ab, nn_ba = tdm.match_mnn(da, db, "bf16")
        agree = float(((nn_ab == nn_ab32).float().mean() + (nn_ba == nn_ba32).float().mean()) / 2)
        pp = set(map(tuple, pairs[:int(npairs.item())].cpu().numpy().tolist()))
        out[prec]["rel_l2_vs_fp32_form"] = rel
        out[prec]["nn_index_agreement_vs_fp32_form"] = agree
        same = (nn_ab == nn_ab32)
        for thr in (1.01, 1.05, 1.1):
            sel = margin > thr
            out[prec]["nn_agreement_where_margin_gt_%g" % thr] = (
                float(same[sel].float().mean()) if bool(sel.any()) else None, float(sel.float().mean()))
        out[prec]["mutual_pairs_shared_with_fp32_form"] = len(pp & p32) / max(len(p32), 1)
    ms_mnn, _ = _event_ms(torch, lambda: tdm.match_mnn(desc["bf16"][0], desc["bf16"][1], "bf16"))
    os.unlink(wfile)
    if rank == 0:
        print(json.dumps({
            "metric": "descriptor patches/s (BF16 form)", "value": out["bf16"]["patches_per_s"], "unit": "patches/s",
            "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic",
            "config": {"workload": "5000 keypoints of a 150k-point synthetic fragment, 5000 30^3 patches, 9-layer net",
                       "forms": out, "mnn_5000x5000_bf16_ms": ms_mnn,
                       "mnn_5000x5000_tflops": 2.0 * 5000 * 5000 * 512 / ms_mnn / 1e9,
                       "fp32_nn_margin_median": float(margin.median()),
                       "note": "rel-L2 against the FP64 oracle is checked in tests/ (BF16 <= 1e-2)"}}))
    return 0


def run_batch(args, rank, world, local):
    """64 fragments of seeded rooms (points log-uniform in [20k, 300k],
    keypoints uniform in [500, 5000], voxel 1 or 2 cm by coin flip) described
    as one batch per step: one persistent launch per stage, the sequence
    replayed as a CUDA graph, conv tiles from the autotuner.  FP8 (E4M3
    conv3..conv8, BF16 conv1..conv2), BF16 and FP32 forms on the same batch."""
    import torch
    import __graft_entry__ as ge
    tdm = ge.load()
    from tdm_gb300 import synth
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    peaks, kind = load_peaks()
    rng = np.random.default_rng(20260002)
    frags = []
    for p in range(args.batch_fragments // 2):  # both views of a seeded room pair, each subsampled on its own
        a, b, _ = synth.fragment_pair(20262000 + p, n_points=300_000)
        for pts in (a, b):
            n = min(int(np.exp(rng.uniform(np.log(20_000), np.log(300_000)))), pts.shape[0])
            sel = np.sort(rng.choice(pts.shape[0], n, replace=False))
            frags.append((pts[sel], 0.01 if rng.random() < 0.5 else 0.02, int(rng.integers(500, 5001))))
    F = len(frags)
    pts = np.concatenate([f[0] for f in frags]).astype(np.float32)
    off = np.concatenate([[0], np.cumsum([f[0].shape[0] for f in frags])]).astype(np.int64)
    vs = [f[1] for f in frags]
    ks = [f[2] for f in frags]
    seeds = [3000 + f for f in range(F)]
    K = int(sum(ks))
    pd = torch.from_numpy(pts).to(dev)
    kp_buf = torch.empty((K, 3), dtype=torch.float32, device=dev)
    desc_buf = torch.empty((K, 512), dtype=torch.float32, device=dev)
    # seeded 256-patch calibration batch and a 2048-patch tuning batch from a separate fragment
    cp = synth.fragment(20269998, n_points=150_000)
    cpd = torch.from_numpy(cp).to(dev)
    cg = tdm.grid_from_points_host(cp)
    _, ckg = tdm.keypoints(cpd, tdm.keypoint_indices(20269998, cp.shape[0], 2048, device=dev), cg)
    tune = tdm.gather(tdm.tdf(cpd, cg), cg, ckg)
    wfile = os.path.join(tempfile.gettempdir(), "tdm_batch_weights_%d.marvin" % os.getpid())
    tdm.write_seeded_weights(wfile, 20260000)
    forms, descs = {}, {}
    clk = None
    launches = None
    for prec in ("fp8", "bf16", "fp32"):
        net = tdm.Net(marvin_path=wfile, precision=prec)
        tiles = None
        if prec == "fp8":
            net.calibrate(tune[:256].contiguous())
        if prec != "fp32":
            tiles = net.autotune(tune, reps=2)
        if args.net_chunk > 0:
            net.set_max_batch(args.net_chunk)
        batch = tdm.Batch(net, max_fragments=F, max_points=pts.shape[0], max_keypoints=K,
                          max_voxels=3_000_000_000, use_graph=True)
        steps = args.steps if prec != "fp32" else 1
        warm = max(2, args.warmup) if prec != "fp32" else 2  # the first call runs directly and captures
        for _ in range(warm):
            _, _, grids = batch.describe(pd, off, vs, ks, seeds, kp_buf, desc_buf)
        stream = torch.cuda.current_stream()
        torch.cuda.synchronize()
        if prec == "bf16":
            clocks = Clocks(local)
            clocks.start()
        l0 = tdm.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            batch.describe(pd, off, vs, ks, seeds, kp_buf, desc_buf)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        if prec == "bf16":
            clk = clocks.stop()
            launches = tdm.launch_count() - l0
        st = batch.stats()
        descs[prec] = desc_buf.clone()
        forms[prec] = {"ms_per_batch": ms, "fragments_per_s": F * 1000.0 / ms, "patches_per_s": K * 1000.0 / ms,
                       "net_tflops_useful": K * NET_FLOP_PER_PATCH / ms / 1e9, "steps": steps,
                       "graph_replayed": st["replayed"], "launches_per_batch": st["launches_per_call"],
                       "tiles": tiles}
        if prec == "fp8":
            voxels = sum(g.voxels for g in grids)
            forms[prec]["voxels"] = voxels
            forms[prec]["batch_device_gb"] = batch.device_bytes / 1e9
        batch.close()
        net.close()
    ref = descs["fp32"].double()
    for prec in ("fp8", "bf16"):
        forms[prec]["rel_l2_vs_fp32_form"] = float(torch.linalg.norm(descs[prec].double() - ref) / torch.linalg.norm(ref))
    os.unlink(wfile)
    # headline: the BF16 form (the form within the 1e-2 descriptor tolerance);
    # FP8 (E4M3 conv3-8, ~8e-2 from the exact net) is reported beside it
    ms16 = forms["bf16"]["ms_per_batch"]
    achieved = K * NET_FLOP_PER_PATCH / ms16 / 1e9
    if rank == 0:
        print(json.dumps({
            "metric": "batched fragments described/s (BF16 form)", "value": F * 1000.0 / ms16, "unit": "fragments/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms16, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic",
            "config": {"workload": "%d fragments of seeded rooms, %d..%d points (log-uniform), %d keypoints in total "
                                   "(uniform 500..5000 each), voxel 1 or 2 cm; TDF, keypoints, gather and the net "
                                   "as one replayed CUDA graph per batch" % (F, min(len(f[0]) for f in frags),
                                                                            max(len(f[0]) for f in frags), K),
                       "points": int(pts.shape[0]), "keypoints": K, "forms": forms,
                       "fp8_note": "FP8 is outside the 1e-2 descriptor tolerance (E4M3 rounding, ~8e-2)",
                       "fp8_over_fp32": forms["fp32"]["ms_per_batch"] / forms["fp8"]["ms_per_batch"],
                       "bf16_over_fp32": forms["fp32"]["ms_per_batch"] / forms["bf16"]["ms_per_batch"],
                       "l2": "working set > L2 (%.1f GB of grids)" % (forms["fp8"]["voxels"] * 6 / 1e9)},
            "roofline": {"kernel": "whole batch (net dominant)", "bound": "tensor", "achieved": achieved,
                         "peak": peaks["bf16_tflops_sustained"], "unit": "TFLOP/s",
                         "frac": achieved / peaks["bf16_tflops_sustained"],
                         "note": "useful net FLOPs per batch / batch time, against the measured BF16 sustained peak "
                                 "(%s); the batch runs about a second at full load" % kind},
            "clocks": clk, "gpu_launches": launches}))
    return 0


def run_registration(args, rank, world, local):
    """Geometric-registration benchmark of the reference, end to end on a
    synthetic scene: every fragment pair registered (BF16 path), its surface
    overlap computed on the GPU and filtered as writeLog.m does (> 0.30), the
    ground truth made as getGtInfoLog.m does (pairs overlapping >= 0.30 at
    3 cm, information from <= 5,000 correspondences within 6 mm), and the log
    scored with mrEvaluateRegistration.m's recall / precision."""
    import torch
    import __graft_entry__ as ge
    tdm = ge.load()
    from scipy.spatial import cKDTree
    from tdm_gb300 import evaluation, synth
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    views = synth.scene_fragments(20266000, n_views=args.reg_views, n_points=args.points)
    F = len(views)
    pts = [torch.from_numpy(p).to(dev) for p, _ in views]
    wfile = os.path.join(tempfile.gettempdir(), "tdm_reg_weights_%d.marvin" % os.getpid())
    tdm.write_seeded_weights(wfile, 20260000)
    net = tdm.Net(marvin_path=wfile, precision="bf16")
    pipe = tdm.Pipeline(net, max_keypoints=args.keypoints, max_points=args.points + 16, max_voxels=80_000_000,
                        match_precision="bf16", ransac_seed=20260000, ransac_iters=args.ransac_iters)
    pairs = [(i, j) for i in range(F) for j in range(i + 1, F)]
    pipe.register(pts[0], pts[1], seed=1, k=args.keypoints)  # warm-up
    tdm.overlap(pts[0], pts[1], np.eye(4)[:3], 0.05)  # warm-up: the first call in a process takes ~0.24 s
    # describe once, register many (getKeyptsAndDesc.m, then register2Fragments.m
    # per pair): every view is described into the device store once
    store = tdm.Store(F * 2100 * args.keypoints + (1 << 20))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    launches0 = tdm.launch_count()
    for i in range(F):
        store.describe(pipe, i + 1, pts[i], 1000 + i, args.keypoints)
    torch.cuda.synchronize()
    t_desc = time.perf_counter() - t0
    results = []
    for i, j in pairs:
        r = tdm.register_stored(pipe, store, i + 1, j + 1)
        rt = np.array(r.rt).reshape(4, 4)
        ov = tdm.overlap(pts[i], pts[j], rt[:3], 0.05)
        results.append((i, j, rt, ov[0] / pts[i].shape[0]))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    launches = tdm.launch_count() - launches0
    store_stats = store.stats()
    store.close()
    log = evaluation.log_records(results, F)
    gt_log, gt_info, rot_err = [], [], []
    rng = np.random.default_rng(5)
    for (i, j), (_, _, rt, _) in zip(pairs, results):
        rel = np.linalg.inv(views[i][1]) @ views[j][1]
        if tdm.overlap(pts[i], pts[j], rel[:3], 0.03)[0] / pts[i].shape[0] < 0.3:
            continue
        q = views[j][0].astype(np.float64) @ rel[:3, :3].T + rel[:3, 3]
        d, _ = cKDTree(views[i][0]).query(q, k=1)
        corres = q[d < 0.006]
        if corres.shape[0] > 5000:
            corres = corres[rng.choice(corres.shape[0], 5000, replace=False)]
        gt_log.append((i, j, F, rel))
        gt_info.append((i, j, F, evaluation.gt_information(corres)))
        dR = rel[:3, :3].T @ rt[:3, :3]
        rot_err.append(float(np.degrees(np.arccos(np.clip((np.trace(dR) - 1) / 2, -1, 1)))))
    recall, precision = evaluation.evaluate_registration(log, gt_log, gt_info)
    pipe.close()
    net.close()
    os.unlink(wfile)
    if rank == 0:
        print(json.dumps({
            "metric": "fragment pairs registered and scored/s (BF16)", "value": len(pairs) / wall, "unit": "pairs/s",
            "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic",
            "config": {"workload": "%d fragments of one synthetic room (%d points, %d keypoints each): all %d pairs "
                                   "registered, GPU surface overlap, writeLog filter, mrEvaluateRegistration scoring"
                                   % (F, args.points, args.keypoints, len(pairs)),
                       "pairs": len(pairs), "logged_pairs": len(log), "gt_pairs": len(gt_log),
                       "net_passes": F, "describe_s": t_desc, "match_and_overlap_s": wall - t_desc,
                       "gpu_launches": launches, "store": store_stats,
                       "recall": recall, "precision": precision,
                       "rotation_error_deg_median_gt_pairs": float(np.median(rot_err)) if rot_err else None,
                       "note": "random He-normal weights: the scores measure the pipeline, not a trained net"}}))
    return 0


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.serve:
        return run_serve(args, rank, world, local)
    if args.tsdf:
        return run_tsdf(args, rank, world, local)
    if args.descriptors:
        return run_descriptors(args, rank, world, local)
    if args.batch:
        return run_batch(args, rank, world, local)
    if args.registration:
        return run_registration(args, rank, world, local)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
