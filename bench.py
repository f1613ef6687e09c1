#!/usr/bin/env python3
"""Throughput benchmark of the multi-pass PIV path on one GB300.

Workload: 1024x1024 uint8 synthetic particle-image pairs (0.03 particles/px,
sinusoidal shear u = 6 sin(2 pi y/256), v = 2 cos(2 pi x/512)), three passes
64 -> 32 -> 16 px at 50% overlap (n_fft = 2, so 128/64/32-point DFTs),
bilinear deformation on pass 2 and cubic B-spline on pass 3 (deforming_order
1, 3, 3), Gaussian subpixel fit, median validation (tol 2, 3x3) with two
revalidated spring replacements, smoothn with GCV between passes, float32.

A step is one run of the whole pipeline over a batch of pairs resident in
HBM (captured once as a CUDA graph and replayed). ``value`` is pairs/s over
the timed steps; ``e2e`` is the same through the public Python API with the
frames copied from pinned host memory and the fields copied back every step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--pairs B] [--impl gpu|reference]

Under torchrun each rank processes its own batch on its own GPU (replicas,
no collective on the data path); rank 0 prints one JSON line.
"""

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "openpiv-python-gpu_gb300")
for p in (PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "frame pairs/s (1024x1024, 64->32->16 px three-pass PIV) on 1 GB300"
WORKLOAD = ("1024x1024 uint8 pairs, 0.03 ppp, shear 6/2 px; 64->32->16 px @50%, n_fft=2; deforming_order (1,3,3); "
            "median validation tol 2 + 2 revalidated spring replacements; smoothn GCV; float32")
FRAME = (1024, 1024)
DISTINCT = 16
# Arithmetic of the correlation DFTs per form (fields, fits, validation and
# deformation are float32; smoothn's GCV float64 in every form).
DTYPE_OF_FORM = {
    "fft": "f32",
    "tensor": "f16 operands, f32 accumulation (tcgen05 kind::f16)",
    "tensor_split": "f16 hi/lo operand pairs, 3 products per stage, f32 accumulation (tcgen05 kind::f16)",
    "tensor_refined": "f16 operands, f32 accumulation (tcgen05 kind::f16) for the integer peak; f32 direct sums "
                      "for the subpixel fit; near ties on the f32 FFT",
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--pairs", type=int, default=128, help="pairs per step per GPU")
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--dft", choices=["fft", "tensor", "tensor_split", "tensor_refined"], default="tensor_refined",
                    help="correlation engine of the chosen form (default: the refined tensor form, float32 FFT "
                         "parity)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-modes", action="store_true",
                    help="skip the mixed-size, serving and precision runs the default line summarises")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain FP32 FFT form beside the tensor form")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default correlation launch variants instead of autotuning them per pass")
    ap.add_argument("--no-others", action="store_true",
                    help="skip timing the other tensor forms (fp16, hi/lo split, refined) beside the chosen one")
    ap.add_argument("--no-split", action="store_true",
                    help="skip timing the hi/lo split tensor form beside the chosen one")
    ap.add_argument("--serve", action="store_true",
                    help="serving form instead: Poisson arrivals of mixed-size pairs through the continuous-batching "
                         "loop, p50/p99 latency and pairs/s beside the plain per-pair path")
    ap.add_argument("--mixed", action="store_true",
                    help="batched form instead: one submission of 64 pairs of four frame sizes, replayed as one graph")
    ap.add_argument("--precision", action="store_true",
                    help="precision form instead: 16 pairs of 2048x2048, 32->16 px at 75%% overlap, the faster of "
                         "the hi/lo split and refined tensor forms beside the other tensor forms and the plain FP32 "
                         "FFT form, RMS vs the float64 oracle")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: arrivals per second")
    ap.add_argument("--requests", type=int, default=400, help="serving: number of requests")
    return ap.parse_args()


def piv_settings():
    from openpiv_gpu import synthetic

    kw = dict(synthetic.CONFIGS[2]["piv"])
    mss = kw.pop("min_search_size")
    return mss, kw


def _make_pair(k):
    sys.path.insert(0, PKG)
    from openpiv_gpu import synthetic

    a, b, _, _ = synthetic.config_case(2, k)
    return a, b


def _make_serving_pair(args):
    k, shape = args
    sys.path.insert(0, PKG)
    from openpiv_gpu import synthetic

    a, b, _, _ = synthetic.config_case(5, k, shape=tuple(shape))
    return a, b


def _make_mixed_pair(k):
    sys.path.insert(0, PKG)
    from openpiv_gpu import synthetic

    a, b, _, _ = synthetic.config_case(4, k)
    return a, b


def _make_precision_pair(k):
    sys.path.insert(0, PKG)
    from openpiv_gpu import synthetic

    a, b, _, _ = synthetic.config_case(3, k)
    return a, b


def _oracle_case(args):
    """Float64 oracle fields of pair k of workload cfg (optionally resized):
    (u, v, seconds)."""
    cfg, k, shape = args
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, PKG)
    sys.path.insert(0, ROOT)
    from oracle.piv_oracle import OraclePIV
    from openpiv_gpu import synthetic

    a, b, _, piv = synthetic.config_case(cfg, k, shape=None if shape is None else tuple(shape))
    piv = dict(piv)
    piv["dtype_f"] = "float64"
    mss = piv.pop("min_search_size")
    t = time.perf_counter()
    u, v = OraclePIV(a.shape, mss, **piv)(a, b)
    return u, v, time.perf_counter() - t


def _rms(u, v, u64, v64):
    import numpy as np

    return float(np.sqrt(np.mean((np.asarray(u, dtype=np.float64) - u64) ** 2 +
                                 (np.asarray(v, dtype=np.float64) - v64) ** 2)))


def _precision_oracle(args):
    """Float64 oracle fields of the 512x512 accuracy case of the precision workload."""
    k, shape = args
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, PKG)
    sys.path.insert(0, ROOT)
    from oracle.piv_oracle import OraclePIV
    from openpiv_gpu import synthetic

    a, b, _, piv = synthetic.config_case(3, k, shape=shape)
    piv = dict(piv)
    piv["dtype_f"] = "float64"
    mss = piv.pop("min_search_size")
    u, v = OraclePIV(a.shape, mss, **piv)(a, b)
    return a, b, u, v


def generate_pairs(n):
    """n distinct seeded pairs (seed 2000 + k), rendered in a spawn pool."""
    import multiprocessing as mp

    workers = max(1, min(n, os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_make_pair, range(n))


# ---------------------------------------------------------------------------
# CPU oracle (the reference algorithm restated in NumPy/SciPy).
# ---------------------------------------------------------------------------
def _oracle_pair(args):
    k, dtype_f = args
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, PKG)
    sys.path.insert(0, ROOT)
    from oracle.piv_oracle import OraclePIV
    from openpiv_gpu import synthetic

    a, b, _, piv = synthetic.config_case(2, k)
    piv = dict(piv)
    piv["dtype_f"] = dtype_f
    mss = piv.pop("min_search_size")
    t = time.perf_counter()
    u, v = OraclePIV(a.shape, mss, **piv)(a, b)
    return time.perf_counter() - t, u, v


def cpu_pool(workers):
    import multiprocessing as mp

    return mp.get_context("spawn").Pool(workers)


def cpu_throughput(pool, workers, steps, warmup, dtype_f="float32"):
    """Times `steps` rounds of one oracle pair per worker; returns pairs/s."""
    for _ in range(warmup):
        pool.map(_oracle_pair, [(k % DISTINCT, dtype_f) for k in range(workers)])
    t0 = time.perf_counter()
    for s in range(steps):
        pool.map(_oracle_pair, [((s * workers + k) % DISTINCT, dtype_f) for k in range(workers)])
    dt = time.perf_counter() - t0
    return steps * workers / dt, dt


# ---------------------------------------------------------------------------
# Clock sampling during the timed region.
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self, first_sample_s=3.0):
        """Start sampling every 200 ms and wait (at most `first_sample_s`) for
        the first sample, so that a timed region of a fraction of a second
        is not over before nvidia-smi has started."""
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=fd,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            os.unlink(self.path)
            return
        finally:
            os.close(fd)
        deadline = time.monotonic() + first_sample_s
        while time.monotonic() < deadline and self.proc.poll() is None and os.path.getsize(self.path) == 0:
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1].split()[0]), float(parts[2].split()[0]), parts[5:9]))
                except ValueError:
                    continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, s in enumerate(r) if s.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# Roofline helpers.
# ---------------------------------------------------------------------------
def tc_executed_flops(ss, N, split=False):
    """FLOPs the tensor engine executes per window pair: packed real DFT along x
    (both frames), along y (both frames), the inverse along f_r over N/2 packed
    columns as two products of K = N on the folded frequency pairs, real
    inverse along f_c (three products per stage with hi/lo split operands)."""
    macs = 2 * ss * ss * N + 2 * N * ss * N + (N // 2) * (2 * N) * N + N * N * N
    return 2 * macs * (3 if split else 1)


def corr_flops(ss, N):
    """Algorithmic FLOPs of one window-pair correlation: two real-to-complex and
    one complex-to-real 2-D FFT at 2.5 N^2 log2(N^2) each, the conjugate
    product and the mean removal."""
    return 3 * 2.5 * N * N * math.log2(N * N) + 6 * N * (N // 2 + 1) + 4 * ss * ss


def sgemm_tflops(torch):
    """FP32 SIMT reference throughput: cuBLAS SGEMM with TF32 disabled."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda")
    b = torch.randn(n, n, device="cuda")
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return 2 * n ** 3 / (best * 1e-3) / 1e12


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernels from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


# ---------------------------------------------------------------------------
# Arms.
# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
# Ranks (replicas only: each rank processes its own pairs; the process group
# only aligns the timed regions and takes the slowest rank's time).
# ---------------------------------------------------------------------------
def shard_pairs(rank, batch, distinct=DISTINCT):
    """Indices of the distinct synthetic pairs rank `rank` processes: batch
    pairs starting at rank * batch, cycling through the distinct pairs."""
    return [(rank * batch + k) % distinct for k in range(batch)]


def max_over_ranks(value, dist=None):
    """The largest `value` over the ranks of the default process group (the
    value itself without one)."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    pool = cpu_pool(workers)
    value, dt = cpu_throughput(pool, workers, args.steps, args.warmup)
    pool.close()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded particle images)",
        "config": {"workload": WORKLOAD, "pairs_per_step": workers, "frame": list(FRAME)},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": workers, "kind": "port",
                         "sample": f"{workers} pairs per step, one per worker process, NumPy/SciPy restatement "
                                   "of the reference algorithm in float32"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    torch.cuda.set_device(local)

    # CPU pool first (spawn), before heavy CUDA work.
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_pool(os.cpu_count() or 1)

    import __graft_entry__

    __graft_entry__.build()
    from openpiv_gpu import _lib
    from openpiv_gpu.gpu_process import PIVGPU

    lib = _lib.load()
    B = args.pairs
    pairs = generate_pairs(DISTINCT)
    idx = shard_pairs(rank, B)
    host_a = np.stack([pairs[i][0] for i in idx])
    host_b = np.stack([pairs[i][1] for i in idx])
    fa = torch.as_tensor(host_a).cuda()
    fb = torch.as_tensor(host_b).cuda()
    mss, kw = piv_settings()
    stream = torch.cuda.Stream()

    def make(dft):
        proc = PIVGPU(FRAME, mss, **kw, dft=dft, autotune=not args.no_autotune)
        with torch.cuda.stream(stream):
            for _ in range(max(1, args.warmup)):
                proc.run_batch(fa, fb)
        stream.synchronize()
        return proc

    def graph_time(proc):
        plan = proc.plan_handle(fa, B)
        m, n = proc.piv_fields[-1].field_shape
        u = torch.empty((B, m, n), dtype=torch.float64, device="cuda")
        v = torch.empty_like(u)
        val = torch.empty((B, m, n), dtype=torch.uint8, device="cuda")
        out = torch.empty_like(val)
        nk = ctypes.c_int(0)
        s = stream.cuda_stream
        _lib.check(lib.piv_plan_graph_capture(plan, B, fa.data_ptr(), fb.data_ptr(), u.data_ptr(), v.data_ptr(),
                                              val.data_ptr(), out.data_ptr(), ctypes.byref(nk), s))
        for _ in range(args.warmup):
            _lib.check(lib.piv_plan_graph_launch(plan, s))
        stream.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            _lib.check(lib.piv_plan_graph_launch(plan, s))
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms = e0.elapsed_time(e1)
        return ms, nk.value, (u, v)

    proc = make(args.dft)
    sampler = ClockSampler(local)
    sampler.start()
    ms, kernels, (u_dev, v_dev) = graph_time(proc)
    clocks = sampler.stop()
    ms = max_over_ranks(ms, dist)
    ms_step = ms / args.steps
    value = B * world / (ms_step * 1e-3)
    windows_per_pair = sum(f.n_wins for f in proc.piv_fields)

    # End to end through the public API: pinned host frames in, fields out
    # (PIVGPU.run_batches: two plans on two streams, so that a batch's upload
    # and download overlap the previous batch's kernels). Measured right after
    # the chosen form's own timing, before the other forms' pipelines are
    # built beside it (a user runs one).
    pin_a = torch.as_tensor(host_a).pin_memory()
    pin_b = torch.as_tensor(host_b).pin_memory()
    na, nb = pin_a.numpy(), pin_b.numpy()
    for _ in proc.run_batches((na, nb) for _ in range(args.warmup)):
        pass
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for res_u, res_v in proc.run_batches((na, nb) for _ in range(args.steps)):
        pass
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, dist)
    m, n = proc.piv_fields[-1].field_shape
    e2e = {"value": B * world * args.steps / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": int(2 * B * FRAME[0] * FRAME[1]),
           "d2h_bytes_per_step": int(B * m * n * (8 + 8 + 1 + 1))}

    plain = None
    proc_plain = None
    if args.dft != "fft" and not args.no_plain:
        proc_plain = make("fft")
        ms_p, _, _ = graph_time(proc_plain)
        ms_p = max_over_ranks(ms_p, dist)
        plain = {"pairs_per_s": B * world / (ms_p / args.steps * 1e-3), "ms_per_step": ms_p / args.steps}
        plain["chosen_over_plain"] = value / plain["pairs_per_s"]
    # The other tensor forms, timed the same way.
    others, other_procs = {}, {}
    for form in ("tensor", "tensor_split", "tensor_refined"):
        if form == args.dft or args.dft == "fft" or args.no_others or (form == "tensor_split" and args.no_split):
            continue
        other_procs[form] = make(form)
        ms_o, _, _ = graph_time(other_procs[form])
        ms_o = max_over_ranks(ms_o, dist)
        others[form] = {"pairs_per_s": B * world / (ms_o / args.steps * 1e-3), "ms_per_step": ms_o / args.steps}
        if plain:
            others[form]["over_plain"] = others[form]["pairs_per_s"] / plain["pairs_per_s"]
    split = others.get("tensor_split")
    proc_split = other_procs.get("tensor_split")

    # Stage breakdown (CUDA events inside the run, same stream).
    plan = proc.plan_handle(fa, B)
    _lib.check(lib.piv_plan_set_timing(plan, 1))
    n_stage_runs = 3
    with torch.cuda.stream(stream):
        for _ in range(n_stage_runs):
            proc.run_batch(fa, fb)
    stream.synchronize()
    n_it = len(proc.piv_fields)
    cap = n_it * 6 + 2
    buf = (ctypes.c_float * cap)()
    runs = ctypes.c_int(0)
    _lib.check(lib.piv_plan_stage_times(plan, buf, cap, ctypes.byref(runs)))
    _lib.check(lib.piv_plan_set_timing(plan, 0))
    stage_ms = {}
    for k in range(n_it):
        for s, name in enumerate(_lib.STAGES):
            t = buf[k * 6 + s] / max(1, runs.value)
            if t > 0:
                stage_ms[f"it{k}.{name}"] = round(t, 4)

    # Dominant kernel roofline: the correlation stage with the largest time.
    corr = {k: v for k, v in stage_ms.items() if k.endswith("correlate")}
    dom = max(corr, key=corr.get)
    kdom = int(dom[2:dom.index(".")])
    f = proc.piv_fields[kdom]
    N = proc._iterations[kdom].fft_size
    n_win = B * f.n_wins
    flops = n_win * corr_flops(f.search_size, N)
    achieved = flops / (corr[dom] * 1e-3) / 1e12
    peaks = measured_peaks()
    traffic_w = ncu_traffic()
    on_tensor = N == 2 * f.search_size and (
        args.dft in ("tensor", "tensor_refined", "tensor_split") and f.search_size in (16, 32, 64))
    if on_tensor:
        peak = peaks.get("bf16_tflops", 1900.0)
        unit, bound = "TFLOP/s", "tensor"
        src = "MEASURED_PEAKS.json bf16_tflops (burst)" if "bf16_tflops" in peaks else "fallback 1900 TFLOP/s"
        key = f"correlate_tc{'s' if args.dft == 'tensor_split' else ''}_N{N}"
    else:
        peak, unit, bound, src = sgemm_tflops(torch), "TFLOP/s", "fp32", "cuBLAS SGEMM (TF32 off) measured here"
        key = f"correlate_fft_N{N}"
    per_window_traffic = traffic_w.get(key)
    roofline = {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
                "traffic": per_window_traffic * n_win if per_window_traffic else None,
                "kernel": f"correlate pass {kdom + 1} (ss={f.search_size}, N={N}, {n_win} windows/launch, "
                          f"{'tcgen05' if on_tensor else 'fft'}"
                          f"{'; the stage: fp16 engine, peak refinement and near-tie FFT reruns' if args.dft == 'tensor_refined' else ''})",
                "peak_source": src, "launch_ms": corr[dom],
                "algorithmic_flops_per_window": corr_flops(f.search_size, N)}
    if on_tensor:
        roofline["executed_tflops"] = (n_win * tc_executed_flops(f.search_size, N, args.dft == "tensor_split"
                                                                 and f.search_size in (16, 32))
                                       / (corr[dom] * 1e-3) / 1e12)
        roofline["executed_frac"] = roofline["executed_tflops"] / peak
    if roofline["traffic"]:
        # The same launch against the HBM roofline: DRAM bytes / launch time.
        hbm = peaks.get("hbm_gbs")
        roofline["dram_gbs"] = roofline["traffic"] / (corr[dom] * 1e-3) / 1e9
        roofline["dram_frac"] = roofline["dram_gbs"] / hbm if hbm else None
    if on_tensor and args.dft != "tensor":
        # The refined and split forms' correlation stages hold more than one
        # kernel; the dominant kernel is a pass's tensor-core engine alone,
        # timed here with CUDA events on its stream over the step's pairs and
        # that pass's geometry (passes 2 and 3 correlate deformed float32
        # frames: the step's frames in float32 stand in for them).
        engine = {}
        frames_f32 = (fa.float(), fb.float())
        for k, fk in enumerate(proc.piv_fields):
            Nk = proc._iterations[k].fft_size
            if not (Nk == 2 * fk.search_size and fk.search_size in (16, 32, 64)):
                continue
            mode = "tensor_split" if args.dft == "tensor_split" and fk.search_size in (16, 32) else "tensor"
            da, db, pt = (fa, fb, "u8") if k == 0 else (frames_f32[0], frames_f32[1], "f32")
            ue = torch.empty((B, *fk.field_shape), dtype=torch.float32, device="cuda")
            ve = torch.empty_like(ue)

            def run_engine():
                _lib.check(lib.piv_correlate(ctypes.byref(fk.geometry), B, da.data_ptr(), db.data_ptr(),
                                             _lib.PIXEL[pt], 0, Nk, 1, _lib.SUBPIXEL["gaussian"], None, ue.data_ptr(),
                                             ve.data_ptr(), None, None, 0, 2, None, _lib.DFT[mode], stream.cuda_stream))

            for _ in range(3):
                run_engine()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(5):
                run_engine()
            e1.record(stream)
            stream.synchronize()
            engine[k] = (e0.elapsed_time(e1) / 5, mode, Nk)
        if engine:
            ke = max(engine, key=lambda k: engine[k][0])
            ms_e, mode, Ne = engine[ke]
            fe = proc.piv_fields[ke]
            n_win_e = B * fe.n_wins
            achieved_e = n_win_e * corr_flops(fe.search_size, Ne) / (ms_e * 1e-3) / 1e12
            tw = traffic_w.get(f"correlate_tc{'s' if mode == 'tensor_split' else ''}_N{Ne}")
            stage = dict(roofline)
            roofline = {"bound": "tensor", "achieved": achieved_e, "peak": peak, "unit": "TFLOP/s",
                        "frac": achieved_e / peak, "traffic": tw * n_win_e if tw else None,
                        "kernel": f"{'k_corr_tc64' if fe.search_size == 64 else f'k_corr_tc<{fe.search_size}>'} "
                                  f"({mode} engine) alone, pass {ke + 1} (ss={fe.search_size}, N={Ne}, "
                                  f"{n_win_e} windows/launch); the slowest engine launch of the step",
                        "peak_source": src, "launch_ms": ms_e,
                        "algorithmic_flops_per_window": corr_flops(fe.search_size, Ne),
                        "engine_ms_per_pass": {f"pass {k + 1}": round(v[0], 4) for k, v in engine.items()}}
            roofline["executed_tflops"] = (n_win_e * tc_executed_flops(fe.search_size, Ne, mode == "tensor_split")
                                           / (ms_e * 1e-3) / 1e12)
            roofline["executed_frac"] = roofline["executed_tflops"] / peak
            if roofline["traffic"] and peaks.get("hbm_gbs"):
                roofline["dram_gbs"] = roofline["traffic"] / (ms_e * 1e-3) / 1e9
                roofline["dram_frac"] = roofline["dram_gbs"] / peaks["hbm_gbs"]
            roofline["stage"] = stage

    device_status = proc.status()  # PIV_OK unless a bounded device-side wait gave up

    # Accuracy of every form timed here: pair 0 against the float64 oracle and
    # the float32 parity oracle (the reference algorithm), and the near-tie
    # windows (integer peaks the engine does not resolve) of a whole batch.
    accuracy = None
    if rank == 0 and not args.no_accuracy and cpu is not None:
        (_, u64, v64), (_, u32, v32) = cpu.map(_oracle_pair, [(0, "float64"), (0, "float32")])
        rms = lambda a, b, c, d: float(np.sqrt(np.mean((a - b) ** 2 + (c - d) ** 2)))

        def form_accuracy(p):
            pu, pv = p.run_batch(fa, fb)
            ties = p.near_ties()
            gu, gv = pu[0].cpu().numpy(), pv[0].cpu().numpy()
            return {"rms_px_vs_fp64_oracle": rms(gu, u64, gv, v64), "rms_px_vs_fp32_oracle": rms(gu, u32, gv, v32),
                    "max_px_vs_fp32_oracle": float(max(np.abs(gu - u32).max(), np.abs(gv - v32).max())),
                    "near_ties_per_pass": ties, "windows_per_pass": [B * f.n_wins for f in p.piv_fields]}

        forms = {args.dft: form_accuracy(proc)}
        if proc_plain is not None:
            forms["fft"] = form_accuracy(proc_plain)
        for form, p in other_procs.items():
            forms[form] = form_accuracy(p)
        accuracy = dict(forms[args.dft], form=args.dft, forms=forms,
                        pair="pair 0 of the step against the oracles; near ties over the whole step")

    cpu_baseline = None
    if cpu is not None:
        workers = os.cpu_count() or 1
        cval, cdt = cpu_throughput(cpu, workers, 1, 0)
        cpu.close()
        cpu_baseline = {"value": cval, "unit": "pairs/s", "cores": workers, "kind": "port",
                        "sample": f"{workers} pairs, one per worker process (NumPy/SciPy restatement of the "
                                  f"reference algorithm, float32), {cdt:.1f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE_OF_FORM[args.dft], "data": "synthetic (seeded particle images)",
            "config": {"workload": WORKLOAD, "pairs_per_step": B, "distinct_pairs": DISTINCT, "frame": list(FRAME),
                       "form": args.dft, "graph": True,
                       "l2": "inputs larger than L2 (B x 2 MiB frames + 8 MiB float frames per pair per pass)"},
            "windows_per_s": value * windows_per_pair, "windows_per_pair": windows_per_pair,
            "plain_form": plain, "split_form": split, "other_forms": others,
            "tuning": {"form": [t["name"] for t in proc.tuning()],
                       "default_ms": [t["ms"][0] for t in proc.tuning()],
                       "tuned_ms": [None if t["ms"][t["variant"]] is None else t["ms"][t["variant"]]
                                    for t in proc.tuning()],
                       "plain": [t["name"] for t in proc_plain.tuning()] if proc_plain is not None else None,
                       "variants_ms": [dict(zip(t["variants"], t["ms"])) for t in proc.tuning()]},
            "e2e": e2e, "gpu_launches": kernels * args.steps, "kernels_per_step": kernels,
            "roofline": roofline, "cpu_baseline": cpu_baseline, "clocks": clocks, "accuracy": accuracy,
            "device_status": device_status,
            "stage_ms": stage_ms,
        }
        if world == 1 and not args.no_modes:
            line["modes"] = other_modes()
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def other_modes(timeout_s=300):
    """The mixed-size submission, serving and precision workloads, each run
    once by this script in a process of its own (after the timed steps
    above), summarised for the default line; a mode that fails or runs out
    of time reports why instead (the three together take under two minutes
    on a GB300; the limit bounds the default run if one stalls)."""
    runs = {"mixed": ["--mixed", "--steps", "5", "--warmup", "3"], "serve": ["--serve"],
            "precision": ["--precision", "--steps", "5", "--warmup", "3"]}
    keep = {"mixed": ("metric", "value", "unit", "form", "chosen", "plain_form", "chosen_over_plain", "config"),
            "serve": ("metric", "value", "unit", "p50_ms", "p99_ms", "mean_ms", "requests", "arrival_rate", "form",
                      "plain_per_pair", "accuracy", "continuous_batching", "device_status", "config"),
            "precision": ("metric", "value", "unit", "form", "ms_per_step", "chosen", "fp16_tensor_form", "plain_form",
                          "chosen_over_plain", "config")}
    out = {}
    for name, extra in runs.items():
        try:
            r = subprocess.run([sys.executable, os.path.abspath(__file__)] + extra, capture_output=True, text=True,
                               timeout=timeout_s, cwd=ROOT)
            lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not lines:
                out[name] = {"error": f"exit {r.returncode}: {r.stderr.strip().splitlines()[-1:] or ''}"}
                continue
            d = json.loads(lines[-1])
            out[name] = {k: d[k] for k in keep[name] if k in d}
            if name in ("mixed", "precision") and isinstance(out[name].get("chosen"), dict):
                out[name]["chosen"] = {k: v for k, v in out[name]["chosen"].items() if k not in ("tuning",)}
        except subprocess.TimeoutExpired:
            out[name] = {"error": f"did not finish within {timeout_s} s"}
    return out


def run_serve(args):
    """Serving form: Poisson arrivals (rate args.rate) of pairs whose size is
    drawn uniformly from the five serving sizes, through PIVServer (the chosen
    form, then the other two tensor forms on the same arrivals; continuous
    batching, lanes per size) and, beside it, through the plain per-pair path
    (each pair alone, in arrival order, FP32 FFT form)."""
    import multiprocessing as mp

    import numpy as np
    import torch

    sys.path.insert(0, PKG)
    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.gpu_process import PIVGPU
    from openpiv_gpu.serving import PIVServer, serve_arrivals

    shapes = list(synthetic._CFG5_SHAPES)
    per_shape = 2
    jobs = [(100 + k, shapes[k % len(shapes)]) for k in range(per_shape * len(shapes))]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        rendered = pool.map(_make_serving_pair, jobs)
    pool_by_shape = {}
    for (k, shape), pair in zip(jobs, rendered):
        pool_by_shape.setdefault(tuple(shape), []).append(pair)
    _build.build()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(5000)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, args.requests))
    picks = rng.integers(len(shapes), size=args.requests)
    frames = [pool_by_shape[tuple(shapes[i])][j % per_shape] for j, i in enumerate(picks)]
    # Accuracy: the first pair of every size against the float64 oracle, run
    # on the host cores while the GPU serves.
    oracle_pool = mp.get_context("spawn").Pool(len(shapes))
    acc_jobs = {tuple(sh): oracle_pool.apply_async(_oracle_case, ((5, 100 + i, sh),)) for i, sh in enumerate(shapes)}
    first_pair = {tuple(sh): pool_by_shape[tuple(sh)][0] for sh in shapes}
    settings = dict(synthetic.CONFIGS[5]["piv"])

    def serve_form(form):
        server = PIVServer(settings, max_batch=8, slots_per_shape=2, dft=form)
        for shape in shapes:  # lanes, plans and first launches outside the timed run
            a, b = pool_by_shape[tuple(shape)][0]
            server.submit(a, b)
        server.drain()
        server.done = []
        done, secs = serve_arrivals(server, frames, arrivals)
        stats = server.latency_stats()
        # The first pair of every size through the same server and lanes.
        acc_reqs = {sh: server.submit(*first_pair[sh]) for sh in first_pair}
        server.drain()
        res = {"pairs_per_s": len(done) / secs, "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"],
               "mean_ms": stats["mean_ms"], "requests": len(done), "form": form,
               "device_status": max(l.proc.status() for l in server.lanes.values()),
               "continuous_batching": {"max_batches_in_flight": server.max_in_flight,
                                       "overlapping_batch_pairs": server.overlapping_batches(),
                                       "held_for_memory": server.held_for_memory},
               "uv": {sh: (r.u, r.v) for sh, r in acc_reqs.items()}}
        server.close()
        return res

    served = {form: serve_form(form) for form in dict.fromkeys((args.dft, "tensor", "tensor_refined"))}
    # Plain per-pair path: each pair alone, in arrival order, on the FP32 FFT form.
    kw = dict(settings)
    mss = kw.pop("min_search_size")
    plain = {tuple(sh): PIVGPU(tuple(sh), mss, dft="fft", **kw) for sh in shapes}
    for sh in shapes:
        a, b = pool_by_shape[tuple(sh)][0]
        plain[tuple(sh)].run_batch(a[None], b[None], host_out=True)
    lat = []
    t0 = time.perf_counter()
    for t_arr, (a, b) in zip(arrivals, frames):
        while time.perf_counter() - t0 < t_arr:
            pass
        plain[a.shape].run_batch(a[None], b[None], host_out=True)
        lat.append(time.perf_counter() - t0 - t_arr)
    plain_secs = time.perf_counter() - t0
    lat = np.array(lat)
    for sh, job in acc_jobs.items():
        u64, v64, secs_o = job.get()
        for res in served.values():
            res.setdefault("rms_px_vs_fp64_oracle", {})[f"{sh[1]}x{sh[0]}"] = _rms(*res["uv"][sh], u64, v64)
    for res in served.values():
        res.pop("uv")
    chosen = served[args.dft]
    oracle_pool.close()
    line = {
        "metric": "serving pairs/s with p50/p99 latency (Poisson arrivals, 5 frame sizes, 64->32->16 px three-pass PIV)",
        "value": chosen["pairs_per_s"], "unit": "pairs/s", "n_gpus": 1, "higher_is_better": True,
        "p50_ms": chosen["p50_ms"], "p99_ms": chosen["p99_ms"], "mean_ms": chosen["mean_ms"],
        "requests": chosen["requests"], "arrival_rate": args.rate, "form": args.dft, "max_batch": 8,
        "slots_per_shape": 2,
        "forms": {form: {k: v for k, v in res.items() if k != "continuous_batching"} for form, res in served.items()},
        "plain_per_pair": {"pairs_per_s": args.requests / plain_secs, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                           "p99_ms": float(np.percentile(lat, 99) * 1e3), "form": "fft"},
        "config": {"workload": "Poisson stream, sizes uniform over " + ", ".join(f"{w}x{h}" for h, w in shapes) +
                   "; particle density U[0.01, 0.04], vortex or shear up to 12 px; 64->32->16 px @50%, median "
                   "validation, 2 revalidated spring replacements, smoothn GCV; float32",
                   "data": "synthetic (2 seeded pairs per size, reused)"},
        "device_status": chosen["device_status"],
        "accuracy": {"rms_px_vs_fp64_oracle": chosen["rms_px_vs_fp64_oracle"],
                     "case": "the first pair of every size, served by the same loop, against the float64 oracle"},
        "continuous_batching": chosen["continuous_batching"],
    }
    print(json.dumps(line), flush=True)


def run_mixed(args):
    """Batched form: 64 pairs, 16 each of 512x512, 1280x800, 1024x768 and
    2048x2048 (each with its own seeded vortex or shear field), in one
    submission: per-size plans on their own streams for the per-field stages,
    one correlation launch per pass over every size (tensor forms), captured as
    one CUDA graph, replayed K times (CUDA events). The plain FP32 FFT form of the same
    submission is timed beside it."""
    import multiprocessing as mp

    import torch

    sys.path.insert(0, PKG)
    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.batching import PIVMixedBatch

    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        pairs = pool.map(_make_mixed_pair, range(64))
    # Accuracy: the first pair of every size against the float64 oracle, on
    # the host cores while the GPU runs.
    first = {}
    for k, (a, _) in enumerate(pairs):
        first.setdefault(a.shape, k)
    oracle_pool = mp.get_context("spawn").Pool(len(first))
    acc_jobs = {sh: oracle_pool.apply_async(_oracle_case, ((4, k, None),)) for sh, k in first.items()}
    _build.build()
    torch.cuda.set_device(0)
    settings = dict(synthetic.CONFIGS[4]["piv"])
    shapes = [a.shape for a, _ in pairs]
    out = {}
    for form in dict.fromkeys((args.dft, "tensor", "tensor_refined", "fft")):
        batch = PIVMixedBatch(shapes, settings, dft=form)
        batch.load(pairs)
        batch.capture()
        for _ in range(args.warmup):
            batch.run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(batch.stream)
        for _ in range(args.steps):
            batch.run()
        e1.record(batch.stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        res = batch.results()
        out[form] = {"pairs_per_s": 64 / (ms * 1e-3), "ms_per_submission": ms,
                     "rms_px_vs_fp64_oracle": {f"{sh[1]}x{sh[0]}": (res[k], sh) for sh, k in first.items()},
                     "windows_per_s": batch.windows / (ms * 1e-3), "windows": batch.windows,
                     "device_status": batch.status(), "kernel_nodes": batch.kernel_nodes,
                     "schedule": batch.schedule, "schedule_ms": batch.schedule_ms}
        del batch
        torch.cuda.empty_cache()
    for sh, job in acc_jobs.items():
        u64, v64, _ = job.get()
        for form in out:
            acc = out[form]["rms_px_vs_fp64_oracle"]
            key = f"{sh[1]}x{sh[0]}"
            (gu, gv), _ = acc[key]
            acc[key] = _rms(gu, gv, u64, v64)
    oracle_pool.close()
    line = {
        "metric": "frame pairs/s of one mixed-size submission (64 pairs, 4 sizes, 64->32->16 px three-pass PIV)",
        "value": out[args.dft]["pairs_per_s"], "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "form": args.dft, "chosen": out[args.dft],
        "plain_form": out["fft"], "chosen_over_plain": out[args.dft]["pairs_per_s"] / out["fft"]["pairs_per_s"],
        "other_forms": {f: dict(r, over_plain=r["pairs_per_s"] / out["fft"]["pairs_per_s"])
                        for f, r in out.items() if f not in (args.dft, "fft")},
        "config": {"workload": "16 pairs each of 512x512, 1280x800, 1024x768, 2048x2048; density U[0.01, 0.05], "
                               "vortex or shear up to 10 px; 64->32->16 px @50%, median validation, 2 revalidated "
                               "spring replacements, smoothn GCV; float32",
                   "graph": "one CUDA graph per submission: per-size plans on their own streams for the "
                            "per-field stages; one correlation launch per pass over all four sizes (tensor forms)",
                   "data": "synthetic (seeded particle images)"},
    }
    print(json.dumps(line), flush=True)


def run_precision(args):
    """Precision form (the two-pass 2048x2048 workload at 75% overlap): 16
    resident pairs per step, each form captured as a CUDA graph and replayed
    K times (CUDA events): the hi/lo split and refined tensor forms (the
    faster one is the chosen precision form), the fp16 tensor form and the
    plain FP32 FFT form, every one autotuned first. Accuracy: RMS against
    the float64 oracle on 512x512 pairs of the same particle model, flow and
    settings (the oracle takes minutes on a full 2048x2048 pair)."""
    import ctypes as ct
    import multiprocessing as mp

    import numpy as np
    import torch

    sys.path.insert(0, PKG)
    acc_shape = (512, 512)
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        pairs = pool.map(_make_precision_pair, range(16))
        acc_cases = pool.map(_precision_oracle, [(k, acc_shape) for k in range(4)])
    # One full-size pair (pair 0 of the timed batch) against the float64
    # oracle, on a host core while the GPU runs.
    oracle_pool = mp.get_context("spawn").Pool(1)
    full_job = oracle_pool.apply_async(_oracle_case, ((3, 0, None),))
    import __graft_entry__

    __graft_entry__.build()
    from openpiv_gpu import _lib, synthetic
    from openpiv_gpu.gpu_process import PIVGPU

    lib = _lib.load()
    torch.cuda.set_device(0)
    kw = dict(synthetic.CONFIGS[3]["piv"])
    mss = kw.pop("min_search_size")
    fa = torch.as_tensor(np.stack([p[0] for p in pairs])).cuda()
    fb = torch.as_tensor(np.stack([p[1] for p in pairs])).cuda()
    B = fa.shape[0]
    shape = tuple(fa.shape[1:])
    stream = torch.cuda.Stream()
    out = {}
    for form in ("tensor_split", "tensor_refined", "tensor", "fft"):
        proc = PIVGPU(shape, mss, **kw, dft=form, autotune=True)
        with torch.cuda.stream(stream):
            for _ in range(max(1, args.warmup)):
                proc.run_batch(fa, fb)
        stream.synchronize()
        plan = proc.plan_handle(fa, B)
        m, n = proc.piv_fields[-1].field_shape
        u = torch.empty((B, m, n), dtype=torch.float64, device="cuda")
        v = torch.empty_like(u)
        val = torch.empty((B, m, n), dtype=torch.uint8, device="cuda")
        o = torch.empty_like(val)
        nk = ct.c_int(0)
        _lib.check(lib.piv_plan_graph_capture(plan, B, fa.data_ptr(), fb.data_ptr(), u.data_ptr(), v.data_ptr(),
                                              val.data_ptr(), o.data_ptr(), ct.byref(nk), stream.cuda_stream))
        for _ in range(args.warmup):
            _lib.check(lib.piv_plan_graph_launch(plan, stream.cuda_stream))
        sampler = ClockSampler(0)
        sampler.start()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            _lib.check(lib.piv_plan_graph_launch(plan, stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        clocks = sampler.stop()
        ms = e0.elapsed_time(e1) / args.steps
        windows = sum(f.n_wins for f in proc.piv_fields)
        full_uv = (u[0].cpu().numpy(), v[0].cpu().numpy())
        errs = []
        for a, b, u64, v64 in acc_cases:
            small = PIVGPU(acc_shape, mss, **kw, dft=form)
            gu, gv = small.run_batch(a[None], b[None], host_out=True)
            errs.append(float(np.mean((gu[0] - u64) ** 2 + (gv[0] - v64) ** 2)))
        out[form] = {"pairs_per_s": B / (ms * 1e-3), "ms_per_step": ms, "windows_per_s": B * windows / (ms * 1e-3),
                     "windows_per_pair": windows, "kernels_per_step": nk.value,
                     "rms_px_vs_fp64_oracle": float(np.sqrt(np.mean(errs))), "full_uv": full_uv,
                     "tuning": [t["name"] for t in proc.tuning()], "device_status": proc.status(), "clocks": clocks}
        del proc
        torch.cuda.empty_cache()
    u64, v64, oracle_s = full_job.get()
    oracle_pool.close()
    for form in out:
        gu, gv = out[form].pop("full_uv")
        out[form]["rms_px_vs_fp64_oracle_full_pair"] = _rms(gu, gv, u64, v64)
    # The chosen precision form: the faster of the two float32-accurate tensor forms.
    chosen_form = max(("tensor_split", "tensor_refined"), key=lambda f: out[f]["pairs_per_s"])
    chosen = out[chosen_form]
    line = {
        "metric": "frame pairs/s (2048x2048, 32->16 px two-pass PIV at 75% overlap, precision form) on 1 GB300",
        "value": chosen["pairs_per_s"], "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": chosen["ms_per_step"], "higher_is_better": True, "form": chosen_form,
        "dtype": DTYPE_OF_FORM[chosen_form], "data": "synthetic (seeded particle images)", "chosen": chosen,
        "forms": {f: out[f] for f in ("tensor_split", "tensor_refined") if f != chosen_form},
        "fp16_tensor_form": out["tensor"],
        "plain_form": out["fft"], "chosen_over_plain": chosen["pairs_per_s"] / out["fft"]["pairs_per_s"],
        "config": {"workload": "16 resident 2048x2048 uint8 pairs, 0.05 ppp, 8-mode streamfunction flow up to 8 px; "
                               "32 -> 16 px at 75%, n_fft 2, median validation, 2 revalidated spring replacements; "
                               "float32", "graph": True,
                   "accuracy_case": f"rms_px_vs_fp64_oracle: 4 pairs of {acc_shape[0]}x{acc_shape[1]} with the same "
                                    "particle model, flow and settings against the float64 oracle; "
                                    "rms_px_vs_fp64_oracle_full_pair: pair 0 of the timed batch (2048x2048) "
                                    f"against the float64 oracle ({oracle_s:.0f} s on one host core)",
                   "l2": "inputs larger than L2 (16 x 8 MiB frames + 32 MiB float frames per pair)"},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.precision:
        run_precision(args)
        return
    if args.mixed:
        run_mixed(args)
        return
    if args.serve:
        run_serve(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
