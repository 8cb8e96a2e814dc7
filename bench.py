"""Benchmark: forward + adjoint NFFT throughput on the 3-D radial ("koosh-ball")
workload, N = 256^3, 8192 spokes x 512 samples (M = 4,194,304 nodes), FP32,
Kaiser-Bessel window, m = 4, sigma = 2.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one forward NFFT (mul!(fHat, p, f)) plus one adjoint NFFT
(mul!(f, adjoint(p), fHat)) over the whole node set.  value = nodes/s over
the timed steps with inputs resident in HBM; e2e = the same through the
C-ABI calls with the inputs copied from pinned host memory and the results
copied back inside the timed region.  The inputs (1.07 GB oversampled grid,
134 MB image) are larger than L2, so no extra L2 flush is done.

--impl reference times the oracle, the CPU restatement of NFFT.jl's blocked
algorithm (FFT: scipy/pocketfft), on the host cores with all threads.
Under torchrun each rank runs an independent replica (the plan does not
shard); value is the aggregate over ranks.
"""
from __future__ import annotations

import argparse
import atexit
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "nfft.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "fwd+adj NFFT nodes/s @256^3 FP32 (<=1e-5 vs FP64 NDFT) vs plain path; HBM GB/s"
UNIT = "nodes/s"
N3 = (256, 256, 256)
SPOKES, SAMPLES = 8192, 512
M_NODES = SPOKES * SAMPLES
WORKLOAD = "3D radial koosh-ball NFFT fwd+adj, N=256^3, 8192 spokes x 512 samples (M=4194304), KB m=4 sigma=2"
# The workload's configuration, identical in both arms (the GPU arm's tile
# shape and the like go to the line's "run" object).
def config_dict(**kw):
    cfg = {"workload": WORKLOAD, "precision": "FP32", "precompute": "TENSOR",
           "window": "kaiser_bessel, m=4, sigma=2",
           "l2": "inputs larger than L2 (grid 1.07 GB, image 134 MB); no extra flush"}
    cfg.update(kw)
    return cfg
# DRAM bytes (read + write) per launch of the dominant kernel on this workload,
# from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum, one
# launch, tiles 16x8x8): 1.157 GB read + 0.578 GB write.  Not measured in the
# run itself; the line says so.
SPREAD_DRAM_BYTES = 1.735e9
SPREAD_TRAFFIC_SOURCE = ("ncu capture of spread_tile3_rec_kernel on this workload (one launch), "
                         "not measured in this run")
# DRAM bytes (read + write) of one Toeplitz application at 256^3 (the five
# kernels of the fused path), from an ncu capture of the profiling case:
# 2.821 GB read + 1.049 GB write.
TOEPLITZ_DRAM_BYTES = 3.870e9
SPREAD_LIMITER = ("shared-memory wavefronts: 110 per node (ncu, 128^3 case; 4.6e8 per launch = 1.47 ms at one "
                  "per clock per SM, ~91% of it reached) -- the read-modify-write of the padded tile in shared "
                  "memory (16 B per tap; 512 taps per node) bounds the kernel; HBM is not the limiter")


def radial_nodes(dtype=np.float32):
    """Spoke directions on a golden-angle (Fibonacci) spiral over the
    hemisphere, z_i = (i + 1/2)/8192, phi_i = i*pi*(3 - sqrt 5); samples at
    radius r_s = -1/2 + s/512, s = 0..511.  Returns k of shape (3, M)."""
    i = np.arange(SPOKES, dtype=np.float64)
    z = (i + 0.5) / SPOKES
    ph = i * math.pi * (3.0 - math.sqrt(5.0))
    rxy = np.sqrt(1.0 - z * z)
    u = np.stack([rxy * np.cos(ph), rxy * np.sin(ph), z])  # (3, spokes)
    r = -0.5 + np.arange(SAMPLES, dtype=np.float64) / SAMPLES
    k = (u[:, :, None] * r[None, None, :]).reshape(3, -1)
    return np.clip(k, -0.5, 0.5).astype(dtype)


def complex_normal(rng, shape, dtype=np.complex64):
    return ((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / math.sqrt(2)).astype(dtype)


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples (every 50 ms, with nvidia-smi's own
    timestamps).  Start it well before the timed region (nvidia-smi takes a
    moment to come up), bracket the timed region with mark_start() /
    mark_end(), and summary() keeps the samples taken inside it."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0, interval_ms=50):
        self.proc = None
        self.gpu_index = gpu_index
        self.interval_ms = interval_ms
        self.out = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def __enter__(self):
        return self.start()

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self._t.join(timeout=2)
            self.proc = None

    def __exit__(self, *a):
        self.stop()

    def summary(self):
        import datetime
        rows = []
        for line in self.out:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(parts[2]), float(parts[3]), parts[6:10]))
            except ValueError:
                continue
        if not rows:
            return None
        window = "timed region"
        if self.t0 is not None and self.t1 is not None:
            inside = [r for r in rows if self.t0 - 0.005 <= r[0] <= self.t1 + 0.005]
            if not inside:  # region shorter than the interval: the sample nearest to its middle
                mid = 0.5 * (self.t0 + self.t1)
                inside = [min(rows, key=lambda r: abs(r[0] - mid))]
                window = "nearest sample to the timed region"
            rows = inside
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for nm, val in zip(names, r[3]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(r[1] for r in rows), "sm_max_mhz": rows[-1][2],
                "reasons": sorted(reasons), "samples": len(rows), "window": window}


N_ERR_NODES = 4096  # random nodes of the forward error subset
N_ERR_FREQS = 4096  # random output frequencies of the adjoint error subset


def error_subsets(M, n_img, seed=7):
    """Random node indices (forward) and column-major output indices (adjoint)
    of the error measurement, sorted."""
    rng = np.random.default_rng(seed)
    return (np.sort(rng.choice(M, min(M, N_ERR_NODES), replace=False)),
            np.sort(rng.choice(n_img, min(n_img, N_ERR_FREQS), replace=False)))


def frequencies(N, lin):
    """Integer frequencies n - N div 2 (D x len(lin)) of column-major linear indices."""
    idx = np.unravel_index(np.asarray(lin), tuple(N), order="F")
    return np.stack([i - n // 2 for i, n in zip(idx, N)]).astype(np.float64)


def ndft_reference_subsets(k64, f, fhat, sub, lin, device="cuda"):
    """FP64 NDFT (src/direct.jl:99-151) of the inputs at the nodes `sub`
    (forward) and at the column-major output indices `lin` (adjoint), by this
    library's exact direct GPU sums: an NDFT plan of the node subset (forward),
    and the adjoint of an NNDFT plan from all nodes to the frequencies
    n - N div 2 (f[n] = sum_j fHat_j exp(2 pi i k_j . n)).  The tests check
    these sums against the oracle's NDFT on the same subsets."""
    import nfftgb300 as nf
    N = tuple(f.shape)
    pf = nf.NDFTPlan(np.ascontiguousarray(k64[:, sub]), N, device)
    ref_f = (pf * np.asarray(f, np.complex128)).cpu().numpy()
    pa = nf.NNDFTPlan(np.ascontiguousarray(k64), frequencies(N, lin), device)
    ref_a = (pa.adjoint() * np.asarray(fhat, np.complex128)).cpu().numpy()
    return ref_f, ref_a


def rel_l2(x, ref):
    x = np.asarray(x).astype(np.complex128).ravel()
    ref = np.asarray(ref).astype(np.complex128).ravel()
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


def rel_err_subset(k64, f, fhat, y, x, seed=7):
    """Relative l2 errors of the GPU outputs against the FP64 NDFT on 4096
    random nodes (forward) and 4096 random output frequencies (adjoint)."""
    sub, lin = error_subsets(k64.shape[1], int(np.prod(f.shape)), seed)
    ref_f, ref_a = ndft_reference_subsets(k64, f, fhat, sub, lin)
    return {"forward": rel_l2(y[sub], ref_f), "adjoint": rel_l2(x.ravel(order="F")[lin], ref_a),
            "nodes": int(len(sub)), "frequencies": int(len(lin)),
            "reference": "exact FP64 sums (NDFT of the node subset, NNDFT adjoint at the frequency subset) "
                         "on the GPU, checked against the oracle's NDFT in the tests"}


def max_over_ranks(t, world, device):
    """The slowest rank's time (replicas run independently; this is the only
    collective, outside the data path)."""
    if world <= 1:
        return float(t)
    import torch
    import torch.distributed as dist
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def aggregate_nodes_per_s(world, m_nodes, steps, t_max):
    """Whole-job throughput: every rank processes its own replica."""
    return world * m_nodes * steps / t_max


def cpu_reference_run(steps, warmup, budget_s=150.0):
    """The oracle (FP32) on the host cores: full forward + adjoint steps."""
    from oracle import oracle
    lib = oracle.lib()
    threads = lib.oracle_num_threads()
    k = radial_nodes(np.float32)
    rng = np.random.default_rng(123)
    f = complex_normal(rng, N3)
    fhat = complex_normal(rng, M_NODES)
    p = oracle.OraclePlan(k, N3, m=4, sigma=2.0, window="kaiser_bessel", precompute=oracle.TENSOR,
                          dtype=np.float32, fft_workers=threads)
    t_start = time.perf_counter()
    times = []
    done_w = 0
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        p.forward(f)
        p.adjoint(fhat)
        dt = time.perf_counter() - t0
        if it < warmup:
            done_w += 1
        else:
            times.append(dt)
        elapsed = time.perf_counter() - t_start
        if times and elapsed + dt > budget_s and len(times) >= 1:
            break
    per = statistics.median(times)
    return {"value": M_NODES / per, "seconds_per_step": per, "steps": len(times), "warmup": done_w,
            "cores": threads,
            "sample": f"full workload (M={M_NODES}, 256^3, FP32), {len(times)} timed fwd+adj pairs; "
                      f"oracle restatement of NFFT.jl blocked TENSOR, FFT via scipy.fft workers={threads}"}


def oracle_block_size():
    """The reference's _blockSize for the workload's oversampled grid."""
    from oracle import oracle
    return oracle.default_block_size(tuple(2 * n for n in N3))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    r = cpu_reference_run(args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": r["steps"], "warmup": r["warmup"], "ms_per_step": r["seconds_per_step"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict(),
        "run": {"parallelism": "host threads", "block_size": list(oracle_block_size())},
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
                         "sample": r["sample"]},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    import torch.distributed as dist
    import nfftgb300 as nf

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())

    clk = ClockSampler(local).start()  # up and sampling before the timed region
    atexit.register(clk.stop)          # never leave nvidia-smi running
    k = radial_nodes(np.float32)
    rng = np.random.default_rng(123)
    f_h = complex_normal(rng, N3)
    fhat_h = complex_normal(rng, M_NODES)

    # ---- FP32 tiled plan (the product path)
    stats = nf.TimingStats()
    t0 = time.perf_counter()
    pre = {"tensor": nf.TENSOR, "polynomial": nf.POLYNOMIAL, "full": nf.FULL, "linear": nf.LINEAR}[args.precompute]
    bs = tuple(int(v) for v in args.blocksize.split(",")) if args.blocksize else None
    p = nf.plan_nfft(k, N3, m=4, sigma=2.0, window="kaiser_bessel", precompute=pre, timing=stats, blockSize=bs)
    if args.autotune:
        p.autotune(use_cache=True)
    torch.cuda.synchronize()
    t_pre = time.perf_counter() - t0
    f = nf.as_colmajor(f_h, N3, torch.complex64, dev)
    fhat = torch.from_numpy(fhat_h).to(dev)
    y = torch.empty(M_NODES, dtype=torch.complex64, device=dev)
    x = nf.empty_image(N3, torch.complex64, dev)
    lib = nf.load()

    def step():
        p.forward_(y, f)
        p.adjoint_(x, fhat)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    lib.nfft_timing_reset(p._handle)
    launches0 = nf.kernel_launch_count()
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clk.mark_start()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk.mark_end()
    if world > 1:
        dist.barrier()
    clk.stop()
    launches = nf.kernel_launch_count() - launches0
    t_dev = max_over_ranks(ev0.elapsed_time(ev1) * 1e-3, world, dev)
    value = aggregate_nodes_per_s(world, M_NODES, args.steps, t_dev)

    import ctypes
    tot = (ctypes.c_double * 7)()
    calls = (ctypes.c_int64 * 2)()
    lib.nfft_get_timing_totals(p._handle, tot, calls)
    nf_ = max(calls[0], 1)
    na_ = max(calls[1], 1)
    stages = {"deconv_pad_ms": tot[3] / nf_ * 1e3, "fft_fwd_ms": tot[2] / nf_ * 1e3, "gather_ms": tot[1] / nf_ * 1e3,
              "spread_ms": tot[4] / na_ * 1e3, "fft_adj_ms": tot[5] / na_ * 1e3, "crop_ms": tot[6] / na_ * 1e3}

    # ---- e2e through the C-ABI with pinned host buffers.  Every step uploads
    # its inputs (f, fHat) from pinned host memory and downloads its outputs
    # (fHat, f); the copies run on their own streams with three device buffer
    # sets, so step i's transforms overlap the next steps' uploads and the
    # previous steps' downloads (events order each buffer's upload ->
    # transforms -> download).
    f_pin = torch.from_numpy(np.ascontiguousarray(f_h.ravel(order="F"))).pin_memory()
    fhat_pin = torch.from_numpy(fhat_h).pin_memory()
    y_pin = torch.empty(M_NODES, dtype=torch.complex64).pin_memory()
    x_pin = torch.empty(int(np.prod(N3)), dtype=torch.complex64).pin_memory()
    nbuf = 3
    f_flat_d = [torch.empty(int(np.prod(N3)), dtype=torch.complex64, device=dev) for _ in range(nbuf)]
    f_d = [t.reshape(N3[::-1]).permute(2, 1, 0) for t in f_flat_d]
    fhat_d = [torch.empty(M_NODES, dtype=torch.complex64, device=dev) for _ in range(nbuf)]
    y_d = [torch.empty(M_NODES, dtype=torch.complex64, device=dev) for _ in range(nbuf)]
    x_d = [nf.empty_image(N3, torch.complex64, dev) for _ in range(nbuf)]
    x_flat_d = [t.permute(2, 1, 0).reshape(-1) for t in x_d]
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev_in = [torch.cuda.Event() for _ in range(nbuf)]
    ev_done = [torch.cuda.Event() for _ in range(nbuf)]
    ev_out = [torch.cuda.Event() for _ in range(nbuf)]

    def e2e_step(i):
        b = i % nbuf
        with torch.cuda.stream(s_in):
            s_in.wait_event(ev_done[b])          # the transforms of step i - nbuf have read buffer b
            f_flat_d[b].copy_(f_pin, non_blocking=True)
            fhat_d[b].copy_(fhat_pin, non_blocking=True)
            ev_in[b].record(s_in)
        stream.wait_event(ev_in[b])
        stream.wait_event(ev_out[b])             # the outputs of step i - nbuf have been downloaded
        p.forward_(y_d[b], f_d[b])
        p.adjoint_(x_d[b], fhat_d[b])
        ev_done[b].record(stream)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ev_done[b])
            y_pin.copy_(y_d[b], non_blocking=True)
            x_pin.copy_(x_flat_d[b], non_blocking=True)
            ev_out[b].record(s_out)

    for i in range(max(nbuf, args.warmup)):
        e2e_step(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_steps = max(3, args.steps)
    if world > 1:
        dist.barrier()
    e0.record(stream)
    s_in.wait_event(e0)
    for i in range(e2e_steps):
        e2e_step(i)
    for b in range(nbuf):
        stream.wait_event(ev_out[b])
    e1.record(stream)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(e0.elapsed_time(e1) * 1e-3, world, dev)
    e2e_value = aggregate_nodes_per_s(world, M_NODES, e2e_steps, t_e2e)
    h2d = f_pin.numel() * 8 + fhat_pin.numel() * 8
    d2h = y_pin.numel() * 8 + x_pin.numel() * 8

    # ---- accuracy of this run's outputs (outside the timed region)
    err = None
    if rank == 0 and not args.no_check:
        p.forward_(y, f)
        p.adjoint_(x, fhat)
        err = rel_err_subset(k.astype(np.float64), f_h.astype(np.complex128), fhat_h.astype(np.complex128),
                             y.cpu().numpy(), x.cpu().numpy())

    # ---- the plain FP64 path on the same workload (comparator)
    plain = None
    if not args.no_plain:
        k64 = k.astype(np.float64)
        pp = nf.plan_nfft(k64, N3, m=4, sigma=2.0, window="kaiser_bessel", precompute=nf.POLYNOMIAL,
                          blocking=False)
        f64 = f.to(torch.complex128)
        fhat64 = fhat.to(torch.complex128)
        y64 = torch.empty(M_NODES, dtype=torch.complex128, device=dev)
        x64 = nf.empty_image(N3, torch.complex128, dev)
        pp.forward_(y64, f64)
        pp.adjoint_(x64, fhat64)
        torch.cuda.synchronize()
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nplain = 3
        q0.record(stream)
        for _ in range(nplain):
            pp.forward_(y64, f64)
            pp.adjoint_(x64, fhat64)
        q1.record(stream)
        torch.cuda.synchronize()
        t_plain = q0.elapsed_time(q1) * 1e-3
        plain = {"value": M_NODES * nplain / t_plain, "unit": UNIT, "ms_per_step": t_plain / nplain * 1e3,
                 "speedup_of_value": value / world / (M_NODES * nplain / t_plain)}
        del pp, f64, fhat64, y64, x64
        torch.cuda.empty_cache()

    # ---- roofline of the dominant kernel of this library
    peak, peak_kind = measured_peak_hbm()
    s_r, s_c, D = 4, 8, 3
    ng = int(np.prod([2 * n for n in N3]))
    nimg = int(np.prod(N3))
    alg = {
        "spread_ms": M_NODES * (D * s_r + s_c) + ng * s_c,
        "gather_ms": ng * s_c + M_NODES * (D * s_r + s_c),
        # fused x-line kernels: the image and the image rows of the grid (2 N0 x N1 x N2)
        "deconv_pad_ms": nimg * s_c + 2 * nimg * s_c,
        "crop_ms": 2 * nimg * s_c + nimg * s_c,
    }
    dom = max(alg, key=lambda s: stages[s])
    t_dom = stages[dom] * 1e-3
    achieved = alg[dom] / t_dom / 1e9
    kernel_names = {"spread_ms": "spread_tile3_rec_kernel (stage: the kernel alone; its grid was zeroed on a side "
                                 "stream beside the previous gather)",
                    "gather_ms": "interp_tile3_kernel", "deconv_pad_ms": "fft4_x_kernel (forward)",
                    "crop_ms": "fft4_x_kernel (adjoint)"}
    roofline = {"bound": "hbm", "kernel": kernel_names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                "algorithmic_bytes": alg[dom],
                "traffic": SPREAD_DRAM_BYTES if dom == "spread_ms" else None,
                "traffic_source": SPREAD_TRAFFIC_SOURCE if dom == "spread_ms" else None,
                "limiter": SPREAD_LIMITER if dom == "spread_ms" else None}
    pair_bytes = 7 * ng * s_c + 3 * nimg * s_c + 2 * M_NODES * (D * s_r + s_c)
    pair_gbs = pair_bytes / (t_dev / args.steps) / 1e9

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_reference_run(steps=1, warmup=0, budget_s=60.0)
        cpu = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port", "sample": r["sample"]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(precompute=args.precompute.upper()),
            "run": {"block_size": list(p.params.blockSize),
                    "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                    "precision_detail": "FP32 data and sums; FP64 node reduction and deconvolution factors",
                    "plan_seconds": t_pre},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps,
                    "copies": "pinned host <-> device every step on two copy streams, three buffer sets, "
                              "overlapping the neighbouring steps' transforms"},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "pair_hbm_gbs": pair_gbs,
            "stages_ms": stages,
            "rel_err_vs_fp64_ndft": err,
            "plain_fp64_path": plain,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


class SparseBPath:
    """The reference's GPU algorithm restated on this GPU with library calls
    (ext/NFFTGPUArraysExt/implementation.jl:21-136): the |Ntilde| x M sparse
    matrix B of exact window values built once (FULL precompute,
    src/precomputation.jl:81-120, Int32 indices), forward = deconvolve into the
    zero-padded grid + FFT + B^T g, adjoint = B fHat + backward FFT + crop.
    B is a torch CSR matrix (cuSPARSE SpMM on [re, im] columns), the FFT is
    torch.fft (cuFFT), the deconvolution factors are the plan's own.  It is
    the plain-path comparator where B fits (nnz < 2^31)."""

    def __init__(self, k, N, m, sigma, inv, real_dtype, device):
        import warnings
        import torch
        warnings.filterwarnings("ignore", message="Sparse CSR tensor support is in beta")
        self.torch = torch
        D = len(N)
        Nt = tuple(2 * (int(np.ceil(sigma * n)) // 2) for n in N)
        self.N, self.Nt = tuple(N), Nt
        ng = int(np.prod(Nt))
        kk = torch.as_tensor(np.asarray(k, np.float64), device=device)
        M = kk.shape[1]
        L = 2 * m
        b = math.pi * (2.0 - 1.0 / sigma)
        idx = torch.zeros((M, 1), dtype=torch.int64, device=device)
        w = torch.ones((M, 1), dtype=torch.float64, device=device)
        stride = 1
        for d in range(D):
            xs = kk[d] * Nt[d]
            c = torch.floor(xs)
            t = c[:, None] - m + 1 + torch.arange(L, device=device, dtype=torch.float64)[None, :]
            x = (xs[:, None] - t).abs()
            r = torch.sqrt(torch.clamp(m * m - x * x, min=0.0))
            wd = torch.where(x < m, torch.sinh(b * r) / (math.pi * torch.where(r > 0, r, torch.ones_like(r))),
                             torch.zeros_like(x))
            wd = torch.where(x == m, torch.full_like(x, b / math.pi), wd)
            id_d = torch.remainder(t.to(torch.int64), Nt[d]) * stride
            idx = (idx[:, :, None] + id_d[:, None, :]).reshape(M, -1)
            w = (w[:, :, None] * wd[:, None, :]).reshape(M, -1)
            stride *= Nt[d]
        T = idx.shape[1]
        rows = torch.arange(M, device=device, dtype=torch.int64).repeat_interleave(T)
        vals = w.reshape(-1).to(real_dtype)
        with torch.sparse.check_sparse_tensor_invariants(True):
            self.BT = torch.sparse_coo_tensor(torch.stack([rows, idx.reshape(-1)]), vals, (M, ng)).coalesce() \
                .to_sparse_csr()
            self.B = torch.sparse_coo_tensor(torch.stack([idx.reshape(-1), rows]), vals, (ng, M)).coalesce() \
                .to_sparse_csr()
        del idx, w, rows, vals
        # image -> grid index and separable deconvolution factor (column-major)
        gidx = torch.zeros(1, dtype=torch.int64, device=device)
        fac = torch.ones(1, dtype=torch.float64, device=device)
        gstride = 1
        off = 0
        for d in range(D):
            n = torch.arange(N[d], device=device)
            gd = torch.remainder(n - N[d] // 2, Nt[d]) * gstride
            fd = torch.as_tensor(np.asarray(inv[off:off + N[d]], np.float64), device=device)
            gidx = (gidx[None, :] + gd[:, None]).reshape(-1)
            fac = (fac[None, :] * fd[:, None]).reshape(-1)
            gstride *= Nt[d]
            off += N[d]
        self.gidx = gidx
        self.fac = fac.to(real_dtype)
        self.cdtype = torch.complex64 if real_dtype == torch.float32 else torch.complex128
        self.ng = ng

    def forward(self, f_flat):
        torch = self.torch
        g = torch.zeros(self.ng, dtype=self.cdtype, device=f_flat.device)
        g[self.gidx] = f_flat * self.fac
        G = torch.fft.fftn(g.view(self.Nt[::-1])).reshape(-1)
        return torch.view_as_complex((self.BT @ torch.view_as_real(G)).contiguous())

    def adjoint(self, fhat):
        torch = self.torch
        g = torch.view_as_complex((self.B @ torch.view_as_real(fhat)).contiguous())
        G = torch.fft.ifftn(g.view(self.Nt[::-1]), norm="forward").reshape(-1)
        return G[self.gidx] * self.fac


def spiral_nodes(N, interleaves=32, samples=2048, turns=4.0):
    """Archimedean spiral: r = 0.5 t, theta = 2 pi turns t + 2 pi i / interleaves."""
    t = np.arange(samples) / samples
    out = []
    for i in range(interleaves):
        th = 2 * np.pi * turns * t + 2 * np.pi * i / interleaves
        out.append(np.stack([0.5 * t * np.cos(th), 0.5 * t * np.sin(th)]))
    return np.clip(np.concatenate(out, axis=1), -0.5, 0.4999999)


CONFIGS = {
    "plain2d": dict(N=(128, 128), M=16384, m=4, prec=64, nodes="uniform", compensated=False,
                    desc="2-D plain NFFT fwd+adj, N=128^2, M=16384 uniform, KB m=4 sigma=2, TENSOR, FP64"),
    "line1d": dict(N=(1 << 22,), M=1 << 24, m=5, prec=32, nodes="uniform", compensated=True,
                   desc="1-D NFFT fwd+adj, N=2^22, M=2^24 uniform, KB m=5 sigma=2, TENSOR, FP32, compensated"),
    "spiral2d": dict(N=(256, 256), M=65536, m=4, prec=32, nodes="spiral", compensated=False,
                     desc="2-D spiral (32 x 2048) fwd+adj+node gradient, N=256^2, KB m=4 sigma=2, FP32"),
    "radial3d_fp64": dict(N=(256, 256, 256), M=8192 * 512, m=4, prec=64, nodes="radial", compensated=False,
                          desc="3D radial koosh-ball NFFT fwd+adj, N=256^3, 8192 spokes x 512 samples, KB m=4 "
                               "sigma=2, TENSOR, FP64"),
}


def run_config(args):
    """--workload plain2d | line1d | spiral2d: the other configurations,
    measured as extra lines (ours, the sparse-B GPU comparator where B fits,
    the oracle on the host cores)."""
    import torch
    import nfftgb300 as nf
    cfg = CONFIGS[args.workload]
    dev = torch.device("cuda", torch.cuda.current_device())
    N, M, m = cfg["N"], cfg["M"], cfg["m"]
    rdt = np.float32 if cfg["prec"] == 32 else np.float64
    cd = torch.complex64 if cfg["prec"] == 32 else torch.complex128
    rng = np.random.default_rng(123)
    if cfg["nodes"] == "spiral":
        k = spiral_nodes(N[0])
    elif cfg["nodes"] == "radial":
        k = radial_nodes(np.float64)
    else:
        k = rng.random((len(N), M)) - 0.5
    k = k.astype(rdt)
    M = k.shape[1]
    f_h = complex_normal(rng, N, np.complex128)
    fh_h = complex_normal(rng, M, np.complex128)
    p = nf.plan_nfft(k, N, m=m, sigma=2.0, precompute=nf.TENSOR, compensated=cfg["compensated"])
    if args.autotune:
        p.autotune(use_cache=True)
    f = nf.as_colmajor(f_h, N, cd, dev)
    fh = torch.as_tensor(fh_h).to(device=dev, dtype=cd)
    y = torch.empty(M, dtype=cd, device=dev)
    x = nf.empty_image(N, cd, dev)
    grad = args.workload == "spiral2d"
    dk = torch.empty((M, len(N)), dtype=p.dtype, device=dev).t() if grad else None

    def step():
        p.forward_(y, f)
        p.adjoint_(x, fh)
        if grad:
            p.grad_nodes_(dk, f, fh)

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / steps

    l0 = nf.kernel_launch_count()
    t_ours = timed(step, args.steps, args.warmup)
    launches = (nf.kernel_launch_count() - l0) // (args.steps + args.warmup)
    rebin = None
    if grad:
        # a node-optimisation step moves the nodes: nodes! (check, binning,
        # window tensor, tasks) precedes fwd + adj + dk every step, as
        # nfftgb300.autodiff.nfft_nodes does on every call
        kd = torch.as_tensor(k).to(dev)

        def step_rebin():
            p.nodes_(kd)
            step()

        t_rb = timed(step_rebin, args.steps, args.warmup)
        rebin = {"value": M / t_rb, "unit": UNIT, "ms_per_step": t_rb * 1e3,
                 "nodes_ms": (t_rb - t_ours) * 1e3,
                 "what": "each step re-bins the nodes (nodes!) before fwd + adj + dk, as a node-optimisation "
                         "step does"}
    yo, xo = y.cpu().numpy(), x.cpu().numpy()
    k64 = k.astype(np.float64)
    err = rel_err_subset(k64, f_h, fh_h, yo, xo)
    line = {"metric": f"{args.workload}: fwd+adj{'+dk' if grad else ''} NFFT nodes/s", "value": M / t_ours,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_ours * 1e3, "higher_is_better": True, "dtype": "f32" if cfg["prec"] == 32 else "f64",
            "data": "synthetic", "config": {"workload": cfg["desc"], "block_size": list(p.params.blockSize)},
            "gpu_launches_per_step": launches, "rel_err_vs_fp64_ndft": err}
    if rebin is not None:
        line["with_rebinning"] = rebin
    # the reference's GPU algorithm (sparse B), where it fits
    if not args.no_plain and M * (2 * m) ** len(N) < 2 ** 31:
        inv = np.concatenate([p.deconv_factors()[d] for d in range(len(N))])
        sb = SparseBPath(k, N, m, 2.0, inv, p.dtype, dev)
        f_flat = f.permute(*reversed(range(len(N)))).reshape(-1).contiguous()
        t_sb = timed(lambda: (sb.forward(f_flat), sb.adjoint(fh)), args.steps, args.warmup)
        ys = sb.forward(f_flat).cpu().numpy()
        line["sparse_b_gpu"] = {"value": M / t_sb, "unit": UNIT, "ms_per_step": t_sb * 1e3,
                                "speedup_of_value": t_sb / t_ours, "nnz": int(sb.BT._nnz()),
                                "rel_diff_forward_vs_ours": rel_l2(ys, yo),
                                "what": "reference GPU algorithm restated: FULL sparse B (cuSPARSE SpMM via torch) + "
                                        "cuFFT (torch.fft) + deconvolution; fwd+adj only"}
        del sb
        torch.cuda.empty_cache()
    if not args.no_cpu_baseline:
        from oracle import oracle
        lib = oracle.lib()
        threads = lib.oracle_num_threads()
        op = oracle.OraclePlan(k, N, m=m, sigma=2.0, precompute=oracle.TENSOR, dtype=rdt, fft_workers=threads)
        fr, fhr = f_h.astype(np.complex128 if rdt == np.float64 else np.complex64), fh_h.astype(
            np.complex128 if rdt == np.float64 else np.complex64)
        times = []
        t_start = time.perf_counter()
        while len(times) < 5 and time.perf_counter() - t_start < 60:
            t0 = time.perf_counter()
            op.forward(fr)
            op.adjoint(fhr)
            times.append(time.perf_counter() - t0)
        per = statistics.median(times)
        line["cpu_baseline"] = {"value": M / per, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"full workload, {len(times)} fwd+adj pairs (no dk); oracle restatement "
                                          f"of NFFT.jl blocked TENSOR, scipy.fft workers={threads}"}
    print(json.dumps(line), flush=True)
    return 0


def batched_plans(seed=4, nplans=64):
    """64 2-D FP32 plans: N_i from {64, 96, 128, 192, 256, 384, 512} (grids of
    2 N_i, radix-3 sizes included), M_i = floor(10^U(4, 6)), nodes U[-1/2, 1/2)^2."""
    rng = np.random.default_rng(seed)
    sizes = [64, 96, 128, 192, 256, 384, 512]
    out = []
    for _ in range(nplans):
        n = int(rng.choice(sizes))
        M = int(10 ** rng.uniform(4, 6))
        out.append(((rng.random((2, M)) - 0.5).astype(np.float32), (n, n)))
    return out


def run_batched(args):
    """--workload batched2d: the 64 batched 2-D plans, one graph-replayed
    batch call per direction against a loop of single-plan calls."""
    import torch
    import nfftgb300 as nf
    dev = torch.device("cuda", torch.cuda.current_device())
    probs = batched_plans()
    plans = [nf.plan_nfft(k, N, m=4, sigma=2.0, precompute=nf.TENSOR) for k, N in probs]
    if args.autotune:
        for p in plans:
            p.autotune(use_cache=True)
    batch = nf.NFFTBatch(plans)
    rng = np.random.default_rng(5)
    fs = [nf.as_colmajor(complex_normal(rng, N), N, torch.complex64, dev) for _, N in probs]
    vs = [torch.from_numpy(complex_normal(rng, k.shape[1])).to(dev) for k, _ in probs]
    ys = [torch.empty(k.shape[1], dtype=torch.complex64, device=dev) for k, _ in probs]
    xs = [nf.empty_image(N, torch.complex64, dev) for _, N in probs]
    total_m = sum(k.shape[1] for k, _ in probs)

    def step_batch():
        batch.forward_(ys, fs)
        batch.adjoint_(xs, vs)

    def step_loop():
        for p, y, f in zip(plans, ys, fs):
            p.forward_(y, f)
        for p, x, v in zip(plans, xs, vs):
            p.adjoint_(x, v)

    out = {}
    stream = torch.cuda.current_stream(dev)
    for name, step in (("batch", step_batch), ("loop", step_loop)):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        l0 = nf.kernel_launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        t = ev0.elapsed_time(ev1) * 1e-3
        out[name] = {"value": total_m * args.steps / t, "ms_per_step": t / args.steps * 1e3,
                     "host_launch_calls": nf.kernel_launch_count() - l0}
    print(json.dumps({
        "metric": "batched 2-D fwd+adj NFFT nodes/s (64 plans, FP32)", "value": out["batch"]["value"],
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": out["batch"]["ms_per_step"], "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "64 plans, N_i in {64..512}^2, M_i = floor(10^U(4,6)), KB m=4 sigma=2, TENSOR",
                   "total_nodes": total_m, "grid_sizes": sorted({2 * N[0] for _, N in probs})},
        "loop_of_single_plans": out["loop"],
        "note": "batch launches are captured once per direction into a CUDA graph; host_launch_calls counts "
                "launches issued from the host (0 for graph replays)"}))
    return 0


def run_toeplitz(args):
    """--workload toeplitz3d: the Gram operator A^H A of the radial 256^3 plan
    applied as a Toeplitz convolution (NFFTTools' convolveToeplitzKernel!) on
    the 512^3 grid -- the fused pruned-FFT path against the cuFFT sequence of
    the reference (pad, FFT, product, IFFT, crop) and against the forward +
    adjoint NFFT pair it replaces.  The kernel lambda comes from
    calculateToeplitzKernel (adjoint NFFT of ones on a 512^3 plan); the timed
    loop applies lambda / max|lambda| so repeated applications stay finite
    (same work)."""
    import torch
    import nfftgb300 as nf
    from nfftgb300 import tools
    dev = torch.device("cuda", torch.cuda.current_device())
    N = (256, 256, 256)
    k = radial_nodes(np.float32)
    M = k.shape[1]
    t0 = time.perf_counter()
    tz = tools.Toeplitz(N, torch.complex64, dev)
    if args.small:
        # profiling case: the same 256^3 application with a seeded random
        # kernel (no 512^3 plan, no comparison arms; ~3.5 GB on the device)
        g = torch.Generator(device=dev).manual_seed(1)
        lam = tz.empty_kernel()
        lam.copy_(torch.randn(lam.shape, dtype=torch.complex64, device=dev, generator=g))
    else:
        lam = tools.calculate_toeplitz_kernel(N, k, m=4, sigma=2.0, toeplitz=tz, precompute=nf.TENSOR)
    torch.cuda.synchronize()
    t_kernel = time.perf_counter() - t0
    torch.cuda.empty_cache()
    lam_t = lam / lam.abs().max()
    if args.small:
        del lam
        x = nf.empty_image(N, torch.complex64, dev)
        x.copy_(torch.randn(N, dtype=torch.complex64, device=dev))
        y = x.clone()
        for _ in range(args.warmup + args.steps):
            tz.convolve_(y, lam_t)
        torch.cuda.synchronize()
        print(json.dumps({"workload": "toeplitz3d profiling case (random kernel)", "applications":
                          args.warmup + args.steps}))
        return 0
    ref = tools.Toeplitz(N, torch.complex64, dev, fft="cufft")
    rng = np.random.default_rng(3)
    x_h = complex_normal(rng, N)
    x = nf.as_colmajor(x_h, N, torch.complex64, dev)
    y = x.clone()
    y2 = x.clone()
    p = nf.plan_nfft(k, N, m=4, sigma=2.0, precompute=nf.TENSOR)
    if args.autotune:
        p.autotune(use_cache=True)
    fh = torch.empty(M, dtype=torch.complex64, device=dev)
    xa = nf.empty_image(N, torch.complex64, dev)
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        l0 = nf.kernel_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / args.steps, (nf.kernel_launch_count() - l0) // args.steps

    with ClockSampler(torch.cuda.current_device()) as clk:
        time.sleep(0.3)  # nvidia-smi up and sampling before the timed region
        for _ in range(args.warmup):
            tz.convolve_(y, lam_t)
        torch.cuda.synchronize()
        clk.mark_start()
        t_fused, launches = timed(lambda: tz.convolve_(y, lam_t))
        clk.mark_end()
    t_cufft, _ = timed(lambda: ref.convolve_(y2, lam_t))
    t_pair, _ = timed(lambda: (p.forward_(fh, x), p.adjoint_(xa, fh)))
    # one application of the true kernel against A^H A through the NFFT pair
    y.copy_(x)
    tz.convolve_(y, lam)
    p.forward_(fh, x)
    p.adjoint_(xa, fh)
    y2.copy_(x)
    ref.convolve_(y2, lam)
    torch.cuda.synchronize()
    d_pair = float((y - xa).abs().double().norm() / xa.abs().double().norm())
    d_cufft = float((y - y2).abs().double().norm() / y2.abs().double().norm())
    n_img = float(np.prod(N))
    sc = 8.0
    design_bytes = 34 * n_img * sc      # pruned passes: x 3, y 6, fused z 16 (incl. lambda 8), y' 6, x' 3
    compulsory = 10 * n_img * sc        # y in, lambda, y out
    peak, peak_src = measured_peak_hbm()
    achieved = design_bytes / t_fused / 1e9
    line = {
        "metric": "toeplitz3d: A^H A applications/s (Toeplitz convolution, 256^3 image, 512^3 kernel, FP32)",
        "value": 1.0 / t_fused, "unit": "applications/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_fused * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "Toeplitz Gram operator of the 3-D radial plan: N=256^3, kernel of 8192 spokes x 512 "
                               "samples (M=4194304) on 512^3, KB m=4 sigma=2",
                   "l2": "kernel 1.07 GB and grid 1.07 GB exceed L2; no extra flush",
                   "kernel_seconds": t_kernel},
        "gpu_launches_per_step": launches,
        "equivalent_nodes_per_s": M / t_fused,
        "roofline": {"bound": "hbm", "kernels": "fft4_x_kernel, fft4_lines_kernel, fft4_toeplitz_kernel, "
                                                "fft4_lines_kernel, fft4_x_kernel (whole application)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src, "algorithmic_bytes": design_bytes,
                     "compulsory_bytes": compulsory, "traffic": TOEPLITZ_DRAM_BYTES},
        "cufft_sequence": {"ms_per_step": t_cufft * 1e3, "speedup_of_value": t_cufft / t_fused,
                           "rel_diff_vs_fused": d_cufft,
                           "what": "the reference's sequence on the GPU: zero-fill + corner copy, cuFFT, "
                                   "product, cuFFT back, crop"},
        "nfft_pair": {"ms_per_step": t_pair * 1e3, "speedup_of_value": t_pair / t_fused,
                      "rel_diff_vs_toeplitz": d_pair,
                      "what": "forward + adjoint NFFT of the same plan (A^H A without the kernel)"},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        from oracle import oracle
        threads = oracle.lib().oracle_num_threads()
        lam_h = lam_t.cpu().numpy()
        times = []
        t_start = time.perf_counter()
        while len(times) < 2 and time.perf_counter() - t_start < 40:
            ta = time.perf_counter()
            oracle.convolve_toeplitz(x_h, lam_h, dtype=np.complex64, workers=threads)
            times.append(time.perf_counter() - ta)
        per = statistics.median(times)
        line["cpu_baseline"] = {"value": 1.0 / per, "unit": "applications/s", "cores": threads, "kind": "port",
                                "sample": f"full workload, {len(times)} applications; oracle restatement of "
                                          f"convolveToeplitzKernel!, scipy.fft workers={threads}, FP32"}
    print(json.dumps(line), flush=True)
    return 0


def run_extras(args):
    """--workload extras: one JSON line per widened row, each measured on the
    device with CUDA events (W warm-up, K timed steps):
      windows x precompute modes of the 256^3 radial plan (fwd+adj, rel. error
      vs the FP64 NDFT on node / frequency subsets);
      a directional plan: 2-D NFFTs (dims 1:2) of the 64 slices of a
      256 x 256 x 64 stack, 2-D radial nodes (256 spokes x 512 samples),
      against 64 single 2-D plans;
      a directional plan whose transform dims follow a column index (dims 2:3
      of a 64 x 256 x 256 stack, same nodes), tiled path against the atomic
      per-(column, node) path;
      3-D NFCT and NFST plans, N = 64^3, 2^20 nodes in [0, 1/2)^3 (fwd +
      transpose, error vs the direct GPU sums on 64 nodes);
      NFFTTools' sdc (20 iterations) on the 2-D spiral (config 5's nodes)."""
    import torch
    import nfftgb300 as nf
    from nfftgb300 import tools
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / args.steps

    def emit(metric, value, unit, ms, config, **extra):
        line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "data": "synthetic",
                "config": config}
        line.update(extra)
        print(json.dumps(line), flush=True)

    # ---- windows x precompute modes, 256^3 radial, FP32
    k = radial_nodes(np.float32)
    M = k.shape[1]
    rng = np.random.default_rng(123)
    f_h = complex_normal(rng, N3, np.complex128)
    fh_h = complex_normal(rng, M, np.complex128)
    f = nf.as_colmajor(f_h, N3, torch.complex64, dev)
    fh = torch.as_tensor(fh_h).to(device=dev, dtype=torch.complex64)
    y = torch.empty(M, dtype=torch.complex64, device=dev)
    x = nf.empty_image(N3, torch.complex64, dev)
    k64 = k.astype(np.float64)
    sub, lin = error_subsets(M, int(np.prod(N3)))
    ref_f, ref_a = ndft_reference_subsets(k64, f_h, fh_h, sub, lin)
    table = {}
    for window in ("kaiser_bessel", "gauss", "spline", "kaiser_bessel_rev", "cosh_type"):
        for pre in ("TENSOR", "POLYNOMIAL", "LINEAR", "FULL"):
            p = nf.plan_nfft(k, N3, m=4, sigma=2.0, window=window, precompute=getattr(nf, pre), blockSize=(16, 8, 8))
            t = timed(lambda: (p.forward_(y, f), p.adjoint_(x, fh)))
            yo = y.cpu().numpy()
            xo = x.cpu().numpy().ravel(order="F")
            table[f"{window}/{pre}"] = {"nodes_per_s": M / t, "ms": t * 1e3,
                                        "err_fwd": rel_l2(yo[sub], ref_f), "err_adj": rel_l2(xo[lin], ref_a)}
            del p
            torch.cuda.empty_cache()
    base = table["kaiser_bessel/TENSOR"]
    emit("windows x precompute: fwd+adj NFFT nodes/s @256^3 radial FP32 m=4 (kaiser_bessel/TENSOR as value)",
         base["nodes_per_s"], UNIT, base["ms"],
         {"workload": WORKLOAD, "block_size": [16, 8, 8], "grid": "each plan's own"}, dtype="f32", table=table)
    del f, fh, y, x
    torch.cuda.empty_cache()

    # ---- directional: 2-D NFFTs of the slices of a 256 x 256 x 64 stack
    nsp, nsa = 256, 512
    ang = np.arange(nsp) * np.pi * (3.0 - math.sqrt(5.0))
    r = -0.5 + np.arange(nsa) / nsa
    k2 = np.stack([np.outer(np.cos(ang), r).ravel(), np.outer(np.sin(ang), r).ravel()]).astype(np.float32)
    J = k2.shape[1]
    Nd = (256, 256, 64)
    pd = nf.plan_nfft(k2, Nd, dims=(1, 2), m=4, sigma=2.0)
    fd = nf.as_colmajor(complex_normal(rng, Nd), Nd, torch.complex64, dev)
    vd = nf.as_colmajor(complex_normal(rng, pd.NOut), pd.NOut, torch.complex64, dev)
    yd = nf.empty_image(pd.NOut, torch.complex64, dev)
    xd = nf.empty_image(Nd, torch.complex64, dev)
    t_dir = timed(lambda: (pd.forward_(yd, fd), pd.adjoint_(xd, vd)))
    yd_h = yd.cpu().numpy()
    ps = nf.plan_nfft(k2, (256, 256), m=4, sigma=2.0, precompute=nf.TENSOR)
    ys = torch.empty(J, dtype=torch.complex64, device=dev)
    xs = nf.empty_image((256, 256), torch.complex64, dev)
    fsl = [fd[:, :, z].clone() for z in range(Nd[2])]
    vsl = [vd[:, z].contiguous() for z in range(Nd[2])]

    def loop():
        for z in range(Nd[2]):
            ps.forward_(ys, fsl[z])
            ps.adjoint_(xs, vsl[z])
    t_loop = timed(loop)
    ps.forward_(ys, fsl[5])
    d5 = rel_l2(yd_h[:, 5], ys.cpu().numpy())
    emit("directional 2-D NFFT (dims 1:2) of a 256x256x64 stack: fwd+adj node values/s", J * Nd[2] / t_dir,
         "node values/s", t_dir * 1e3,
         {"workload": "N=(256,256,64), dims=1:2, 2-D golden-angle radial 256 spokes x 512 samples (J=131072), "
                      "KB m=4 sigma=2, LINEAR (as the reference's directional plan)"},
         dtype="f32", loop_of_64_single_2d_plans={"ms_per_step": t_loop * 1e3, "speedup_of_value": t_loop / t_dir},
         rel_diff_slice5_vs_single_plan=d5)
    del pd, ps, fd, vd, yd, xd, fsl, vsl
    torch.cuda.empty_cache()

    # ---- directional, transform dims after a column index: dims 2:3 of a 64 x 256 x 256 stack
    Nq = (64, 256, 256)
    fq = nf.as_colmajor(complex_normal(rng, Nq), Nq, torch.complex64, dev)
    t_q = {}
    for tiled in ("1", "0"):
        os.environ["NFFT_GB300_DIRECTIONAL_TILED"] = tiled
        pq = nf.plan_nfft(k2, Nq, dims=(2, 3), m=4, sigma=2.0)
        vq = nf.as_colmajor(complex_normal(rng, pq.NOut), pq.NOut, torch.complex64, dev)
        yq = nf.empty_image(pq.NOut, torch.complex64, dev)
        xq = nf.empty_image(Nq, torch.complex64, dev)
        t_q[tiled] = timed(lambda: (pq.forward_(yq, fq), pq.adjoint_(xq, vq)))
        del pq, vq, yq, xq
    os.environ.pop("NFFT_GB300_DIRECTIONAL_TILED", None)
    emit("directional 2-D NFFT (dims 2:3) of a 64x256x256 stack: fwd+adj node values/s", J * Nq[0] / t_q["1"],
         "node values/s", t_q["1"] * 1e3,
         {"workload": "N=(64,256,256), dims=2:3 (64 columns before the transform dims), the 2-D radial nodes "
                      "above (J=131072), KB m=4 sigma=2, LINEAR"},
         dtype="f32", atomic_path={"ms_per_step": t_q["0"] * 1e3, "speedup_of_value": t_q["0"] / t_q["1"]})
    del fq
    torch.cuda.empty_cache()

    # ---- 3-D NFCT / NFST
    Nt = (64, 64, 64)
    Mt = 1 << 20
    kt = (0.5 * rng.random((3, Mt))).astype(np.float32)
    sel = rng.choice(Mt, 64, replace=False)
    for kind in ("nfct", "nfst"):
        plan = (nf.plan_nfct if kind == "nfct" else nf.plan_nfst)(kt, Nt, m=4, sigma=2.0)
        shp = plan.size_in()
        ft = nf.as_colmajor(rng.standard_normal(shp).astype(np.float32), shp, torch.float32, dev)
        vt = torch.as_tensor(rng.standard_normal(Mt).astype(np.float32)).to(dev)
        gt = torch.empty(Mt, dtype=torch.float32, device=dev)
        xt = nf.empty_image(shp, torch.float32, dev)
        t_t = timed(lambda: (plan.forward_(gt, ft), plan.transpose_(xt, vt)))
        plan.forward_(gt, ft)
        direct = (nf.NDCTPlan if kind == "nfct" else nf.NDSTPlan)(kt[:, sel], Nt) * ft
        err = rel_l2(gt.cpu().numpy()[sel], direct.cpu().numpy())
        emit(f"3-D {kind.upper()} fwd+transpose nodes/s, N=64^3, 2^20 nodes, FP32", Mt / t_t, UNIT, t_t * 1e3,
             {"workload": f"{kind.upper()} N=64^3 (NFFT of 128^3), M=2^20 nodes in [0,1/2)^3, KB m=4 sigma=2"},
             dtype="f32", rel_err_vs_direct_gpu_sums=err)
        del plan, ft, vt, gt, xt
        torch.cuda.empty_cache()

    # ---- sdc on the 2-D spiral
    ksp = spiral_nodes(256).astype(np.float32)
    psd = nf.plan_nfft(ksp, (256, 256), m=4, sigma=2.0, precompute=nf.TENSOR)
    t_sdc = timed(lambda: tools.sdc(psd, iters=20))
    emit("NFFTTools sdc (20 iterations) on the 2-D spiral 256^2, FP32: weight sets/s", 1.0 / t_sdc, "weight sets/s",
         t_sdc * 1e3, {"workload": "32 interleaves x 2048 samples, N=256^2, KB m=4 sigma=2, TENSOR"}, dtype="f32")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precompute", default="tensor", choices=["tensor", "polynomial", "full", "linear"],
                    help="window evaluation of the plan (PrecomputeFlags)")
    ap.add_argument("--blocksize", default=None, help="spreading tile, e.g. 16,8,8 (NFFTParams.blockSize)")
    ap.add_argument("--autotune", type=int, default=1, help="1: pick the tile with the library's autotuner")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--small", action="store_true",
                    help="profiling case of the same kernels: N=128^3, 2048 spokes x 256 samples (same node "
                         "density; 134 MB grid, above L2) -- not a bench line")
    ap.add_argument("--workload", default="radial3d",
                    choices=["radial3d", "batched2d", "plain2d", "line1d", "spiral2d", "radial3d_fp64",
                             "toeplitz3d", "extras"],
                    help="radial3d: the headline line; the others print extra lines for the other configurations")
    args = ap.parse_args()
    if args.workload == "batched2d":
        return run_batched(args)
    if args.workload == "toeplitz3d":
        return run_toeplitz(args)
    if args.workload == "extras":
        return run_extras(args)
    if args.workload in CONFIGS:
        return run_config(args)
    if args.small:
        global N3, SPOKES, SAMPLES, M_NODES, WORKLOAD
        N3, SPOKES, SAMPLES = (128, 128, 128), 2048, 256
        M_NODES = SPOKES * SAMPLES
        WORKLOAD = ("3D radial koosh-ball NFFT fwd+adj, N=128^3, 2048 spokes x 256 samples (M=524288), "
                    "KB m=4 sigma=2 (profiling case)")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
