"""Benchmark of the headline workload: Zernike GLQ forward + backward
transforms at order 200 on a batch of 64 functions (the reference's
zt::GLQTransformerGeo), in the split-precision form (BF16 fixed-point slices
on tcgen05) and in the plain FP64 form on the same GPU.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision split|fp64|auto] [--order 200] [--batch 64]

One step = forward_transform then backward_transform of the whole batch
(grid -> coefficients -> grid).  Inputs: coefficients drawn i.i.d.
N(0, (n+1)^-3) for valid (n,l,m), Im(m=0) = 0, seeds 1..batch, synthesised to
the order-200 ball grid by the FP64 backward transform (synthetic data; the
reference publishes no dataset).  The batch of grids (8.5 GB) is larger than
L2, so every step streams its inputs from HBM.

Prints one JSON line (rank 0).  `value` is transforms/s over the timed region
with inputs resident in HBM; `e2e` is the same metric through the C-ABI with
pinned host buffers (host<->device copies inside the timed region).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from zest_gb300.replicas import max_over_ranks, replica_seed0, whole_job_rate  # noqa: E402

METRIC = "Zernike fwd+bwd transforms/s, order 200x64: split-prec vs FP64 GPU at 1e-11 err"
# DRAM read + write bytes of one forward+backward step per function at order
# 200, from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of
# the launches of a step at batch 4, which grow in proportion to the batch:
# the seven split GEMM launches (6.464 GB) and the six slicing launches
# (5.376 GB)
GEMM_DRAM_BYTES_PER_FUNCTION_ORDER200 = 6.464e9 / 4
SLICE_DRAM_BYTES_PER_FUNCTION_ORDER200 = 5.376e9 / 4
# the least a forward+backward transform can move at order 200: the grid read
# and written once, the coefficients written and read once
MIN_BYTES_PER_FUNCTION_ORDER200 = 288.7e6
UNIT = "transforms/s"


# --------------------------------------------------------------------------
def zt_flops_per_function(L: int) -> dict:
    """Canonical (reference-algorithm) flop count of one forward+backward
    transform: 2 * [2 nlat nrad L(L+1) + 4 nrad T(L) + 2.5 nrad nlat nlon log2 nlon]."""
    nlon, nlat, nrad = 2 * L - 1, L + 1, (L + 1 + 7) // 8 * 8
    T = (L + 1) * (L + 3) * (2 * L + 1) // 24
    leg = 2 * nlat * nrad * L * (L + 1)
    rad = 4 * nrad * T
    fft = 2.5 * nrad * nlat * nlon * np.log2(nlon)
    return {"legendre": 2 * leg, "radial": 2 * rad, "fft": 2 * fft, "total": 2 * (leg + rad + fft)}


def zt_coeffs(L: int, batch: int, seed0: int = 1) -> np.ndarray:
    """c_nlm ~ N(0, (n+1)^-3) i.i.d., Im(m=0) = 0, seed seed0 + b for item b."""
    from zest_gb300 import zt_coeff_size
    T = zt_coeff_size(L)
    n_of = np.zeros(T, dtype=np.int64)
    m_of = np.zeros(T, dtype=np.int64)
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            base = (n + 1) * (n + 3) * (2 * n + 1) // 24 + (l * l) // 4
            n_of[base:base + l + 1] = n
            m_of[base:base + l + 1] = np.arange(l + 1)
    sd = (n_of + 1.0) ** -1.5
    out = np.empty((batch, T, 2))
    for b in range(batch):
        rng = np.random.default_rng(seed0 + b)
        x = rng.standard_normal((T, 2)) * sd[:, None]
        x[m_of == 0, 1] = 0.0
        out[b] = x
    return out


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        smax = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        power = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(self.rows), "reasons": reasons}


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return {"hbm_gbs": p["hbm_gbs"], "bf16_tflops": p["bf16_tflops"],
                "bf16_tflops_sustained": p.get("bf16_tflops_sustained"), "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


# --------------------------------------------------------------------------
def cpu_reference_sample(grids_host: np.ndarray, L: int, nthreads: int):
    """The reference zest library (oracle/_ref) on the host cores: one
    function per thread, forward + backward, each thread's transformer built
    before the timing.  Returns (transforms/s, kind, sample)."""
    from oracle import Reference
    try:
        ref = Reference()
        kind = "reference"
        n = min(nthreads, grids_host.shape[0])
        secs, _, _ = ref.zt_fwd_bwd_steps(grids_host[:n], L, nthreads, nsteps=1)
        return n / float(secs[0]), kind, (f"{n} order-{L} functions fwd+bwd, one per thread on {nthreads} threads, "
                                          "transformers built before the timing")
    except (FileNotFoundError, OSError):
        from oracle import Oracle
        orc = Oracle()
        t0 = time.perf_counter()
        c = orc.zt_forward(grids_host[0], L)
        orc.zt_backward(c, L)
        secs = time.perf_counter() - t0
        return 1.0 / secs, "port", f"1 order-{L} function fwd+bwd, oracle port, 1 thread"


def reference_grids(ref, coeffs: np.ndarray, L: int, nthreads: int) -> np.ndarray:
    """Grids of the coefficient batch by the reference's own backward
    transform, items in parallel on host threads (ctypes releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=nthreads) as ex:
        return np.stack(list(ex.map(lambda b: ref.zt_backward(coeffs[b], L), range(coeffs.shape[0]))))


def run_reference_arm(args, rank: int, world: int) -> None:
    """`--impl reference`: the reference CPU implementation on the host cores,
    on the same workload: every step transforms the whole batch (64
    functions at order 200), forward then backward, spread over all host
    threads.  Each thread builds its reference transformer once, before the
    timed steps, as a reference user transforming many functions would.  The
    CPU has no clocks to warm up: the warm-up is one untimed step of one
    function per thread."""
    if rank != 0:
        return
    from oracle import Reference
    L, nthreads = args.order, os.cpu_count() or 1
    try:
        ref = Reference()
    except (FileNotFoundError, OSError) as exc:
        print(json.dumps({"impl": "reference", "unavailable": f"reference library not built: {exc}"}))
        return
    per_step = args.batch
    coeffs = zt_coeffs(L, per_step)
    grids = reference_grids(ref, coeffs, L, nthreads)
    ref.zt_fwd_bwd_steps(grids[:min(nthreads, per_step)], L, nthreads, nsteps=1)  # warm-up
    times, _, _ = ref.zt_fwd_bwd_steps(grids, L, nthreads, nsteps=args.steps)
    total = float(np.sum(times))
    value = per_step * args.steps / total
    sample = (f"the whole batch: {per_step} order-{L} functions fwd+bwd per step on {nthreads} threads, "
              "transformers built once before the timed steps")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "step_ms": [round(1e3 * float(t), 1) for t in times],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "zernike_glq_fwd_bwd", "order": L, "batch": args.batch, "precision": "fp64",
                   "conventions": "GLQTransformerGeo (unnormed Zernike, 4pi SH, no CS phase)",
                   "grid": [2 * L - 1, L + 1, (L + 1 + 7) // 8 * 8], "parallelism": f"{nthreads} host threads",
                   "sample_per_step": per_step, "warmup": "one untimed step of one function per thread",
                   "build": "g++ -O3 (-mcpu=native on aarch64)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "reference", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# --------------------------------------------------------------------------
def run_sh(args, rank: int, world: int, barrier) -> None:
    """Spherical harmonics at lmax 1023 (order 1024), batch 8: real
    coefficients N(0, (l+1)^-2) (4pi normalisation, no Condon-Shortley phase),
    synthesised to the LonLat grid (2047 x 1024) and transformed back; one step
    = backward then forward of the batch.  Timed in FP64 and, unless
    --precision fp64, with the Legendre sums in split precision on the tensor
    cores (the value reported).  Error = max over items of
    max|c - c_in| / max|c_in| (the round trip is exact in exact arithmetic)."""
    import torch
    import zest_gb300 as zg
    ctx = zg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    L, B = 1024, 8
    ncoef = zg.st_coeff_size(L)
    rng = np.random.default_rng(1024 + rank)
    l_of = np.zeros(ncoef, dtype=np.int64)
    for l in range(L):
        l_of[l * (l + 1) // 2:(l + 1) * (l + 2) // 2] = l
    c = rng.normal(size=(B, ncoef, 2)) / (l_of[None, :, None] + 1.0)
    c[:, [l * (l + 1) // 2 for l in range(L)], 1] = 0.0
    dev = torch.device("cuda", torch.cuda.current_device())
    cd = torch.from_numpy(c.ravel()).to(dev)
    gd = torch.empty(B * int(np.prod(zg.st_grid_shape(L))), dtype=torch.float64, device=dev)
    cout = torch.empty_like(cd)

    def step():
        ctx.st_backward(cd, L, batch=B, out=gd)
        ctx.st_forward(gd, L, batch=B, out=cout)

    def timed(nsteps, nwarm):
        for _ in range(nwarm):
            step()
        torch.cuda.synchronize()
        barrier()
        sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        sampler.start()
        ctx.profile(True)
        ctx.profile_read(reset=True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(nsteps):
            step()
        e1.record()
        torch.cuda.synchronize()
        clocks = sampler.stop()
        prof = ctx.profile_read(reset=True)
        flops = ctx.profile_flops(reset=True)
        ctx.profile(False)
        ms = max_over_ranks(e0.elapsed_time(e1), None) / nsteps
        err = max(float(np.max(np.abs(x - y)) / np.max(np.abs(y)))
                  for x, y in zip(cout.cpu().numpy().reshape(B, -1), c.reshape(B, -1)))
        timed.flops = (flops[0] / nsteps, flops[1] / nsteps)
        return ms, {k: v[0] / nsteps for k, v in prof.items()}, clocks, err

    ms64, st64, clocks64, err64 = timed(args.steps, args.warmup)
    split = args.precision != "fp64"
    if split:
        g64 = gd.clone()
        ctx.set_precision(zg.PRECISION_SPLIT, 6)
        ms, stages, clocks, err = timed(args.steps, args.warmup)
        ctx.st_backward(cd, L, batch=B, out=gd)
        torch.cuda.synchronize()
        d_grid = float(((gd - g64).abs().reshape(B, -1).amax(1) / g64.abs().reshape(B, -1).amax(1)).max())
        ctx.set_precision(zg.PRECISION_FP64)
    else:
        ms, stages, clocks, err, d_grid = ms64, st64, clocks64, err64, None
    roofline = None
    if split and stages.get("split_gemm"):
        useful, issued = timed.flops
        achieved = useful / (stages["split_gemm"] * 1e-3) / 1e12
        peaks = measured_peaks()
        peak = peaks["bf16_tflops_sustained"] or peaks["bf16_tflops"]
        roofline = {"bound": "tensor", "kernel": "split_gemm_kernel (all launches of a step)", "achieved": achieved,
                    "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                    "algorithmic": "BF16 MMA flops of the slice products on valid rows",
                    "useful_tflop_per_step": useful / 1e12, "issued_tflop_per_step": issued / 1e12,
                    "peak_source": peaks["source"] + " bf16 sustained"}
    # CPU baseline: the compiled reference, one transformer per item and thread
    # built before the timing, one step of backward + forward of the 8 items
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            from oracle import Reference
            ref = Reference()
            nthreads = min(B, os.cpu_count() or 1)
            secs, _, cref = ref.st_bwd_fwd_steps(c, L, nthreads, nsteps=1)
            cpu = {"value": B / float(secs[0]), "unit": "transforms/s", "cores": nthreads, "kind": "reference",
                   "sample": f"the whole batch: {B} items backward + forward, one per thread, transformers "
                             "built before the timing",
                   "roundtrip_max_rel_err": float(max(np.max(np.abs(x - y)) / np.max(np.abs(y))
                                                      for x, y in zip(cref.reshape(B, -1), c.reshape(B, -1))))}
        except (FileNotFoundError, OSError) as exc:
            cpu = {"unavailable": str(exc)}
    if rank == 0:
        print(json.dumps({
            "metric": "SH backward+forward transforms/s, lmax 1023 x 8" + (", split-precision Legendre sums"
                                                                             if split else ", FP64"),
            "value": world * B / (ms * 1e-3), "unit": "transforms/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 digit slices, fp64 recombination" if split else "f64",
            "data": "synthetic", "config": {"workload": "sh_glq_bwd_fwd", "order": 1024, "batch": B,
                                            "layout": "LonLat", "conventions": "GLQTransformerGeo",
                                            "precision": "split" if split else "fp64"},
            "roundtrip_max_rel_err": err,
            "backward_grid_max_rel_err_vs_fp64": d_grid,
            "fp64_gpu": {"value": world * B / (ms64 * 1e-3), "ms_per_step": ms64, "stages_ms": st64,
                         "roundtrip_max_rel_err": err64},
            "split_vs_fp64": (ms64 / ms) if split else None,
            "stages_ms": stages, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks}), flush=True)


def run_evaluate(args, rank: int, world: int, barrier) -> None:
    """Zernike expansions evaluated at arbitrary points (zt::GridEvaluator):
    order 100, batch 8, c_nlm ~ N(0, (n+1)^-2), on the product grid of 200
    longitudes, 100 colatitudes and 100 radii drawn uniformly (seeded).  One
    step = the evaluation of the batch (tables, radial, Legendre and longitude
    sums), FP64.  The dominant stage is the longitude sum, a dense FP64
    product of 2 * nlon * (nlat * nrad) * 2L flops per item, reported against
    the FP64 pipe's 1.20 TFLOP/s.  The reference's evaluator (one thread per
    item) is timed on one item for the CPU baseline."""
    import torch
    import zest_gb300 as zg
    ctx = zg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    L, B, nlon, nlat, nrad = 100, 8, 200, 100, 100
    rng = np.random.default_rng(4242 + rank)
    c = zt_coeffs(L, B, seed0=replica_seed0(rank, B))
    lon = rng.uniform(0.0, 2.0 * np.pi, nlon)
    colat = rng.uniform(0.0, np.pi, nlat)
    rad = rng.uniform(0.0, 1.0, nrad)
    dev = torch.device("cuda", torch.cuda.current_device())
    cd = torch.from_numpy(c.ravel()).to(dev)
    lon_d, colat_d, rad_d = (torch.from_numpy(v).to(dev) for v in (lon, colat, rad))
    vd = torch.empty(B * nlon * nlat * nrad, dtype=torch.float64, device=dev)

    def step():
        ctx.zt_evaluate(cd, L, lon_d, colat_d, rad_d, batch=B, out=vd)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    ctx.profile(True)
    ctx.profile_read(reset=True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    prof = ctx.profile_read(reset=True)
    ms = max_over_ranks(e0.elapsed_time(e1), None) / args.steps
    stages = {k: v[0] / args.steps for k, v in prof.items()}
    lon_flops = 2.0 * nlon * nlat * nrad * 2 * L * B
    lon_ms = stages.get("eval_longitude")
    achieved = lon_flops / (lon_ms * 1e-3) / 1e12 if lon_ms else None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            from oracle import Reference
            ref = Reference()
            t0 = time.perf_counter()
            want = ref.zt_evaluate(c[0], L, lon, colat, rad)
            secs = time.perf_counter() - t0
            got = vd[: nlon * nlat * nrad].cpu().numpy()
            cpu = {"value": 1.0 / secs, "unit": "expansions/s", "cores": 1, "kind": "reference",
                   "sample": "one order-100 expansion on the 200 x 100 x 100 points, zt::GridEvaluator",
                   "max_rel_err_vs_reference": float(np.max(np.abs(got - want.ravel())) / np.max(np.abs(want)))}
        except (FileNotFoundError, OSError) as exc:
            cpu = {"unavailable": str(exc)}
    if rank == 0:
        print(json.dumps({
            "metric": "Zernike expansions evaluated at arbitrary points per second, order 100, 2e6 points",
            "value": world * B / (ms * 1e-3), "unit": "expansions/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "zernike_grid_evaluator", "order": L, "batch": B,
                       "points": [nlon, nlat, nrad], "conventions": "GLQTransformerGeo"},
            "roofline": {"bound": "fp64", "kernel": "gemm64_kernel<EvLon> (longitude sum)", "achieved": achieved,
                         "peak": 1.20, "unit": "TFLOP/s", "frac": achieved / 1.20 if achieved else None,
                         "peak_source": "DFMA microbenchmark on GB300 (1.20 TFLOP/s)"},
            "stages_ms": stages, "cpu_baseline": cpu, "clocks": clocks}), flush=True)


def _timed_loop(step, args, barrier):
    """Warm-up, then args.steps steps between CUDA events on the current stream
    (the context's stream is the legacy default stream): ms per step, clocks."""
    import torch
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    return max_over_ranks(e0.elapsed_time(e1), None) / args.steps, clocks


def run_spectra(args, rank: int, world: int, barrier) -> None:
    """Power spectra (power_spectra.hpp): the SH spectra of 8 expansions at
    lmax 1023 (the C2 coefficients) per step, and beside them the Zernike
    spectra of 64 expansions at order 200.  One thread per output sums over m
    in FP64; the bound is reading the coefficients once.  The CPU baseline is
    the C restatement of the same sums on one item."""
    import torch
    import zest_gb300 as zg
    ctx = zg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    L, B = 1024, 8
    rng = np.random.default_rng(1024 + rank)
    ncoef = zg.st_coeff_size(L)
    c = rng.normal(size=(B, ncoef, 2))
    dev = torch.device("cuda", torch.cuda.current_device())
    cd = torch.from_numpy(c.ravel()).to(dev)
    sd = torch.empty(B * L, dtype=torch.float64, device=dev)
    ms, clocks = _timed_loop(lambda: ctx.st_power_spectrum(cd, L, batch=B, out=sd), args, barrier)
    Lz, Bz = 200, 64
    zc = torch.from_numpy(zt_coeffs(Lz, Bz, seed0=replica_seed0(rank, Bz)).ravel()).to(dev)
    zs = torch.empty(Bz * (((Lz + 1) * (Lz + 1)) >> 2), dtype=torch.float64, device=dev)
    ms_z, _ = _timed_loop(lambda: ctx.zt_power_spectrum(zc, Lz, batch=Bz, out=zs), args, barrier)
    nbytes = B * ncoef * 16 + B * L * 8
    achieved = nbytes / (ms * 1e-3) / 1e9
    peaks = measured_peaks()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import Oracle
        orc = Oracle()
        t0 = time.perf_counter()
        want = orc.st_power_spectrum(c[0].ravel(), L)
        secs = time.perf_counter() - t0
        got = sd[:L].cpu().numpy()
        cpu = {"value": 1.0 / secs, "unit": "spectra/s", "cores": 1, "kind": "port",
               "sample": "one lmax-1023 SH spectrum, C restatement",
               "max_rel_err_vs_port": float(np.max(np.abs(got - want)) / np.max(np.abs(want)))}
    if rank == 0:
        print(json.dumps({
            "metric": "SH power spectra per second, lmax 1023 x 8", "value": world * B / (ms * 1e-3),
            "unit": "spectra/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "sh_power_spectrum", "order": L, "batch": B},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                         "algorithmic": "coefficients read once + spectra written"},
            "zernike_order200_x64": {"ms": ms_z, "spectra_per_s": world * Bz / (ms_z * 1e-3)},
            "cpu_baseline": cpu, "clocks": clocks}), flush=True)


def run_lsq(args, rank: int, world: int, barrier) -> None:
    """Least-squares fits to scattered data (st::LSQTransformer): 16 data
    vectors at 20,000 seeded points fitted with SH expansions of order 32
    (1,024 real unknowns) per step; the design matrix is built on the device
    and solved by the library's blocked Householder QR.  Beside it, the
    Zernike fit of order 12.  The CPU baseline is numpy's least-squares solve
    of the same design matrix, built from the oracle's tables outside the
    timed region."""
    import torch
    import zest_gb300 as zg
    ctx = zg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    L, B, npts = 32, 16, 20000
    rng = np.random.default_rng(3232 + rank)
    lat = np.arcsin(rng.uniform(-1, 1, npts))
    lon = rng.uniform(0, 2 * np.pi, npts)
    data = rng.normal(size=(B, npts))
    dev = torch.device("cuda", torch.cuda.current_device())
    dd = torch.from_numpy(data.ravel()).to(dev)
    lat_d, lon_d = (torch.from_numpy(v).to(dev) for v in (lat, lon))
    cd = torch.empty(B * 2 * zg.st_coeff_size(L), dtype=torch.float64, device=dev)
    ms, clocks = _timed_loop(lambda: ctx.st_lsq(dd, L, lat_d, lon_d, batch=B, out=cd), args, barrier)
    Lz = 12
    r = rng.uniform(0, 1, npts) ** (1 / 3)
    colat = np.arccos(rng.uniform(-1, 1, npts))
    r_d, colat_d = (torch.from_numpy(v).to(dev) for v in (r, colat))
    czd = torch.empty(B * 2 * zg.zt_coeff_size(Lz), dtype=torch.float64, device=dev)
    ms_z, _ = _timed_loop(lambda: ctx.zt_lsq(dd, Lz, r_d, lon_d, colat_d, batch=B, out=czd), args, barrier)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import Oracle, tri_idx
        orc = Oracle()
        P = orc.plm_real(L, 0, 0, np.sin(lat))
        cols = []
        for l in range(L):
            for m in range(l + 1):
                p_ = P[tri_idx(l, m)]
                cols.append(p_ * np.cos(m * lon))
                if m:
                    cols.append(p_ * np.sin(m * lon))
        A = np.stack(cols, axis=1)
        t0 = time.perf_counter()
        np.linalg.lstsq(A, data.T, rcond=None)
        secs = time.perf_counter() - t0
        cpu = {"value": B / secs, "unit": "fits/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "numpy lstsq of the same 20000 x 1024 design matrix, 16 right-hand sides"}
    if rank == 0:
        print(json.dumps({
            "metric": "SH least-squares fits per second, order 32, 20000 points, 16 data vectors",
            "value": world * B / (ms * 1e-3), "unit": "fits/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "sh_lsq", "order": L, "points": npts, "batch": B},
            "roofline": None, "zernike_order12": {"ms": ms_z, "fits_per_s": world * B / (ms_z * 1e-3)},
            "cpu_baseline": cpu, "clocks": clocks}), flush=True)


def run_rotate(args, rank: int, world: int, barrier) -> None:
    """Rotor::rotate of 256 Zernike expansions of order 64 (the alignment
    configuration's batch), Haar-uniform Euler angles, coefficients
    N(0, (n+1)^-2): the FP64 rotation (one warp per (n, l) vector) and, in
    split precision, the two X(+-pi/2) products of all vectors of one l as
    split GEMMs on the tensor cores.  One step = one rotation call on device
    memory (in place)."""
    import torch
    import zest_gb300 as zg
    ctx = zg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    L, B = 64, 256
    rng = np.random.default_rng(6400 + rank)
    c = zt_coeffs(L, B, seed0=replica_seed0(rank, B)) * 1.0
    e = np.stack([rng.uniform(0, 2 * np.pi, B), np.arccos(rng.uniform(-1, 1, B)), rng.uniform(0, 2 * np.pi, B)], 1)
    dev = torch.device("cuda", torch.cuda.current_device())
    c0 = torch.from_numpy(c.ravel()).to(dev)
    ed = torch.from_numpy(np.ascontiguousarray(e).ravel()).to(dev)
    cd = c0.clone()
    out = {}
    for name, prec in (("fp64", zg.PRECISION_FP64), ("split", zg.PRECISION_SPLIT)):
        ctx.set_precision(prec, 6 if prec else 0)
        ms, clocks = _timed_loop(lambda: ctx.zt_rotate(cd, L, ed, batch=B), args, barrier)
        cd.copy_(c0)
        ctx.zt_rotate(cd, L, ed, batch=B)
        torch.cuda.synchronize()
        out[name] = {"ms": ms, "result": cd.clone(), "clocks": clocks}
        cd.copy_(c0)
    ctx.set_precision(zg.PRECISION_FP64)
    a, b = out["split"]["result"].reshape(B, -1), out["fp64"]["result"].reshape(B, -1)
    err = float(((a - b).abs().amax(1) / b.abs().amax(1)).max())
    if rank == 0:
        print(json.dumps({
            "metric": "Zernike rotations per second, order 64 x 256 (Rotor::rotate)",
            "value": world * B / (out["split"]["ms"] * 1e-3), "unit": "rotations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["split"]["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 digit slices, fp64 recombination",
            "data": "synthetic", "config": {"workload": "zernike_rotate", "order": L, "batch": B},
            "fp64_gpu": {"value": world * B / (out["fp64"]["ms"] * 1e-3), "ms_per_step": out["fp64"]["ms"]},
            "split_vs_fp64": out["fp64"]["ms"] / out["split"]["ms"],
            "max_rel_err_vs_fp64": err, "clocks": out["split"]["clocks"]}), flush=True)


def run_batching(args, rank: int, world: int, barrier) -> None:
    """4096 expansions, orders drawn uniformly from [8, 128] (sorted), c_nlm ~
    N(0, (n+1)^-2) with Im(m=0) = 0, Haar-uniform Euler angles; one step =
    Rotor::rotate of every expansion then its backward transform, all through
    zest_gpu_zt_rotate_backward_ragged (a CUDA graph replay after the first
    call).  Reports expansions/s and the step's HBM traffic against the
    measured copy bandwidth."""
    import torch
    import zest_gb300 as zg
    ctx = zg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    precision = args.precision if args.precision != "auto" else "split"
    ctx.set_precision(zg.PRECISION_SPLIT if precision == "split" else zg.PRECISION_FP64, args.slices)
    ctx.set_autotune(True)
    rng = np.random.default_rng(4096 + rank)
    n = args.items
    orders = np.sort(rng.integers(8, 129, size=n)).astype(np.int32)
    csz = [2 * zg.zt_coeff_size(int(L)) for L in orders]
    gsz = [int(np.prod(zg.zt_grid_shape(int(L)))) for L in orders]
    dev = torch.device("cuda", torch.cuda.current_device())
    coeffs = torch.empty(sum(csz), dtype=torch.float64, device=dev)
    grids = torch.empty(sum(gsz), dtype=torch.float64, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(4096 + rank)
    scales = {}
    off = 0
    for L, c in zip(orders, csz):
        L = int(L)
        if L not in scales:
            sc = np.zeros((c // 2, 2))
            for nn in range(L):
                for l in range(nn & 1, nn + 1, 2):
                    base = (nn + 1) * (nn + 3) * (2 * nn + 1) // 24 + (l * l) // 4
                    sc[base:base + l + 1] = (nn + 1) ** -1.0
                    sc[base, 1] = 0.0
            scales[L] = torch.from_numpy(sc.ravel()).to(dev)
        coeffs[off:off + c] = torch.randn(c, dtype=torch.float64, device=dev, generator=gen) * scales[L]
        off += c
    e = np.stack([rng.uniform(0, 2 * np.pi, n), np.arccos(rng.uniform(-1, 1, n)), rng.uniform(0, 2 * np.pi, n)], 1)
    euler = torch.from_numpy(np.ascontiguousarray(e).ravel()).to(dev)
    ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)  # eager run, autotuning, graph capture
    for _ in range(args.warmup):
        ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)
    ctx.synchronize()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    stream = torch.cuda.current_stream()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # the library works on its own stream: time with host-synchronised events around it
    ctx.synchronize()
    e0.record(stream)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)
    ctx.synchronize()
    t1 = time.perf_counter()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ms = (t1 - t0) * 1e3 / args.steps

    # error against the FP64 form on identical inputs: one more call in each
    # precision from the same coefficients (the rotation works in place)
    c0 = coeffs.clone()
    ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)
    ctx.synchronize()
    g_split = grids.clone() if precision == "split" else None
    err_vs_fp64 = None
    if g_split is not None:
        coeffs.copy_(c0)
        ctx.set_precision(zg.PRECISION_FP64)
        ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)
        ctx.synchronize()
        err_vs_fp64 = 0.0
        goff = 0
        for L in np.unique(orders):   # items of one order are contiguous and of one size
            cnt = int(np.sum(orders == L))
            gs = int(np.prod(zg.zt_grid_shape(int(L))))
            a = g_split[goff:goff + cnt * gs].reshape(cnt, gs)
            b = grids[goff:goff + cnt * gs].reshape(cnt, gs)
            err_vs_fp64 = max(err_vs_fp64, float(((a - b).abs().amax(1) / b.abs().amax(1)).max()))
            goff += cnt * gs
        g_split = None
        ctx.set_precision(zg.PRECISION_SPLIT, args.slices)

    # CPU baseline: the reference's Rotor::rotate + backward_transform on all
    # host threads, on a bounded sample of the batch (every 8th item of the
    # sorted orders: the same distribution); every 64th item is also compared
    # with this library's result
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            from oracle import Reference
            ref = Reference()
            coff = np.concatenate([[0], np.cumsum(csz)])
            goffs = np.concatenate([[0], np.cumsum(gsz)])
            c0_h = c0.cpu().numpy()
            e_h = e
            pick = np.arange(0, n, 8)
            sample_c = np.concatenate([c0_h[coff[i]:coff[i + 1]] for i in pick])
            nthreads = os.cpu_count() or 1
            secs, _ = ref.zt_rotate_backward_ragged(orders[pick], sample_c, e_h[pick], nthreads)
            check = np.arange(0, n, 64)
            chk_c = np.concatenate([c0_h[coff[i]:coff[i + 1]] for i in check])
            _, want = ref.zt_rotate_backward_ragged(orders[check], chk_c, e_h[check], nthreads, want_grids=True)
            worst, woff = 0.0, 0
            for i in check:
                gs = int(gsz[i])
                got = grids[goffs[i]:goffs[i] + gs].cpu().numpy()
                w = want[woff:woff + gs]
                worst = max(worst, float(np.max(np.abs(got - w)) / np.max(np.abs(w))))
                woff += gs
            cpu = {"value": pick.size / secs, "unit": "expansions/s", "cores": nthreads, "kind": "reference",
                   "sample": f"{pick.size} of the {n} items (every 8th of the sorted orders), Rotor::rotate + "
                             "backward_transform, contiguous runs of equal cost per thread, rotors and "
                             "transformers built before the timing",
                   "max_rel_err_vs_reference": worst,
                   "compared_items": int(check.size),
                   "compared_form": "fp64" if precision == "split" else precision}
        except (FileNotFoundError, OSError) as exc:
            cpu = {"unavailable": str(exc)}

    T = np.array([zg.zt_coeff_size(int(L)) for L in orders], dtype=np.float64)
    G = np.array(gsz, dtype=np.float64)
    bytes_step = float(np.sum(32 * T + 16 * T + 8 * G))
    peaks = measured_peaks()
    achieved = bytes_step / (ms * 1e-3) / 1e9
    if rank == 0:
        print(json.dumps({
            "metric": "Zernike rotate + backward expansions/s, 4096 orders U{8..128}",
            "value": world * n / (ms * 1e-3), "unit": "expansions/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "bf16-slices + f64",
            "data": "synthetic", "config": {"workload": "zernike_ragged_rotate_backward", "items": n,
                                            "orders": "U{8..128} sorted", "precision": precision,
                                            "graph": "CUDA graph replay", "autotune": True},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                         "algorithmic": "32 T(L) rotate in place + 16 T(L) coefficient read + 8 G(L) grid write",
                         "bytes_per_step": bytes_step},
            "timing": "host wall clock around K graph launches, device synchronised on both sides",
            "max_rel_err_vs_fp64": err_vs_fp64,
            "error_measure": "max over items of max|g - g_fp64| / max|g_fp64| of the backward grids",
            "cpu_baseline": cpu, "clocks": clocks}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["split", "fp64", "auto"], default="auto")
    ap.add_argument("--order", type=int, default=200)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=["transforms", "batching", "sh", "evaluate", "spectra", "lsq", "rotate"],
                    default="transforms",
                    help="transforms: the headline (order 200 x 64 forward+backward); batching: 4096 "
                         "expansions of orders U{8..128}, rotate + backward in one graph")
    ap.add_argument("--items", type=int, default=4096)
    ap.add_argument("--no-autotune", action="store_true",
                    help="use the size rule for the FP64 tile shapes instead of timing them on first use")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return

    import torch
    import zest_gb300 as zg

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        dist = tdist

    def barrier():
        if dist is not None:
            dist.barrier()

    if args.workload == "batching":
        run_batching(args, rank, world, barrier)
        return
    if args.workload == "sh":
        run_sh(args, rank, world, barrier)
        return
    if args.workload == "evaluate":
        run_evaluate(args, rank, world, barrier)
        return
    if args.workload == "spectra":
        run_spectra(args, rank, world, barrier)
        return
    if args.workload == "lsq":
        run_lsq(args, rank, world, barrier)
        return
    if args.workload == "rotate":
        run_rotate(args, rank, world, barrier)
        return

    L, B = args.order, args.batch
    ctx = zg.Context(local_rank)
    if args.no_autotune:
        ctx.set_autotune(False)
    precision = args.precision
    if precision == "auto":
        try:
            ctx.set_precision(zg.PRECISION_SPLIT, args.slices)
            precision = "split"
        except zg.ZestGPUError:
            precision = "fp64"
    ctx.set_precision(zg.PRECISION_FP64)

    gsz = int(np.prod(zg.zt_grid_shape(L)))
    csz = 2 * zg.zt_coeff_size(L)
    coeffs_h = zt_coeffs(L, B, seed0=replica_seed0(rank, B))
    coeffs_d = torch.from_numpy(coeffs_h.ravel()).cuda()
    grids_d = ctx.zt_backward(coeffs_d, L, batch=B)          # FP64 synthesis of the inputs
    cbuf = torch.empty(B * csz, dtype=torch.float64, device="cuda")
    gout = torch.empty(B * gsz, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    def step():
        ctx.zt_forward(grids_d, L, batch=B, out=cbuf)
        ctx.zt_backward(cbuf, L, batch=B, out=gout)

    def timed(nsteps: int, nwarm: int, sampler=None):
        for _ in range(nwarm):
            step()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        n0 = zg.launch_count()
        ctx.profile(True)
        ctx.profile_read(reset=True)
        if sampler:
            sampler.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(nsteps):
            step()
        e1.record()
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        prof = ctx.profile_read(reset=True)
        ctx.profile(False)
        launches = zg.launch_count() - n0
        barrier()
        flops = ctx.profile_flops(reset=True)
        ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
        return ms, prof, launches, clocks, flops

    # ---- plain FP64 form (always measured: it is the ratio's denominator) ----
    fp64_steps = args.steps
    fp64_warm = args.warmup
    sampler = ClockSampler(local_rank) if precision == "fp64" else None
    ms64, prof64, launches64, clocks64, _ = timed(fp64_steps, fp64_warm, sampler)
    ref_coeffs = cbuf.clone()
    ref_grids = gout.clone()
    result = {"fp64": {"ms_per_step": ms64 / fp64_steps, "value": world * B * fp64_steps / (ms64 * 1e-3),
                       "stages_ms": {k: v[0] / fp64_steps for k, v in prof64.items()}}}

    flops = zt_flops_per_function(L)
    peaks = measured_peaks()
    def relerr(x, ref):
        return float(((x - ref).abs().reshape(B, -1).amax(1) / ref.abs().reshape(B, -1).amax(1)).max())

    errors = None
    if precision == "split":
        ctx.set_precision(zg.PRECISION_SPLIT, args.slices)
        sampler = ClockSampler(local_rank)
        ms, prof, launches, clocks, tflops = timed(args.steps, args.warmup, sampler)
        err_rt = relerr(gout, ref_grids)          # split fwd -> split bwd vs fp64 fwd -> fp64 bwd
        # each transform on identical inputs: forward of the same grids, backward of the same coefficients
        ctx.zt_forward(grids_d, L, batch=B, out=cbuf)
        err_c = relerr(cbuf, ref_coeffs)
        ctx.zt_backward(ref_coeffs, L, batch=B, out=gout)
        ctx.set_precision(zg.PRECISION_FP64)
        g64 = ctx.zt_backward(ref_coeffs, L, batch=B)
        err_g = relerr(gout, g64)
        del g64
        errors = {"forward_coeffs": err_c, "backward_grid": err_g, "roundtrip_grid": err_rt,
                  "measure": "max over the batch of max|x - x_fp64| / max|x_fp64| per function"}
        dtype = "bf16 digit slices (8-bit fixed point, 6 per operand), fp32 exact level sums, fp64 recombination"
    else:
        ms, prof, launches, clocks, tflops = ms64, prof64, launches64, clocks64, (0.0, 0.0)
        dtype = "f64"
    value = whole_job_rate(B * args.steps, world, ms * 1e-3)

    # ---- roofline of the dominant stage, from the live CUDA-event stage timings ----
    steps_run = args.steps
    stage_ms = {k: v[0] / steps_run for k, v in prof.items()}
    stage_n = {k: v[1] / steps_run for k, v in prof.items()}
    if precision == "split":
        gemm_ms = stage_ms.get("split_gemm", float("nan"))
        useful, issued = tflops[0] / steps_run, tflops[1] / steps_run
        achieved = useful / (gemm_ms * 1e-3) / 1e12 if gemm_ms == gemm_ms and gemm_ms > 0 else None
        peak = peaks["bf16_tflops_sustained"] or peaks["bf16_tflops"]
        # DRAM bytes of the eight split_gemm_kernel launches of one step, from one
        # ncu capture at order 200 x 4 (7.30 GB, proportional to the batch)
        launches_per_step = stage_n.get("split_gemm", 8.0) or 8.0
        traffic = GEMM_DRAM_BYTES_PER_FUNCTION_ORDER200 * B / launches_per_step if L == 200 else None
        roofline = {"bound": "tensor", "kernel": "split_gemm_kernel (per launch, averaged over a step's launches)",
                    "achieved": achieved,
                    "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if achieved else None,
                    "traffic": traffic, "traffic_unit": "bytes per launch (ncu dram read + write)",
                    "peak_source": peaks["source"] + " bf16 sustained",
                    "algorithmic": "BF16 MMA flops of the slice products on valid rows",
                    "useful_tflop_per_step": useful / 1e12, "issued_tflop_per_step": issued / 1e12,
                    "issued_rate": issued / (gemm_ms * 1e-3) / 1e12 if achieved else None,
                    "dram_rate_tbs": (traffic * launches_per_step / (gemm_ms * 1e-3) / 1e12
                                      if traffic and gemm_ms == gemm_ms and gemm_ms > 0 else None),
                    "hbm_peak_tbs": peaks["hbm_gbs"] / 1e3 if peaks.get("hbm_gbs") else None}
        if L == 200:
            gb, sb = GEMM_DRAM_BYTES_PER_FUNCTION_ORDER200 * B, SLICE_DRAM_BYTES_PER_FUNCTION_ORDER200 * B
            roofline["step_traffic"] = {
                "gemm_bytes": gb, "slice_bytes": sb, "total_bytes": gb + sb,
                "algorithmic_min_bytes": MIN_BYTES_PER_FUNCTION_ORDER200 * B,
                "total_over_min": (gb + sb) / (MIN_BYTES_PER_FUNCTION_ORDER200 * B),
                "slice_rate_tbs": (sb / (stage_ms["split_slice"] * 1e-3) / 1e12
                                   if stage_ms.get("split_slice") else None),
                "source": "ncu dram read + write of the launches of one step at batch 4, times batch / 4"}
    else:
        # FP64 form: the dominant stage is the folded Legendre contraction, bound by
        # the FP64 pipe (1.20 TFLOP/s DFMA measured on this GPU model)
        leg_ms = stage_ms.get("legendre_fwd", 0.0) + stage_ms.get("legendre_bwd", 0.0)
        leg_flops = B * flops["legendre"] / 2.0  # folded: half the reference's Legendre flops
        achieved = leg_flops / (leg_ms * 1e-3) / 1e12 if leg_ms else None
        roofline = {"bound": "fp64", "kernel": "legendre_fwd+legendre_bwd", "achieved": achieved,
                    "peak": 1.20, "unit": "TFLOP/s", "frac": achieved / 1.20 if achieved else None,
                    "traffic": None, "peak_source": "DFMA microbenchmark on GB300 (1.20 TFLOP/s)"}

    # ---- end to end through the C-ABI with pinned host buffers ----
    e2e = None
    if precision == "split":
        ctx.set_precision(zg.PRECISION_SPLIT, args.slices)
    if not args.no_e2e:
        # pinned host buffers from cudaHostAlloc (torch's pinned allocator);
        # ordinary allocations pinned with zest_gpu_host_register ran this
        # step at 1.2 s instead of 0.09 s on the GB300 host
        gh = torch.empty(B * gsz, dtype=torch.float64, pin_memory=True)
        gh.copy_(grids_d.cpu())
        ch = torch.empty(B * csz, dtype=torch.float64, pin_memory=True)
        go = torch.empty(B * gsz, dtype=torch.float64, pin_memory=True)

        def e2e_step():
            ctx.zt_forward(gh, L, batch=B, out=ch)
            ctx.zt_backward(ch, L, batch=B, out=go)

        for _ in range(2):  # first touches of the pinned buffers by the copy engines
            e2e_step()
        torch.cuda.synchronize()
        barrier()
        n_e2e = max(10, args.steps)
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            t1 = time.perf_counter()
            e2e_step()
            torch.cuda.synchronize()
            step_ms.append(round(1e3 * (time.perf_counter() - t1), 2))
        secs = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
        # the host link is shared: single steps can take longer, so the mean
        # over all steps is reported and each step's time is listed
        e2e = {"value": whole_job_rate(B * n_e2e, world, secs), "unit": UNIT,
               "h2d_bytes_per_step": B * (gsz + csz) * 8, "d2h_bytes_per_step": B * (csz + gsz) * 8,
               "host_buffers": "pinned (cudaHostAlloc)",
               "steps": n_e2e, "step_ms": step_ms,
               "value_is": "mean over the steps (total transforms / total time)",
               "mean_step_ms": float(np.mean(step_ms)),
               "median_step_ms": float(np.median(step_ms)),
               "rate_at_median_step": world * B / (float(np.median(step_ms)) * 1e-3),
               "host_chunk_bytes": 256 << 20, "pipelined": "uploads, transforms and downloads overlap per chunk"}
        del gh, ch, go

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        grids_host = grids_d[: 16 * gsz].reshape(16, -1).cpu().numpy() if B >= 16 else \
            grids_d.reshape(B, -1).cpu().numpy()
        v, kind, sample = cpu_reference_sample(np.ascontiguousarray(grids_host), L, os.cpu_count() or 1)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": kind, "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {"workload": "zernike_glq_fwd_bwd", "order": L, "batch": B, "precision": precision,
                       "conventions": "GLQTransformerGeo (unnormed Zernike, 4pi SH, no CS phase)",
                       "grid": list(zg.zt_grid_shape(L)), "l2": "inputs larger than L2 (batch of grids 8.5 GB)",
                       "parallelism": f"replicas x{world}"},
            "fp64_gpu": {"value": result["fp64"]["value"], "ms_per_step": result["fp64"]["ms_per_step"],
                         "stages_ms": result["fp64"]["stages_ms"]},
            "split_vs_fp64": value / result["fp64"]["value"] if precision == "split" else None,
            "max_rel_err_vs_fp64": errors,
            "stages_ms": stage_ms, "stage_launches_per_step": stage_n,
            "canonical_gflop_per_function": flops["total"] / 1e9,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clocks,
        }
        print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()



if __name__ == "__main__":
    main()
