#!/usr/bin/env python3
"""Benchmark: batched SIRT slice-iterations/s on one GB300 (per rank).

Workload (the headline configuration): 64 independent slices per GPU, each a
seeded random-ellipse 1024^2 phantom centred in the 1448^2 reconstruction
grid, 1200 angles over [0, pi), 1448 bins; clean sinograms from the Joseph
forward projector, Poisson noise at I0 = 1e5, log-transformed. SIRT with
relaxation_factor 0.25.

  value   slice-iterations/s with sinograms and volumes resident in HBM; one
          step = one SIRT iteration over all 64 slices (one CUDA-graph launch:
          transpose + FP + BP kernels), timed with CUDA events on the
          library's stream, max over ranks.
  e2e     the same metric through the public C ABI with host buffers:
          ufoir_sirt_process on the 64 host sinograms with num-iterations 10
          (the plugin default), including the host->device copy of the
          sinograms and the device->host copy of the volumes.
  --impl reference   the reference's CPU implementation of the path: its own
          OpenCL kernel sources compiled for the host through the oracle's
          OpenCL-C shim (oracle/_ref), driven by the oracle's restatement of
          its host loop, all host threads (the C port where the kernel
          sources are absent).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ufoir|reference]
                       [--methods] [--quick] [--no-serve] [--projector-models]
  --methods            also time the other method workloads (C1, C2 one slice,
                       C3a/b, C4) with a CPU oracle baseline each, and the
                       Joseph/Siddon projector pair
  --projector-models   only the Joseph/Siddon projector timing on one slice
"""
import argparse
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
sys.path.insert(0, os.path.join(ROOT, "ufo-ir_gb300"))

METRIC = "SIRT slice-iters/s @1024²×1200 ang; serve p50/p99 latency vs plain per-job path"
N_DETS, N_ANGLES, PHANTOM, SLICES, I0, RELAX = 1448, 1200, 1024, 64, 1e5, 0.25
E2E_ITERS = 10
E2E_CALLS = 3
# serve trace: the configured request mix (job shapes, methods, iteration
# counts, arrival rate, budget) with its first SERVE_JOBS jobs
SERVE_JOBS = 12
SERVE_TRACE_JOBS = 2000
SERVE_RATE = 200.0
SERVE_SIZES = ((256, 367), (512, 724), (1024, 1448), (2048, 2900))
SERVE_BUDGET = 150 * 10**9
SERVE_SEED = 5005


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Dist:
    """Host-side barrier and max-reduction for timing; no data-path collective."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_median": statistics.median(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-slice DRAM bytes of the dominant kernels from one ncu capture, if committed."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def slice_seeds(rank, S):
    """Phantom seeds of a rank's S slices: ranks reconstruct disjoint slices."""
    return [2000 + rank * S + i for i in range(S)]


def make_inputs(ufoir, ctx, proj, rank, S):
    """Phantoms -> Joseph FP on the GPU -> Poisson noise -> device sinograms."""
    from ufoir import synth
    n, na = N_DETS, N_ANGLES
    vols = np.empty((S, n, n), np.float32)
    for i, seed in enumerate(slice_seeds(rank, S)):
        vols[i] = synth.ellipse_phantom(n, PHANTOM, 10, seed=seed)
    d_vol = ufoir.DeviceArray.from_numpy(ctx, vols)
    d_sino = ufoir.DeviceArray(ctx, (S, na, n), zero=True)
    proj.set(correction_scale=1.0, relaxation=1.0)
    proj.forward(d_vol, d_sino)
    clean = d_sino.download()
    noisy = np.empty_like(clean)
    for i in range(S):
        noisy[i], _ = synth.poisson_noise(clean[i], I0, seed=3000 + rank * S + i)
    d_sino.upload(noisy)
    return d_sino, d_vol, noisy


def _cpu_oracle():
    """The oracle (test infrastructure, used here only as the CPU baseline and
    as the reference result to compare with) with all host threads; which = "ref" when the reference's
    own kernels were built (oracle/_ref), else "port"."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    which = "ref" if pyoracle.ref_available() else "port"
    return pyoracle, threads, which


def _cpu_kind(which):
    return "reference" if which == "ref" else "port"


def _cpu_what(which):
    return ("the reference's OpenCL kernels compiled for the host (oracle/_ref) + the oracle's host loop"
            if which == "ref" else "the oracle's C port of the reference kernels and host loop")


def cpu_baseline(noisy_slice, gpu_result=None):
    """The reference's CPU path on one slice of the workload: one full SIRT
    iteration (all 1200 angles). With gpu_result (slice 0 of the e2e call,
    E2E_ITERS iterations), also the accuracy check: the oracle's result and its FP64
    twin's for the same call, and their relative L2 errors."""
    pyoracle, threads, which = _cpu_oracle()
    step = np.float32(np.pi / N_ANGLES)
    sino = np.ascontiguousarray(noisy_slice, np.float32)
    p = pyoracle.projector(N_DETS, N_ANGLES, step)
    R, Cw = pyoracle.sirt_weights(p, which=which)
    x = np.zeros((N_DETS, N_DETS), np.float32)
    t0 = time.perf_counter()
    pyoracle.sirt_iterate(p, sino, R, Cw, x, 1, RELAX, which=which)
    dt = time.perf_counter() - t0
    out = {"value": 1.0 / dt, "unit": "slice-iters/s", "cores": threads, "kind": _cpu_kind(which),
           "sample": f"1 slice {N_DETS}^2, one SIRT iteration over all {N_ANGLES} angles, {dt:.2f} s; "
                     + _cpu_what(which)}
    if gpu_result is not None:
        want = pyoracle.sirt(pyoracle.projector(N_DETS, N_ANGLES, step), sino, E2E_ITERS, RELAX, which=which)
        want_d = pyoracle.sirt_d(pyoracle.projector(N_DETS, N_ANGLES, step), sino, E2E_ITERS, RELAX)
        g = np.asarray(gpu_result, np.float64)
        out["accuracy"] = {
            "result": f"slice 0 of the e2e call ({E2E_ITERS} SIRT iterations)", "compared_with": _cpu_what(which),
            "rel_l2_vs_oracle": float(np.linalg.norm(g - want) / np.linalg.norm(want)),
            "bit_exact_vs_oracle": bool(np.array_equal(gpu_result, want)),
            "rel_l2_vs_fp64_twin": float(np.linalg.norm(g - want_d) / np.linalg.norm(want_d)),
            "oracle_rel_l2_vs_fp64_twin": float(np.linalg.norm(want.astype(np.float64) - want_d) /
                                                np.linalg.norm(want_d)),
            "bar": "rel-L2 <= 1e-4 against the reference after the stated iterations"}
    return out


def workload_config(S):
    """The workload both arms measure (the reference arm on a bounded sample of it)."""
    return {"workload": f"batched SIRT, {S} slices x {N_DETS}^2 grid ({PHANTOM}^2 phantoms), {N_ANGLES} angles, "
                        f"{N_DETS} bins",
            "slices_per_gpu": S, "n_dets": N_DETS, "n_angles": N_ANGLES, "relaxation_factor": RELAX}


DATA = ("synthetic: seeded random-ellipse 1024^2 phantoms in a 1448^2 grid, Joseph FP, "
        "Poisson noise I0=1e5, log")


def run_reference(args, dist):
    """--impl reference: the reference's CPU path, rank 0 only."""
    if dist.rank != 0:
        return None
    from ufoir import synth
    pyoracle, threads, which = _cpu_oracle()
    step = np.float32(np.pi / N_ANGLES)
    vol = synth.ellipse_phantom(N_DETS, PHANTOM, 10, seed=2000)
    p = pyoracle.projector(N_DETS, N_ANGLES, step)
    sino, _ = synth.poisson_noise(pyoracle.forward(p, vol, which=which), I0, seed=3000)
    R, Cw = pyoracle.sirt_weights(p, which=which)
    x = np.zeros((N_DETS, N_DETS), np.float32)
    for _ in range(args.warmup):
        pyoracle.sirt_iterate(p, sino, R, Cw, x, 1, RELAX, which=which)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pyoracle.sirt_iterate(p, sino, R, Cw, x, 1, RELAX, which=which)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    sample = (f"per step: 1 slice {N_DETS}^2 of the {SLICES}-slice workload, one SIRT iteration over all "
              f"{N_ANGLES} angles; " + _cpu_what(which))
    return {"metric": METRIC, "value": value, "unit": "slice-iters/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": DATA,
            "config": {**workload_config(args.slices),
                       "step": "a bounded sample of the workload: one SIRT iteration of one of its slices "
                               "(all angles) per step, on the host cores",
                       "threads": threads},
            "cpu_baseline": {"value": value, "unit": "slice-iters/s", "cores": threads, "kind": _cpu_kind(which),
                             "sample": sample},
            "e2e": {"value": value, "unit": "slice-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_ufoir(args, dist):
    import ufoir
    n, na, S = N_DETS, N_ANGLES, args.slices
    ctx = ufoir.Context(dist.local)
    step = float(np.float32(np.pi / na))
    proj = ufoir.ParallelProjector(ctx, step=step, angles_num=na, is_forward=0)
    d_sino, d_vol, noisy = make_inputs(ufoir, ctx, proj, dist.rank, S)
    if args.arithmetic == "fast":
        proj.set(arithmetic=ufoir.ARITH_FAST)

    batch = ufoir.SirtBatch(proj, d_sino, d_vol, relaxation_factor=RELAX)
    for _ in range(max(args.warmup, 0)):
        batch.run(1)
    kernel_ms = batch.profile()     # one eager iteration with CUDA events per launch
    sm_count = ctx.sm_count()

    clocks = ClockSampler(dist.local)
    dist.barrier()
    ctx.synchronize()
    clocks.start()
    l0 = ctx.kernel_launches()
    ctx.timer_begin()
    for _ in range(args.steps):
        batch.run(1)
    ms = ctx.timer_end()
    launches = ctx.kernel_launches() - l0
    clock_info = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)
    value = S * args.steps * dist.world / (ms_max / 1e3)
    fast = None
    if not args.quick and dist.rank == 0:
        fast = fast_section(ufoir, ctx, batch, d_sino, d_vol, args, sm_count, clock_info)
    batch.close()

    e2e, per_job = None, {}
    if not args.quick:
        e2e, per_job = end_to_end(ufoir, ctx, proj, d_sino, d_vol, noisy, dist, S)
    serve = None
    if not args.quick and not args.no_serve and dist.rank == 0:
        serve = serve_section(ufoir, ctx, args.serve_jobs)
    mixed = None
    if not args.quick and dist.rank == 0:
        mixed = mixed_batch_section(ufoir, ctx)
        mixed["small_jobs"] = mixed_batch_section(ufoir, ctx, sizes=SERVE_SIZES[:2], n_jobs=32, max_angles=600,
                                                  seed=MIX_SEED + 1)
    methods = methods_section(ufoir, ctx, cpu=not args.no_cpu_baseline) if args.methods and dist.rank == 0 else None
    models = projector_models_section(ufoir, ctx) if args.methods and dist.rank == 0 else None

    # roofline of the dominant kernel (live CUDA-event durations above)
    peak, peak_kind = measured_peaks()
    fp_bytes = S * (4 * n * n * 2 + 4 * na * n * 2) + 4 * na * n
    bp_bytes = S * (4 * na * n + 4 * n * n * 2) + 4 * n * n
    fp_samples = S * na * n * math.ceil(n / 64) * 64
    bp_samples = S * n * n * na
    dom = "fp" if kernel_ms["fp"] >= kernel_ms["bp"] else "bp"
    dom_bytes = fp_bytes if dom == "fp" else bp_bytes
    achieved = dom_bytes / (kernel_ms[dom] / 1e3) / 1e9
    traffic = ncu_traffic().get({"fp": "fp_tiles_kernel", "bp": "bp_tiles_kernel"}[dom])
    roofline = {"bound": "hbm", "kernel": {"fp": "fp_tiles_kernel", "bp": "bp_tiles_kernel"}[dom],
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "traffic": traffic * S if traffic else None,
                "algorithmic_bytes_per_launch": dom_bytes,
                "note": "compulsory bytes / kernel time against the measured HBM copy rate; the projectors "
                        "are bound by the FMA pipe (packed FP32 interpolation), not HBM, so this fraction is "
                        "small by construction; compute_bound gives the kernel against its measured ceiling"}
    ceiling = ctx.sample_ceiling()
    ceiling_bp = ctx.sample_ceiling_bp()
    fp_rate = fp_samples / (kernel_ms["fp"] / 1e3)
    bp_rate = bp_samples / (kernel_ms["bp"] / 1e3)
    sample_rate = {"fp_samples_per_s": fp_rate, "bp_samples_per_s": bp_rate,
                   "fp_samples_per_launch": fp_samples, "bp_samples_per_launch": bp_samples,
                   "ceiling_samples_per_s": ceiling, "ceiling_bp_samples_per_s": ceiling_bp,
                   "fp_frac": fp_rate / ceiling if ceiling else None,
                   "bp_frac": bp_rate / ceiling_bp if ceiling_bp else None,
                   "bp_frac_of_fp_ceiling": bp_rate / ceiling if ceiling else None,
                   "ceiling": "measured in this run: each projector's exact per-sample sequence from "
                              "shared memory on every SM, no global traffic (ufoir_sample_ceiling for the "
                              "FP, ufoir_sample_ceiling_bp for the BP)",
                   "fp_samples_note": "the FP's samples are every sample of the reference's 64-sample blocks; "
                                      "where all rays of a warp lie outside the image for a chunk of rows (about "
                                      "an eighth of the chunks at this geometry) the samples are border zeros "
                                      "and only the coordinate recurrence runs, so fp_frac can pass 1"}
    dom_rate = fp_rate if dom == "fp" else bp_rate
    dom_ceiling = ceiling if dom == "fp" else ceiling_bp
    roofline["compute_bound"] = {
        "kernel": roofline["kernel"], "achieved": dom_rate, "peak": dom_ceiling, "unit": "samples/s",
        "frac": dom_rate / dom_ceiling if dom_ceiling else None,
        "peak_source": "measured in this run: ufoir_sample_ceiling%s (the kernel's own per-sample "
                       "packed-FP32 sequence from shared memory on every SM)" % ("" if dom == "fp" else "_bp")}
    roofline["fma_pipe_bound"] = fma_pipe_bound(dom, dom_rate, sm_count, clock_info, fast=False)

    if args.arithmetic == "fast":
        roofline["fma_pipe_bound"] = fma_pipe_bound(dom, dom_rate, sm_count, clock_info, fast=True)
    out = {"metric": METRIC, "value": value, "unit": "slice-iters/s", "n_gpus": dist.world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": DATA,
           "config": {**workload_config(S),
                      "step": "one SIRT iteration over all slices, one CUDA graph (pad+transpose, FP, BP)",
                      "l2": "inputs larger than L2 (about 3 GB resident working set per GPU)",
                      "parallelism": "replicas: slices sharded across ranks, no collective",
                      "arithmetic": args.arithmetic},
           "e2e": e2e, "gpu_launches": launches, "clocks": clock_info, "roofline": roofline,
           "kernel_ms": kernel_ms, "sample_rate": sample_rate,
           **{k: v for k, v in per_job.items() if not k.startswith("_")}}
    if serve is not None:
        out["serve"] = serve
    if mixed is not None:
        out["mixed_batch"] = mixed
    if fast is not None:
        out["fast_arithmetic"] = fast
    if methods is not None:
        out["methods"] = methods
    if models is not None:
        out["projector_models"] = models
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline and not args.quick:
        out["cpu_baseline"] = cpu_baseline(noisy[0], per_job.pop("_e2e_slice0", None))
    per_job.pop("_e2e_slice0", None)
    d_sino.close()
    d_vol.close()
    proj.close()
    ctx.close()
    return out if dist.rank == 0 else None


# FP32 operations per pair of samples on the FMA pipe (packed f32x2: one
# lane-op per sample each), the dominant forms: the BP's coordinate (2),
# floor (3), interpolation (4: 1 - t, two products, their sum) and sum (1);
# the FP's inside form: floor (3), interpolation (4), block sum (1) and the
# coordinate recurrence (1). Fast arithmetic: the BP's shift is folded (1)
# and interpolation + sum take 3 (T1 - T0, acc + T0, one fma); the FP's
# interpolation + sum take 3.
FMA_OPS_PER_SAMPLE = {("bp", False): 10, ("fp", False): 9, ("bp", True): 7, ("fp", True): 7}


def fma_pipe_bound(kernel, rate, sm_count, clock_info, fast):
    """The kernel's sample rate against an FMA-pipe bound independent of its
    code: SMs x 128 FP32 lanes x the SM clock sampled during the timed
    region, divided by the FP32 lane-operations one sample needs."""
    mhz = (clock_info or {}).get("sm_mhz") or 2070.0
    lane_ops = sm_count * 128 * mhz * 1e6
    ops = FMA_OPS_PER_SAMPLE[(kernel, fast)]
    peak = lane_ops / ops
    return {"kernel": {"fp": "fp_tiles_kernel", "bp": "bp_tiles_kernel"}[kernel], "achieved": rate, "peak": peak,
            "unit": "samples/s", "frac": rate / peak,
            "model": f"{sm_count} SMs x 128 FP32 lanes x {mhz:.0f} MHz (sampled) = {lane_ops:.3e} lane-ops/s, "
                     f"/ {ops} FP32 lane-ops per sample ({'fast' if fast else 'exact'} arithmetic)"}


def fast_section(ufoir, ctx, exact_batch, d_sino, d_vol, args, sm_count, clock_info):
    """The same batched SIRT workload with the projector's fast interpolation
    arithmetic: slice-iterations/s (CUDA events, the headline's steps), the
    per-kernel times and sample rates with their FMA-pipe bound, and the
    relative L2 distance of 10 iterations from the exact path's (which equals
    the reference arithmetic bit for bit)."""
    n, na, S = N_DETS, N_ANGLES, args.slices
    step = float(np.float32(np.pi / na))
    projf = ufoir.ParallelProjector(ctx, step=step, angles_num=na, is_forward=0, arithmetic=ufoir.ARITH_FAST)
    d_vol_f = ufoir.DeviceArray(ctx, (S, n, n), zero=True)
    fb = ufoir.SirtBatch(projf, d_sino, d_vol_f, relaxation_factor=RELAX)
    for _ in range(max(args.warmup, 0)):
        fb.run(1)
    kms = fb.profile()
    ctx.synchronize()
    ctx.timer_begin()
    for _ in range(args.steps):
        fb.run(1)
    ms = ctx.timer_end()
    fp_samples = S * na * n * math.ceil(n / 64) * 64
    bp_samples = S * n * n * na
    fp_rate = fp_samples / (kms["fp"] / 1e3)
    bp_rate = bp_samples / (kms["bp"] / 1e3)
    fb.reset()
    fb.run(10)
    exact_batch.reset()
    exact_batch.run(10)
    a = d_vol_f.slice(0).download().astype(np.float64)
    b = d_vol.slice(0).download().astype(np.float64)
    out = {"value": S * args.steps / (ms / 1e3), "unit": "slice-iters/s", "ms_per_step": ms / args.steps,
           "kernel_ms": kms, "fp_samples_per_s": fp_rate, "bp_samples_per_s": bp_rate,
           "fma_pipe_bound_bp": fma_pipe_bound("bp", bp_rate, sm_count, clock_info, fast=True),
           "fma_pipe_bound_fp": fma_pipe_bound("fp", fp_rate, sm_count, clock_info, fast=True),
           "rel_l2_vs_exact_10_iterations_slice0": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
           "what": "projector arithmetic \"fast\": T0 + t (T1 - T0) fused into the sum, BP shift folded; "
                   "the headline value above uses the exact (reference) arithmetic"}
    fb.close()
    d_vol_f.close()
    projf.close()
    return out


def end_to_end(ufoir, ctx, proj, d_sino, d_vol, noisy, dist, S):
    """e2e through the public API with host buffers, and one job per launch vs one batched call."""
    n, na = N_DETS, N_ANGLES
    # e2e through the public API with host (pinned) buffers
    h_sino = ctx.pinned_empty((S, na, n))
    h_sino[...] = noisy
    h_vol = ctx.pinned_empty((S, n, n))
    ufoir.sirt(proj, h_sino, h_vol, num_iterations=1, relaxation_factor=RELAX)   # warm
    # three timed calls, the median reported: host copies that follow a long
    # GPU phase were measured at 11-70 GB/s on the GB300 machine against 190-210
    # GB/s back to back, so single calls of the same work vary by a few %
    calls = []
    for _ in range(E2E_CALLS):
        dist.barrier()
        t0 = time.perf_counter()
        ufoir.sirt(proj, h_sino, h_vol, num_iterations=E2E_ITERS, relaxation_factor=RELAX)
        calls.append(dist.max(time.perf_counter() - t0))
    e2e_s = sorted(calls)[len(calls) // 2]
    e2e = {"value": S * E2E_ITERS * dist.world / e2e_s, "unit": "slice-iters/s",
           "h2d_bytes_per_step": int(h_sino.nbytes), "d2h_bytes_per_step": int(h_vol.nbytes),
           "call": f"ufoir_sirt_process(host buffers, {S} slices, num-iterations {E2E_ITERS}), "
                   f"median of {E2E_CALLS} calls",
           "seconds": e2e_s, "seconds_each_call": calls}

    # one job per launch sequence (plain per-job path) vs the batched call, same API, device data;
    # one untimed single-slice call first, as a per-slice pipeline is past its first slice
    jobs = 8
    ufoir.sirt(proj, d_sino.slice(jobs), d_vol.slice(jobs), num_iterations=E2E_ITERS, relaxation_factor=RELAX)
    t0 = time.perf_counter()
    for i in range(jobs):
        ufoir.sirt(proj, d_sino.slice(i), d_vol.slice(i), num_iterations=E2E_ITERS, relaxation_factor=RELAX)
    plain_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ufoir.sirt(proj, d_sino, d_vol, num_iterations=E2E_ITERS, relaxation_factor=RELAX)
    batched_s = time.perf_counter() - t0
    per_job = {"_e2e_slice0": np.array(h_vol[0], copy=True),
               "plain_per_job": {"value": jobs * E2E_ITERS / plain_s, "unit": "slice-iters/s",
                                 "how": f"{jobs} single-slice ufoir_sirt_process calls, {E2E_ITERS} iterations each, "
                       "after one untimed call"},
               "batched_call": {"value": S * E2E_ITERS / batched_s, "unit": "slice-iters/s",
                                "how": f"one ufoir_sirt_process call on {S} slices, {E2E_ITERS} iterations"}}
    return e2e, per_job


def serve_trace(ufoir, ctx, n_jobs):
    """The serve workload as configured: phantom side P in {256, 512, 1024,
    2048} -> grid n in {367, 724, 1448, 2900}; angles U{90..1800}; method in
    {SART, SIRT, ASD-POCS}; iterations U{10..200} (ASD-POCS: outer
    iterations, inner SART num-iterations 10, the plugin default); Poisson
    arrivals at 200 jobs/s. The first n_jobs jobs of the 2000-job trace are
    run, unchanged."""
    from ufoir import synth
    rng = np.random.default_rng(SERVE_SEED)
    methods = (ufoir.METHOD_SART, ufoir.METHOD_SIRT, ufoir.METHOD_ASDPOCS)
    jobs, t, samples = [], 0.0, 0.0
    cache = {}
    for i in range(n_jobs):
        t += float(rng.exponential(1.0 / SERVE_RATE))
        P, n = SERVE_SIZES[int(rng.integers(len(SERVE_SIZES)))]
        na = int(rng.integers(90, 1801))
        method = methods[int(rng.integers(3))]
        iters = int(rng.integers(10, 201))
        step = float(np.float32(np.pi / na))
        if n not in cache:
            cache[n] = synth.ellipse_phantom(n, P, 10, seed=SERVE_SEED + n)
        proj = ufoir.ParallelProjector(ctx, step=step, angles_num=na, is_forward=1)
        clean = np.zeros((na, n), np.float32)
        proj.forward(cache[n], clean)
        proj.close()
        sino, _ = synth.poisson_noise(clean, 1e5, seed=SERVE_SEED + i)
        if method == ufoir.METHOD_ASDPOCS:
            desc = ufoir.job_desc(method, n, na, step, asdpocs=dict(num_iterations=iters))
            per_iter = 10
        else:
            desc = ufoir.job_desc(method, n, na, step, num_iterations=iters)
            per_iter = 1
        samples += iters * per_iter * 2.0 * n * n * na
        jobs.append((t, desc, sino, method, n, na, iters))
    return jobs, samples


def run_serve(ufoir, ctx, jobs, policy, batch_sirt=False):
    """Submits the trace at its arrival times from one host thread and waits for all jobs."""
    with ufoir.Server(ctx, hbm_budget=SERVE_BUDGET, policy=policy, batch_sirt=batch_sirt) as srv:
        t0 = time.perf_counter()
        ids = []
        for (t, desc, sino, *_rest) in jobs:
            delay = t - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ids.append(srv.submit(desc, sino)[0])
        rc = srv.drain(3600000)
        st = srv.stats()
        st["wall_s"] = time.perf_counter() - t0
        st["drain_status"] = rc
    return st


def serve_section(ufoir, ctx, n_jobs):
    """The configured trace's first n_jobs jobs through three policies:
    one_at_a_time (the plain per-job path, arrival order), sjf_one_at_a_time
    (one job at a time, least work first: the ordering of the continuous loop
    without its overlap) and continuous (overlapping jobs on the GPU)."""
    jobs, samples = serve_trace(ufoir, ctx, n_jobs)
    span = jobs[-1][0]
    out = {"trace": {"jobs": len(jobs),
                     "cut": f"the first {len(jobs)} jobs of the configured {SERVE_TRACE_JOBS}-job trace, "
                            "job shapes, methods and iteration counts unchanged",
                     "arrival": f"Poisson, {SERVE_RATE:g} jobs/s (seed {SERVE_SEED})",
                     "offered_window_s": span, "offered_jobs_per_s": len(jobs) / span if span > 0 else None,
                     "offered_samples": samples,
                     "sizes": "phantom P in {256,512,1024,2048} -> grid n in {367,724,1448,2900}",
                     "angles": "U{90..1800}", "methods": "SART / SIRT / ASD-POCS (uniform)",
                     "iterations": "U{10..200}; ASD-POCS: outer iterations, inner SART num-iterations 10",
                     "noise": "Poisson, I0 = 1e5, log",
                     "hbm_budget_bytes": SERVE_BUDGET,
                     "mix": {m: sum(1 for j in jobs if j[3] == k) for m, k in
                             (("sart", ufoir.METHOD_SART), ("sirt", ufoir.METHOD_SIRT),
                              ("asdpocs", ufoir.METHOD_ASDPOCS))}}}
    keys = ("completed", "failed", "p50_latency_ms", "p99_latency_ms", "mean_latency_ms", "max_latency_ms",
            "p50_queue_ms", "p99_queue_ms", "throughput_jobs_per_s", "busy_seconds", "peak_hbm_bytes",
            "peak_active_jobs", "wall_s", "batched_iterations")
    for name, pol, bs in (("one_at_a_time", ufoir.SERVE_ONE_AT_A_TIME, False),
                          ("sjf_one_at_a_time", ufoir.SERVE_SJF_ONE_AT_A_TIME, False),
                          ("continuous", ufoir.SERVE_CONTINUOUS, False),
                          ("continuous_batched_sirt", ufoir.SERVE_CONTINUOUS, True)):
        st = run_serve(ufoir, ctx, jobs, pol, bs)
        out[name] = {k: st[k] for k in keys if k in st}
        out[name]["samples_per_s"] = samples / st["busy_seconds"] if st.get("busy_seconds") else None
    return out


# mixed batch: SIRT jobs of the serve sizes and angle counts
MIX_JOBS = 16
MIX_ITERS = 20
MIX_SEED = 6006


def mixed_batch_section(ufoir, ctx, sizes=None, n_jobs=None, max_angles=1800, seed=None):
    """A mix of one-slice SIRT jobs of uneven size (grid n in {367, 724, 1448,
    2900}, angles U{90..1800}, seeded), each advanced MIX_ITERS iterations,
    all data resident in HBM, three ways on the same GPU:
      per_job_process  ufoir_sirt_process per job (weights, capture and
                       iterations inside each call: the plain per-job path);
      per_job_resident one resident ufoir_sirt_batch per job, set up before
                       the timer, run one job after another;
      mixed_batch      one ufoir_batch of all jobs, set up before the timer
                       (and the same with the autotuner choosing the forward
                       projector's launch shapes).
    Rates are slice-iterations/s and interpolated samples/s (2 n^2 n_a per
    iteration); each member's result equals its per-job result bit for bit
    (tests/test_gpu_batch.py)."""
    from ufoir import synth
    sizes = sizes or SERVE_SIZES
    n_jobs = n_jobs or MIX_JOBS
    seed = seed or MIX_SEED
    rng = np.random.default_rng(seed)
    jobs, cache = [], {}
    for i in range(n_jobs):
        P, n = sizes[int(rng.integers(len(sizes)))]
        na = int(rng.integers(90, max_angles + 1))
        step = float(np.float32(np.pi / na))
        if n not in cache:
            cache[n] = synth.ellipse_phantom(n, P, 10, seed=seed + n)
        proj = ufoir.ParallelProjector(ctx, step=step, angles_num=na, is_forward=1)
        clean = proj.forward(cache[n], np.zeros((na, n), np.float32))
        proj.close()
        sino, _ = synth.poisson_noise(clean, I0, seed=seed + i)
        jobs.append((n, na, step, ufoir.DeviceArray.from_numpy(ctx, sino), ufoir.DeviceArray(ctx, (n, n), zero=True)))
    samples = float(sum(2.0 * n * n * na for n, na, *_ in jobs)) * MIX_ITERS
    slice_iters = n_jobs * MIX_ITERS
    out = {"workload": f"{n_jobs} one-slice SIRT jobs, grid n in {{{','.join(str(n) for _, n in sizes)}}}, angles "
                       f"U{{90..{max_angles}}} (seed {seed}), {MIX_ITERS} iterations each, data resident in HBM",
           "jobs": [[n, na] for n, na, *_ in jobs], "samples": samples}

    def rate(sec):
        return {"seconds": sec, "slice_iters_per_s": slice_iters / sec, "samples_per_s": samples / sec}

    projs = [ufoir.ParallelProjector(ctx, step=st, angles_num=na, is_forward=0) for n, na, st, *_ in jobs]
    # per-job process calls (one warm pass of one iteration each first)
    for pj, (n, na, st, ds, dv) in zip(projs, jobs):
        ufoir.sirt(pj, ds, dv, num_iterations=1)
    ctx.synchronize()
    t0 = time.perf_counter()
    for pj, (n, na, st, ds, dv) in zip(projs, jobs):
        ufoir.sirt(pj, ds, dv, num_iterations=MIX_ITERS)
    ctx.synchronize()
    out["per_job_process"] = rate(time.perf_counter() - t0)
    # per-job resident batches
    sb = [ufoir.SirtBatch(pj, ds, dv, relaxation_factor=RELAX) for pj, (n, na, st, ds, dv) in zip(projs, jobs)]
    for b in sb:
        b.run(1)
    ctx.synchronize()
    ctx.timer_begin()
    for b in sb:
        b.run(MIX_ITERS)
    out["per_job_resident"] = rate(ctx.timer_end() / 1e3)
    for b in sb:
        b.close()
    # the mixed batch, fixed rules and autotuned
    for name, tune in (("mixed_batch", False), ("mixed_batch_autotuned", True)):
        ctx.set_autotune(tune)
        t0 = time.perf_counter()
        b = ufoir.Batch(ctx, [(ds, dv, dict(step=st, relaxation_factor=RELAX)) for n, na, st, ds, dv in jobs])
        setup_s = time.perf_counter() - t0
        b.run(1)
        ctx.synchronize()
        ctx.timer_begin()
        b.run(MIX_ITERS)
        r = rate(ctx.timer_end() / 1e3)
        r["setup_seconds"] = setup_s
        r["launches_per_iteration"], r["fp_launch_shapes"] = b.launches()
        b.close()
        out[name] = r
    ctx.set_autotune(ufoir.AUTOTUNE_AUTO)      # the context default
    out["speedup_vs_per_job_resident"] = out["mixed_batch"]["slice_iters_per_s"] / out["per_job_resident"]["slice_iters_per_s"]
    out["speedup_autotuned_vs_per_job_resident"] = (out["mixed_batch_autotuned"]["slice_iters_per_s"] /
                                                    out["per_job_resident"]["slice_iters_per_s"])
    for pj in projs:
        pj.close()
    for n, na, st, ds, dv in jobs:
        ds.close()
        dv.close()
    return out


# the other configured workloads:
# (name, method, n_dets, n_angles, phantom side, phantom kind, I0, slices, params)
METHOD_CASES = (
    ("C1 SART 367^2 x 180 angles, 10 iterations", "sart", 367, 180, 256, "ellipses", None, 1,
     dict(num_iterations=10)),
    ("C2 SIRT one slice 1448^2 x 1200 angles, 10 iterations", "sirt", 1448, 1200, 1024, "ellipses", 1e5, 1,
     dict(num_iterations=10)),
    ("C3a ASD-POCS 2900^2 x 90 angles, 1 outer iteration (inner SART 10)", "asdpocs", 2900, 90, 2048, "polygons",
     1e4, 1, dict(num_iterations=1)),
    ("C3b ASD-POCS 2900^2 x 360 angles, 1 outer iteration (inner SART 10)", "asdpocs", 2900, 360, 2048,
     "polygons", 1e4, 1, dict(num_iterations=1)),
    ("C4 SBTV 1448^2 x 720 angles, 16 slices (one batch of the 512), 1 outer iteration", "sbtv", 1448, 720, 1024,
     "ellipses", 1e5, 16, {"num_iterations": 1, "lambda": 0.05, "mu": 1.0}),
)


# methods whose call on one slice the oracle port runs on the host cores: SART
# and ASD-POCS in seconds, 10 SIRT iterations at 1448^2 x 1200 in about 15 s,
# one SBTV outer iteration at 1448^2 x 720 (about 60 FP + BP applications) in
# about a minute
METHOD_CPU = ("sart", "sirt", "asdpocs", "sbtv")


def method_cpu_baseline(method, n, na, step, sino, kw):
    """The reference's CPU path on the first slice of a method workload, the
    same call as the GPU's, on all host cores: its OpenCL kernels compiled for
    the host (oracle/_ref) driven by the oracle's host loop (the C port where
    the kernel sources are absent)."""
    pyoracle, threads, which = _cpu_oracle()
    p = pyoracle.projector(n, na, step)
    sino = np.ascontiguousarray(sino, np.float32)
    t0 = time.perf_counter()
    if method == "sart":
        pyoracle.sart(p, sino, kw["num_iterations"], 0.25, which=which)
    elif method == "sirt":
        pyoracle.sirt(p, sino, kw["num_iterations"], 0.25, which=which)
    elif method == "sbtv":
        pyoracle.sbtv(p, sino, pyoracle.sbtv_params(num_iterations=kw["num_iterations"], lambda_=kw["lambda"],
                                                    mu=kw["mu"], norm_mode=pyoracle.NORM_FP64), which=which)
    else:
        pyoracle.asdpocs(p, sino, pyoracle.asdpocs_params(num_iterations=kw["num_iterations"],
                                                         norm_mode=pyoracle.NORM_FP64), which=which)
    dt = time.perf_counter() - t0
    return {"ms_per_call": dt * 1e3, "cores": threads, "kind": _cpu_kind(which), "sample": "the whole call, slice 0"}


def methods_section(ufoir, ctx, cpu=True):
    """One call of each other configured method workload on one slice,
    resident in HBM: the call time (after one untimed call) and its rate;
    with cpu, the reference's CPU path on the same call beside it."""
    from ufoir import synth
    out = []
    for name, method, n, na, P, kind, i0, S, kw in METHOD_CASES:
        step = float(np.float32(np.pi / na))
        vols = np.stack([synth.phantom_for(n, P, kind, seed=7000 + n + na + i) for i in range(S)])
        proj = ufoir.ParallelProjector(ctx, step=step, angles_num=na, is_forward=1)
        sino = proj.forward(vols, np.zeros((S, na, n), np.float32))
        proj.close()
        if i0:
            for i in range(S):
                sino[i], _ = synth.poisson_noise(sino[i], i0, seed=8000 + n + na + i)
        d_sino = ufoir.DeviceArray.from_numpy(ctx, sino.astype(np.float32))
        d_vol = ufoir.DeviceArray(ctx, (S, n, n), zero=True)
        proj = ufoir.ParallelProjector(ctx, step=step, angles_num=na, is_forward=0)
        fn = getattr(ufoir, method)
        fn(proj, d_sino, d_vol, **kw)
        ctx.synchronize()
        ctx.timer_begin()
        fn(proj, d_sino, d_vol, **kw)
        ms = ctx.timer_end()
        iters = kw["num_iterations"]
        row = {"workload": name, "slices": S, "ms_per_call": ms, "ms_per_iteration": ms / iters,
               "ms_per_slice_iteration": ms / iters / S, "samples_per_slice_iteration_fp_bp": 2.0 * n * n * na}
        if cpu and method in METHOD_CPU:
            row["cpu_baseline"] = method_cpu_baseline(method, n, na, np.float32(step), sino[0], kw)
        out.append(row)
        proj.close()
        d_sino.close()
        d_vol.close()
    return out


def projector_models_section(ufoir, ctx, n=1448, na=1200, reps=5):
    """Forward and backward projection of one resident slice (n^2 grid, na
    angles) under each projector model: the mean time of one call over reps
    calls, after one untimed call, and its rate in pixel-angle pairs per second."""
    from ufoir import synth
    step = float(np.float32(np.pi / na))
    vol = synth.phantom_for(n, 1024, "ellipses", seed=9100)[None]
    d_vol = ufoir.DeviceArray.from_numpy(ctx, vol.astype(np.float32))
    d_sino = ufoir.DeviceArray(ctx, (1, na, n), zero=True)
    out = {"workload": f"one slice, {n}^2 grid, {na} angles, {n} bins, resident in HBM"}
    for model in ("joseph", "siddon"):
        row = {}
        for direction in ("forward", "backward"):
            proj = ufoir.ParallelProjector(ctx, step=step, angles_num=na, model=model,
                                           is_forward=1 if direction == "forward" else 0)
            call = getattr(proj, direction)
            call(d_vol, d_sino)
            ctx.synchronize()
            ctx.timer_begin()
            for _ in range(reps):
                call(d_vol, d_sino)
            ms = ctx.timer_end() / reps
            row[direction] = {"ms": ms, "pixel_angles_per_s": n * n * na / (ms * 1e-3)}
            proj.close()
        out[model] = row
    d_vol.close()
    d_sino.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ufoir", choices=["ufoir", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU baselines (the headline's and, with --methods, each method's)")
    ap.add_argument("--slices", type=int, default=SLICES, help="slices per GPU (64 = the headline workload)")
    ap.add_argument("--quick", action="store_true",
                    help="only the resident timed steps (skip e2e, per-job comparison, serve trace, CPU baseline)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serve trace")
    ap.add_argument("--serve-jobs", type=int, default=SERVE_JOBS,
                    help="jobs of the configured serve trace to run (its first ones)")
    ap.add_argument("--methods", action="store_true",
                    help="also time one call of each other configured method workload (C1, C2, C3a/b, C4)")
    ap.add_argument("--projector-models", action="store_true",
                    help="only time the Joseph and Siddon projectors on one resident 1448^2 x 1200 slice")
    ap.add_argument("--arithmetic", default="exact", choices=["exact", "fast"],
                    help="interpolation arithmetic of the headline's projector (exact = the reference's rounding)")
    ap.add_argument("--mixed-batch", action="store_true",
                    help="only the mixed-batch comparison (per-job vs one batch of uneven SIRT jobs)")
    args = ap.parse_args()
    if args.projector_models:
        import ufoir
        ctx = ufoir.Context(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps(projector_models_section(ufoir, ctx)), flush=True)
        ctx.close()
        return
    if args.mixed_batch:
        import ufoir
        ctx = ufoir.Context(int(os.environ.get("LOCAL_RANK", "0")))
        out = mixed_batch_section(ufoir, ctx)
        out["small_jobs"] = mixed_batch_section(ufoir, ctx, sizes=SERVE_SIZES[:2], n_jobs=32, max_angles=600,
                                                seed=MIX_SEED + 1)
        print(json.dumps(out), flush=True)
        ctx.close()
        return
    dist = Dist()
    try:
        out = run_reference(args, dist) if args.impl == "reference" else run_ufoir(args, dist)
        if out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
