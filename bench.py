"""Benchmark: distinct finite roots per second on one GB300.

Workload (one "step" = one round of the tracker): 65,536 paths on one generic
precision-point task (seed 1: P_k and Pc_k uniform in the unit disk, crank rotations
on the unit circle), start mechanisms from complex normal link/pivot values, a random
unit-modulus gamma, sharpening to 1e-12 at t = 1 in FP64, canonical cognates, finite-root check
(|Z0|/|Z| >= 1e-8), per-root residual, and duplicate removal in a root collection.
A root counts when its path succeeded, it is finite, its row-scaled residual is
<= 1e-10, and it is not a duplicate. Synthetic inputs: the reference ships no
benchmark data; tasks and starts are seeded.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--paths P] [--impl ours|reference]

value    distinct finite roots / second over K rounds (steps) of the chosen configuration run
         through frg_track_rounds with `--depth` rounds in flight (inputs resident in HBM, CUDA
         events on the launching streams); the chosen configuration is mixed precision (FP32
         team kernel with double-float refinement, FP64 for ill-conditioned steps and for
         finishing every root). Plain FP64 on the same seeds, pipelined the same way, gives
         `plain_fp64`, the speed-up and the recall
e2e      the same through the public C ABI with pinned host buffers: the task upload, tracking,
         the copy of roots/codes/residuals back and the host duplicate merge of every round
--impl reference  times the reference algorithm's CPU implementation (the C
         restatement in oracle/, the reference's own sources cannot be built on the GPU
         host) on all host cores, on a bounded sample of the same workload.
Multi-GPU: paths are independent; N ranks each run the workload on their own GPU with
their own seeds (weak scaling) and the job value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "distinct finite roots/sec at >=99.5% recall, residual <=1e-10: chosen vs plain FP64"
UNIT = "roots/s"
RESID_MAX = 1e-10
INF_TOL = 1e-8
TASK_SEED = 1


def workload_config(frg, precision):
    return frg.default_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=INF_TOL,
                              precision=precision)


def count_distinct(frg, roots, codes, resid):
    good = (codes == 0) & (resid <= RESID_MAX)
    c = np.where(good, 0, np.where(codes == 0, 5, codes)).astype(np.int32)
    coll = frg.Collection(1e-6)
    out = coll.merge(roots, c)
    return len(coll), out


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------ FP64 peak
FMA_PEAK_SRC = r"""
template <typename T>
__global__ void fma_peak(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * T(1e-9), x1 = x0 + T(1e-3), x2 = x0 + T(2e-3), x3 = x0 + T(3e-3);
  T x4 = x0 + T(4e-3), x5 = x0 + T(5e-3), x6 = x0 + T(6e-3), x7 = x0 + T(7e-3);
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  if (x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7 == T(123)) out[0] = x0;
}
"""


def measure_fma_peaks():
    """Dense FP64 and FP32 FMA throughput of this GPU (TFLOP/s), measured with
    8 independent FMA chains per thread. MEASURED_PEAKS.json records only HBM and
    bf16 tensor peaks, so the FMA-pipe denominators are measured here."""
    from finite_root_generation_gb300 import build as frg_build

    import ctypes
    so = os.path.join(frg_build.BUILD, "fma_peak2.so")
    os.makedirs(frg_build.BUILD, exist_ok=True)
    src = os.path.join(frg_build.BUILD, "fma_peak.cu")
    if not os.path.exists(so):
        with open(src, "w") as f:
            f.write(FMA_PEAK_SRC)
            f.write(r"""
#include <cuda_runtime.h>
template <typename T>
static float run(int blocks, int threads, int iters) {
  T* out; cudaMalloc(&out, 8);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  fma_peak<T><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e0);
  fma_peak<T><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e1); cudaEventSynchronize(e1);
  float ms; cudaEventElapsedTime(&ms, e0, e1);
  cudaFree(out); cudaEventDestroy(e0); cudaEventDestroy(e1);
  return ms;
}
extern "C" float run_fma_peak(int fp64, int blocks, int threads, int iters) {
  return fp64 ? run<double>(blocks, threads, iters) : run<float>(blocks, threads, iters);
}
""")
        subprocess.run([frg_build.nvcc(), *frg_build.ARCH, "-O3", "-Xcompiler", "-fPIC", "-shared", src, "-o", so],
                       check=True)
    lib = ctypes.CDLL(so)
    lib.run_fma_peak.restype = ctypes.c_float
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    out = {}
    for name, fp64, iters in (("fp64", 1, 4096), ("fp32", 0, 65536)):
        blocks, threads = sms * 8, 256
        ms = lib.run_fma_peak(fp64, blocks, threads, iters)
        out[name] = 2.0 * 8 * iters * blocks * threads / (ms * 1e-3) / 1e12
    return out


# ------------------------------------------------------------------ algorithmic work
def _gen_counts():
    import re
    gen = open(os.path.join(ROOT, "finite_root_generation_gb300", "csrc", "frg_system_gen.cuh")).read()
    return tuple(int(re.search(rf"#define FRG_GEN_{k} (\d+)", gen).group(1)) for k in ("CMUL", "CADD", "SMUL"))


def flops_per_solve():
    """Algorithmic FLOPs of one linear-system step of the team kernels, counting
    complex mul = 6, complex add = 2, real x complex = 2, complex FMA = 8, complex
    reciprocal = 12; zeros are not counted and work repeated across lanes counts once:
      params   q(t), dq/dt of 30 parameters                          30 x 24
      system   7 groups of generated code (FRG_GEN_* counts) + 11 reciprocals
      scale    21 group rows x 18 entries + the u row (23)           x 2
      group    7 x [1 reciprocal + 2 rows x (1 cmul + 17 cfma)]
      fold     7 x 2 patch rows x (1 + 17) cmul + 7 x 2 x 17 complex adds
      LU16     sum_k (15-k) x (cmul + (16-k) cfma) + 16 reciprocals
      backsub  sum_k (6 + 8 k); U recovery 7 x (16 cfma + 1 cmul)
      norm     23 x (cmul + |.|^2)
    A Newton iteration has the same structure (the t-selector replaces the velocity
    patch), so both kinds of step count the same."""
    cm, ca, sm = _gen_counts()
    f = 30 * 24
    f += 7 * (6 * cm + 2 * ca + 2 * sm) + 11 * 12
    f += (21 * 18 + 23) * 2
    f += 7 * (12 + 2 * (6 + 17 * 8))
    f += 7 * 2 * 18 * 6 + 7 * 2 * 17 * 2
    f += sum((15 - k) * (6 + 8 * (16 - k)) for k in range(16)) + 16 * 12
    f += sum(6 + 8 * k for k in range(16)) + 7 * (16 * 8 + 6)
    f += 23 * (6 + 4)
    return f


# ---------------------------------------------------------------------- our impl
def _chosen_overrides():
    """The chosen configuration on top of the workload's: mixed precision, the FP32
    stage also running the endgame and sharpening (double-float refinement), FP64 for
    steps whose condition estimate exceeds 1e5 and for finishing every root, and at most
    10,000 FP64 solves per path (a path still going after that ends as a step-limit
    failure; such paths are crawling near a singularity and set the FP64 tail)."""
    return dict(mixed_rounds=1, lo_endgame=1, cond_switch=1e5, lo_points=1, fp64_budget=10000)


def _round_sets(roots, codes, resid, n, k):
    from finite_root_generation_gb300.metrics import distinct_roots
    R = roots.cpu().numpy().view(np.complex128)
    C = codes.cpu().numpy()
    E = resid.cpu().numpy()
    return [distinct_roots(R[i * n:(i + 1) * n], C[i * n:(i + 1) * n], E[i * n:(i + 1) * n], RESID_MAX)
            for i in range(k)]


def workload_tasks(precision_point_task, ntasks, n):
    """The tasks of a round and their path counts: one generic task (seed 1, points in
    the unit disk) or, for ntasks > 1, tasks from seeds 0..ntasks-1 alternating points in
    the unit disk and points along a random smooth closed curve (the batched uneven
    workload), n paths split evenly."""
    if ntasks <= 1:
        return precision_point_task(TASK_SEED, "disk"), [n]
    if n % ntasks:
        raise SystemExit("--paths must be a multiple of --tasks")
    tasks = np.stack([precision_point_task(i, "disk" if i % 2 == 0 else "curve") for i in range(ntasks)])
    return tasks, [n // ntasks] * ntasks


def _timed_rounds(torch, tracker, d_fpm, ppt, seeds, outs, depth, world):
    """K rounds through frg_track_rounds (device buffers, `depth` rounds in flight),
    bracketed by a barrier and a synchronize on both sides. The library times the
    span with CUDA events on its launching streams (first launch to the last round's
    end); torch events on the current stream bracket the call as a cross-check."""
    roots, codes, resid = outs
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    st = tracker.track_rounds(d_fpm, ppt, seeds, roots, codes, resid=resid, depth=depth)
    ev1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    return st, ev0.elapsed_time(ev1)


def run_ours(args, rank, world):
    import torch

    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300 import build as frg_build
    from finite_root_generation_gb300.metrics import distinct_roots, recall
    from finite_root_generation_gb300.tasks import precision_point_task

    frg_build.build()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    task, ppt = workload_tasks(precision_point_task, args.tasks, args.paths)
    n, k, depth = args.paths, args.steps, args.depth
    chosen_cfg = workload_config(frg, frg.PREC_MIXED)
    for key, v in _chosen_overrides().items():
        setattr(chosen_cfg, key, v)
    chosen = frg.Tracker(chosen_cfg, device=dev)
    plain = frg.Tracker(workload_config(frg, frg.PREC_FP64), device=dev)
    d_fpm = torch.from_numpy(task.view(np.float64).copy()).cuda()
    nbuf = max(k, args.warmup, 1) * n
    outs = (torch.empty((nbuf, 42), dtype=torch.float64, device="cuda"),
            torch.empty(nbuf, dtype=torch.int32, device="cuda"),
            torch.empty(nbuf, dtype=torch.float64, device="cuda"))

    def seed_of(step):
        return 1000003 * (rank + 1) + step

    seeds = [seed_of(i) for i in range(k)]
    # warm-up: W rounds of the chosen configuration and one of the plain one
    warm = [seed_of(-1 - i) for i in range(args.warmup)]
    chosen.track_rounds(d_fpm, ppt, warm, outs[0][: len(warm) * n], outs[1][: len(warm) * n],
                        resid=outs[2][: len(warm) * n], depth=depth)
    plain.track_rounds(d_fpm, [min(c, max(1, 8192 // len(ppt))) for c in ppt], warm[:1], outs[0], outs[1],
                       resid=outs[2], depth=1)
    torch.cuda.synchronize()

    # ---- chosen configuration, inputs resident in HBM (value) ----
    c_outs = tuple(o[: k * n] for o in outs)
    with ClockSampler(dev) as clk:
        c_st, c_torch_ms = _timed_rounds(torch, chosen, d_fpm, ppt, seeds, c_outs, depth, world)
    clocks = clk.summary()
    c_sets = _round_sets(*c_outs, n, k)
    # ---- plain FP64 on the same seeds, pipelined the same way (ratio and recall) ----
    kp = max(1, min(args.plain_steps, k))
    p_st, _ = _timed_rounds(torch, plain, d_fpm, ppt, seeds[:kp], tuple(o[: kp * n] for o in outs), depth, world)
    p_sets = _round_sets(*(o[: kp * n] for o in outs), n, kp)
    rec = [recall(p_sets[i], c_sets[i]) for i in range(kp)]

    # ---- end to end through the C ABI with pinned host buffers (e2e): per round the
    #      task upload, tracking, the copy of roots/codes/residuals back, and the host
    #      duplicate merge of every round ----
    h_roots = torch.empty((k * n, 42), dtype=torch.float64, pin_memory=True)
    h_codes = torch.empty(k * n, dtype=torch.int32, pin_memory=True)
    h_resid = torch.empty(k * n, dtype=torch.float64, pin_memory=True)
    hr, hc, he = h_roots.numpy(), h_codes.numpy(), h_resid.numpy()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    chosen.track_rounds(task, ppt, seeds, hr, hc, resid=he, depth=depth)
    R = hr.view(np.complex128)
    e2e_distinct = sum(len(distinct_roots(R[i * n:(i + 1) * n], hc[i * n:(i + 1) * n], he[i * n:(i + 1) * n],
                                          RESID_MAX)) for i in range(k))
    e2e_s = time.perf_counter() - t0

    track_ms = c_st["track_ms"]
    p_ms = p_st["track_ms"]
    distinct = sum(len(d) for d in c_sets)
    p_distinct = sum(len(d) for d in p_sets)
    t = torch.tensor([track_ms, e2e_s, distinct, e2e_distinct, p_ms, p_distinct], dtype=torch.float64)
    if world > 1:
        tmax, tsum = t.clone().cuda(), t.clone().cuda()
        torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(tsum, op=torch.distributed.ReduceOp.SUM)
        track_ms, e2e_s, p_ms = float(tmax[0]), float(tmax[1]), float(tmax[4])
        distinct, e2e_distinct, p_distinct = float(tsum[2]), float(tsum[3]), float(tsum[5])
    chosen_rounds = chosen.config.mixed_rounds
    chosen.close()
    plain.close()
    if rank != 0:
        return None

    value = distinct / (track_ms * 1e-3)
    value_plain = p_distinct / (p_ms * 1e-3)
    e2e = e2e_distinct / e2e_s
    # roofline of each kernel: algorithmic FLOPs of its launches / their CUDA-event time
    peaks = measure_fma_peaks()
    fps = flops_per_solve()
    solves = c_st["ivp_solves"] + c_st["newton_iters"]
    fp64_solves = c_st["fp64_solves"]
    fp32_solves = solves - fp64_solves
    ms32 = c_st["stage_ms"][0] / k
    ms64 = c_st["stage_ms"][1] / k
    kernels = {
        "team_kernel<MODE_LO, float> (FP32 stage)": {
            "bound": "fp32", "achieved": fp32_solves / k * fps / (ms32 * 1e-3) / 1e12, "peak": peaks["fp32"],
            "ms_per_launch": ms32, "solves_per_launch": fp32_solves / k},
        "team_kernel<MODE_RESUME, double> (FP64 stage)": {
            "bound": "fp64", "achieved": fp64_solves / k * fps / (ms64 * 1e-3) / 1e12, "peak": peaks["fp64"],
            "ms_per_launch": ms64, "solves_per_launch": fp64_solves / k},
    }
    for v in kernels.values():
        v["frac"] = v["achieved"] / v["peak"]
    dom_name = max(kernels, key=lambda kk: kernels[kk]["ms_per_launch"])
    dom = kernels[dom_name]
    p_solves = (p_st["ivp_solves"] + p_st["newton_iters"]) / kp
    p_ms_round = p_st["stage_ms"][1] / kp
    plain_roof = p_solves * fps / (p_ms_round * 1e-3) / 1e12
    h2d = len(ppt) * (16 * 30 + 16 + 8) + 8  # task parameters, gammas, path offsets
    d2h = n * (16 * 21 + 4 + 8)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": k,
        "warmup": args.warmup, "ms_per_step": round(track_ms / k, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded task and start mechanisms)",
        "config": {"workload": (f"Stephenson II FRG rounds of {n} paths on 1 generic complex precision-point task "
                                f"(seed {TASK_SEED})" if len(ppt) == 1 else
                                f"Stephenson II FRG rounds of {n} paths over {len(ppt)} tasks (seeds 0..{len(ppt) - 1}, "
                                "points in the unit disk / along a random closed curve, alternating)")
                               + ", complex-normal start mechanisms, random unit gamma per round; "
                               "FP64 sharpening check, canonical cognates, finite + residual <= 1e-10 checks, "
                               "duplicate removal",
                   "paths_per_step": n, "rounds_in_flight": depth,
                   "chosen": "mixed precision: FP32 team kernel (double-float points and refinement, endgame and "
                             "sharpening included), FP64 team kernel for steps with condition estimate > 1e5 "
                             "(at most 10,000 FP64 solves per path) and for finishing",
                   "l2": f"not flushed: per-round state (start values 816 B, hand-off record 1.2 KB, outputs "
                         f"348 B per path: ~{n * 2364 / 1e6:.0f} MB per round, {depth} rounds in flight) exceeds "
                         "the 129 MB L2",
                   "parallelism": f"replicas x{world}"},
        "plain_fp64": {"value": round(value_plain, 2), "unit": UNIT, "steps": kp,
                       "ms_per_step": round(p_ms / kp, 3),
                       "roofline_frac_fp64": round(plain_roof / peaks["fp64"], 4)},
        "speedup_vs_plain_fp64": round(value / value_plain, 3),
        "recall_vs_plain_fp64": round(min(rec), 5),
        "distinct_roots_per_step": distinct / k / world,
        "torch_event_ms": round(c_torch_ms, 1),
        "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"kernel": dom_name, "bound": dom["bound"], "achieved": round(dom["achieved"], 4),
                     "peak": round(dom["peak"], 4), "unit": "TFLOP/s", "frac": round(dom["frac"], 4),
                     "traffic": None,
                     "peak_source": "FMA peaks measured live by bench.py (MEASURED_PEAKS.json has no FP32/FP64 "
                                    "vector figure)",
                     "flops_per_solve": fps,
                     "kernels": {kk: {x: (round(y, 4) if isinstance(y, float) else y) for x, y in v.items()}
                                 for kk, v in kernels.items()}},
        # per round: start values, FP32 and double-float parameter copies, then per mixed
        # round one FP32-stage and one FP64-stage tracking kernel
        "gpu_launches": (3 + 2 * max(1, chosen_rounds)) * k,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    return line


# ------------------------------------------------------------------- CPU baseline
def cpu_baseline(args, sample_paths=None):
    """The oracle (C restatement of the reference tracker) on all host cores, on the
    first paths of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300.tasks import precision_point_task

    oracle.build()
    o = oracle.Oracle()
    cores = os.cpu_count() or 1
    n = sample_paths or args.cpu_sample
    task = precision_point_task(TASK_SEED, "disk")
    cfg = o.config(start_dist=1)
    # random gamma of task 0 as the library draws it (stream 2^64-1, index 0)
    phi = 2 * np.pi * o.uniform01(1000003, 2**64 - 1, 0)
    gamma = complex(np.cos(phi), np.sin(phi))
    t0 = time.perf_counter()
    roots, codes, work, yf = o.homotopy_batch(task, gamma, 1000003, np.arange(n), cfg=cfg, nthreads=cores,
                                             want_yfinal=True)
    dt = time.perf_counter() - t0
    # finite check and residual as in the device path
    zmax = np.max(np.abs(yf[:, :21]), axis=1)
    inf = (codes == 0) & (np.abs(yf[:, 21]) < INF_TOL * zmax)
    codes = np.where(inf, 7, codes).astype(np.int32)
    coll = frg.Collection(1e-6)
    coll.merge(roots, codes)
    d = len(coll)
    return {"value": round(d / dt, 3), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {n} paths of the workload (seed 1000003), {dt:.1f} s on {cores} threads"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    for _ in range(max(1, args.warmup)):
        cb = cpu_baseline(args, sample_paths=args.cpu_sample)
    t0 = time.perf_counter()
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline(args, sample_paths=args.cpu_sample)["value"])
    dt = time.perf_counter() - t0
    v = float(np.mean(vals))
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded tasks and starts)",
            "config": {"workload": f"Stephenson II FRG round on one precision-point task (seed {TASK_SEED}), "
                                   "complex-normal starts, random gamma, FP64 + sharpening + dedup",
                       "paths_per_step": args.cpu_sample, "precision": "plain FP64",
                       "parallelism": "host threads"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cb["cores"], "kind": "port",
                             "sample": cb["sample"] + "; the reference's own sources are not present on the GPU "
                                       "host, so its C restatement (oracle/frg_oracle.c) is timed"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--paths", type=int, default=65536)
    ap.add_argument("--cpu-sample", type=int, default=8192)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--depth", type=int, default=4, help="rounds in flight")
    ap.add_argument("--tasks", type=int, default=1, help="tasks per round (>1: the batched uneven workload)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "reference":
            if rank != 0:
                return
        else:
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
            dist.init_process_group("nccl")
    line = run_reference(args, rank, world) if args.impl == "reference" else run_ours(args, rank, world)
    if line is not None:
        print(json.dumps(line))
    if world > 1 and args.impl != "reference":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
