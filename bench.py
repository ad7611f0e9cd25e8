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

value    distinct finite roots / second of device tracking time (inputs resident in HBM) of the
         chosen configuration: mixed precision (FP32 team stage, FP64 endgame and sharpening);
         plain FP64 on the same seeds gives `plain_fp64`, the speed-up and the recall
e2e      the same through the public C ABI with host buffers: per step the task upload,
         tracking, the copy of roots/codes/residuals back and the host duplicate merge
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
def _timed_steps(torch, tracker, n, seeds, d_fpm, outs, flush, world):
    """Run one step per seed, step i writing into outs[i] (device buffers), timed as one
    region with CUDA events bracketed by a barrier and a synchronize on both sides.
    L2 is flushed (a 256 MB write) before every step. Returns (ms, per-step stats)."""
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    stats = []
    for sd, (roots, codes, resid) in zip(seeds, outs):
        flush.zero_()
        stats.append(tracker.track_into(d_fpm, [n], sd, roots, codes, resid=resid))
    ev1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    return ev0.elapsed_time(ev1), stats


def _distinct_sets(outs):
    from finite_root_generation_gb300.metrics import distinct_roots
    return [distinct_roots(r.cpu().numpy().view(np.complex128), c.cpu().numpy(), e.cpu().numpy(), RESID_MAX)
            for r, c, e in outs]


def run_ours(args, rank, world):
    import torch

    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300 import build as frg_build
    from finite_root_generation_gb300.metrics import distinct_roots, recall
    from finite_root_generation_gb300.tasks import precision_point_task

    frg_build.build()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    task = precision_point_task(TASK_SEED, "disk")
    n = args.paths
    chosen = frg.Tracker(workload_config(frg, frg.PREC_MIXED), device=dev)
    plain = frg.Tracker(workload_config(frg, frg.PREC_FP64), device=dev)
    d_fpm = torch.from_numpy(task.view(np.float64).copy()).cuda()

    def out_bufs(k):
        return [(torch.empty((n, 42), dtype=torch.float64, device="cuda"),
                 torch.empty(n, dtype=torch.int32, device="cuda"),
                 torch.empty(n, dtype=torch.float64, device="cuda")) for _ in range(k)]

    outs = out_bufs(args.steps)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def seed_of(step):
        return 1000003 * (rank + 1) + step

    for w in range(args.warmup):
        chosen.track_into(d_fpm, [n], seed_of(-1 - w), *outs[0][:2], resid=outs[0][2])
    plain.track_into(d_fpm, [min(n, 8192)], seed_of(-1), *outs[0][:2], resid=outs[0][2])
    torch.cuda.synchronize()

    # ---- chosen configuration, inputs resident in HBM (value) ----
    seeds = [seed_of(k) for k in range(args.steps)]
    with ClockSampler(dev) as clk:
        track_ms, c_stats = _timed_steps(torch, chosen, n, seeds, d_fpm, outs, flush, world)
    clocks = clk.summary()
    c_sets = _distinct_sets(outs)
    # ---- plain FP64 on the same seeds (ratio and recall) ----
    p_seeds = seeds[: max(1, args.plain_steps)]
    p_outs = outs[: len(p_seeds)]
    p_ms, p_stats = _timed_steps(torch, plain, n, p_seeds, d_fpm, p_outs, flush, world)
    p_sets = _distinct_sets(p_outs)
    rec = [recall(p_sets[i], c_sets[i]) for i in range(len(p_seeds))]

    # ---- end to end through the C ABI with host buffers (e2e) ----
    h_roots = np.zeros((n, 21), np.complex128)
    h_codes = np.zeros(n, np.int32)
    h_resid = np.zeros(n, np.float64)
    e2e_distinct = 0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for sd in seeds:
        chosen.track_into(task, [n], sd, h_roots, h_codes, resid=h_resid)
        e2e_distinct += len(distinct_roots(h_roots, h_codes, h_resid, RESID_MAX))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

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
    # roofline of each kernel: algorithmic FLOPs per launch / launch time
    peaks = measure_fma_peaks()
    fps = flops_per_solve()
    k = args.steps
    solves = sum(st["ivp_solves"] + st["newton_iters"] for st in c_stats) / k
    fp64_solves = sum(st["fp64_solves"] for st in c_stats) / k
    fp32_solves = solves - fp64_solves
    ms32 = sum(st["stage_ms"][0] for st in c_stats) / k
    ms64 = sum(st["stage_ms"][1] for st in c_stats) / k
    kernels = {
        "team_kernel<MODE_LO, float> (FP32 stage)": {
            "bound": "fp32", "achieved": fp32_solves * fps / (ms32 * 1e-3) / 1e12, "peak": peaks["fp32"],
            "ms_per_launch": ms32, "solves_per_launch": fp32_solves},
        "team_kernel<MODE_RESUME, double> (FP64 stage)": {
            "bound": "fp64", "achieved": fp64_solves * fps / (ms64 * 1e-3) / 1e12, "peak": peaks["fp64"],
            "ms_per_launch": ms64, "solves_per_launch": fp64_solves},
    }
    for v in kernels.values():
        v["frac"] = v["achieved"] / v["peak"]
    dom_name = max(kernels, key=lambda kk: kernels[kk]["ms_per_launch"])
    dom = kernels[dom_name]
    p_solves = sum(st["ivp_solves"] + st["newton_iters"] for st in p_stats) / len(p_stats)
    p_ms_launch = p_ms / len(p_stats)
    plain_roof = p_solves * fps / (p_ms_launch * 1e-3) / 1e12
    h2d = 16 * 30 + 16 + 16
    d2h = n * (16 * 21 + 4 + 8)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": k,
        "warmup": args.warmup, "ms_per_step": round(track_ms / k, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded task and start mechanisms)",
        "config": {"workload": f"Stephenson II FRG round: {n} paths on 1 generic complex precision-point task "
                               f"(seed {TASK_SEED}), complex-normal start mechanisms, random unit gamma; "
                               "sharpening to 1e-12 in FP64, canonical cognates, finite + residual <= 1e-10 "
                               "checks, duplicate removal",
                   "paths_per_step": n, "chosen": "mixed precision (FP32 team stage, FP64 endgame), team kernels",
                   "l2": "flushed (256 MB write) before every step", "parallelism": f"replicas x{world}"},
        "plain_fp64": {"value": round(value_plain, 2), "unit": UNIT, "steps": len(p_seeds),
                       "ms_per_step": round(p_ms_launch, 3),
                       "roofline_frac_fp64": round(plain_roof / peaks["fp64"], 4)},
        "speedup_vs_plain_fp64": round(value / value_plain, 3),
        "recall_vs_plain_fp64": round(min(rec), 5),
        "distinct_roots_per_step": distinct / k / world,
        "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"kernel": dom_name, "bound": dom["bound"], "achieved": round(dom["achieved"], 4),
                     "peak": round(dom["peak"], 4), "unit": "TFLOP/s", "frac": round(dom["frac"], 4),
                     "traffic": None,
                     "peak_source": "FMA peaks measured live by bench.py (MEASURED_PEAKS.json has no FP32/FP64 "
                                    "vector figure)",
                     "flops_per_solve": fps,
                     "kernels": {kk: {x: (round(y, 4) if isinstance(y, float) else y) for x, y in v.items()}
                                 for kk, v in kernels.items()}},
        # per step: two conversions of the task parameters (FP32, double-float), then
        # per mixed round one FP32-stage and one FP64-stage tracking kernel
        "gpu_launches": (2 + 2 * max(1, chosen_rounds)) * k,
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
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--paths", type=int, default=65536)
    ap.add_argument("--cpu-sample", type=int, default=8192)
    ap.add_argument("--plain-steps", type=int, default=1)
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
