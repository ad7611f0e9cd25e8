"""Benchmark: distinct finite roots per second on one GB300.

Workload (one "step" = one round of the tracker): 65,536 paths on one precision-
point task (seed 1: 8 points uniform in the unit disk, unit crank rotations), start
mechanisms from complex normal link/pivot values, a random unit-modulus gamma, FP64
tracking with sharpening to 1e-12 at t = 1, canonical cognates, finite-root check
(|Z0|/|Z| >= 1e-8), per-root residual, and duplicate removal in a root collection.
A root counts when its path succeeded, it is finite, its row-scaled residual is
<= 1e-10, and it is not a duplicate. Synthetic inputs: the reference ships no
benchmark data; tasks and starts are seeded.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--paths P] [--impl ours|reference]

value    distinct finite roots / second of device tracking time (inputs resident in HBM)
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
extern "C" __global__ void fma_peak_f64(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  if (x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7 == 123.0) out[0] = x0;
}
"""


def measure_fp64_peak():
    """Dense FP64 FMA throughput of this GPU (TFLOP/s), measured with a chain-free
    DFMA kernel. MEASURED_PEAKS.json records only HBM and bf16 tensor peaks."""
    from finite_root_generation_gb300 import build as frg_build

    import ctypes
    so = os.path.join(frg_build.BUILD, "fma_peak.so")
    os.makedirs(frg_build.BUILD, exist_ok=True)
    src = os.path.join(frg_build.BUILD, "fma_peak.cu")
    if not os.path.exists(so):
        with open(src, "w") as f:
            f.write(FMA_PEAK_SRC)
            f.write(r"""
#include <cuda_runtime.h>
extern "C" float run_fma_peak(int blocks, int threads, int iters) {
  double* out; cudaMalloc(&out, 8);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  fma_peak_f64<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e0);
  fma_peak_f64<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1); cudaEventSynchronize(e1);
  float ms; cudaEventElapsedTime(&ms, e0, e1);
  cudaFree(out); cudaEventDestroy(e0); cudaEventDestroy(e1);
  return ms;
}
""")
        subprocess.run([frg_build.nvcc(), *frg_build.ARCH, "-O3", "-Xcompiler", "-fPIC", "-shared", src, "-o", so],
                       check=True)
    lib = ctypes.CDLL(so)
    lib.run_fma_peak.restype = ctypes.c_float
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    ms = lib.run_fma_peak(blocks, threads, iters)
    flops = 2.0 * 8 * iters * blocks * threads
    return flops / (ms * 1e-3) / 1e12


# ------------------------------------------------------------------ algorithmic work
def algorithmic_flops(ivp_solves, newton_iters):
    """Algorithmic FLOPs of the linear-system steps, counting complex mul = 6, complex
    add = 2, real x complex = 2, complex fused multiply-add = 8 (the same convention
    for every variant; zeros of the Jacobian are not counted):
      system  = 7 groups of the generated code (FRG_GEN_* in frg_system_gen.cuh) + 4 reciprocals
      params  = q(t), dq/dt for 30 parameters
      scale   = 22 x 23 real x complex
      LU(ne)  = sum_i (ne-i-1)[(23-i-1) cfma + l + rhs] + back substitution
    """
    gen = open(os.path.join(ROOT, "finite_root_generation_gb300", "csrc", "frg_system_gen.cuh")).read()
    import re
    cm = int(re.search(r"#define FRG_GEN_CMUL (\d+)", gen).group(1))
    ca = int(re.search(r"#define FRG_GEN_CADD (\d+)", gen).group(1))
    sm = int(re.search(r"#define FRG_GEN_SMUL (\d+)", gen).group(1))
    w_sys = 7 * (6 * cm + 2 * ca + 2 * sm + 12) + 4 * 12
    w_par = 30 * 24
    w_scale = 22 * 23 * 2

    def lu(ne, n=23):
        f = 0
        for i in range(ne):
            f += (ne - i - 1) * ((n - i - 1) * 8 + 6 + 8)
        for i in range(n if ne == n else n - 1):
            f += (n - i - 1) * 8 + 6 + 2
        return f
    w_ivp = w_par + w_sys + w_scale + lu(23) + 23 * 8
    w_newton = w_par + w_sys + w_scale + lu(22) + 23 * 4
    return ivp_solves * w_ivp + newton_iters * w_newton, {"ivp": w_ivp, "newton": w_newton}


# ---------------------------------------------------------------------- our impl
def run_ours(args, rank, world):
    import torch

    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300 import build as frg_build
    from finite_root_generation_gb300.tasks import precision_point_task

    frg_build.build()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    task = precision_point_task(TASK_SEED, "disk")
    n = args.paths
    tracker = frg.Tracker(workload_config(frg, frg.PREC_FP64), device=dev)
    d_fpm = torch.from_numpy(task.view(np.float64).copy()).cuda()
    d_roots = torch.empty((n, 42), dtype=torch.float64, device="cuda")
    d_codes = torch.empty(n, dtype=torch.int32, device="cuda")
    d_resid = torch.empty(n, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def seed_of(step):
        return 1000003 * (rank + 1) + step

    for w in range(args.warmup):
        tracker.track_into(d_fpm, [n], seed_of(-1 - w), d_roots, d_codes, resid=d_resid)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    # ---- device-resident timing (value) ----
    track_ms, distinct, ivp, newt, launches = 0.0, 0, 0, 0, 0
    with ClockSampler(dev) as clk:
        for step in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            st = tracker.track_into(d_fpm, [n], seed_of(step), d_roots, d_codes, resid=d_resid)
            launches += 1
            track_ms += st["track_ms"]
            ivp += st["ivp_solves"]
            newt += st["newton_iters"]
            roots = d_roots.cpu().numpy().view(np.complex128)
            d, _ = count_distinct(frg, roots, d_codes.cpu().numpy(), d_resid.cpu().numpy())
            distinct += d
    torch.cuda.synchronize()
    clocks = clk.summary()

    # ---- end to end through the C ABI with host buffers (e2e) ----
    h_roots = np.zeros((n, 21), np.complex128)
    h_codes = np.zeros(n, np.int32)
    h_resid = np.zeros(n, np.float64)
    e2e_distinct = 0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for step in range(args.steps):
        tracker.track_into(task, [n], seed_of(step), h_roots, h_codes, resid=h_resid)
        d, _ = count_distinct(frg, h_roots, h_codes, h_resid)
        e2e_distinct += d
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

    t = torch.tensor([track_ms, e2e_s, distinct, e2e_distinct, ivp, newt], dtype=torch.float64)
    if world > 1:
        tmax = t.clone().cuda()
        tsum = t.clone().cuda()
        torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(tsum, op=torch.distributed.ReduceOp.SUM)
        track_ms, e2e_s = float(tmax[0]), float(tmax[1])
        distinct, e2e_distinct, ivp, newt = (float(x) for x in tsum[2:6])
    tracker.close()
    if rank != 0:
        return None

    value = distinct / (track_ms * 1e-3)
    e2e = e2e_distinct / e2e_s
    flops, per = algorithmic_flops(ivp / world, newt / world)
    achieved = flops / (track_ms / args.steps * 1e-3) / args.steps / 1e12  # per launch / launch time
    peak = measure_fp64_peak()
    h2d = 16 * 30 + 16 + 16  # task, gamma, task offsets
    d2h = n * (16 * 21 + 4 + 8)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(track_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded tasks and starts)",
        "config": {"workload": f"Stephenson II FRG round: {n} paths, 1 precision-point task (seed {TASK_SEED}), "
                               "complex-normal starts, random gamma, FP64 + sharpening + dedup",
                   "paths_per_step": n, "precision": "plain FP64", "l2": "flushed (256 MB write) between steps",
                   "parallelism": f"replicas x{world} (independent paths)"},
        "distinct_roots_per_step": distinct / args.steps / world,
        "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fp64", "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
                     "frac": round(achieved / peak, 4), "traffic": None,
                     "peak_source": "FP64 FMA peak measured live by bench.py (MEASURED_PEAKS.json has no FP64 figure)",
                     "flops_per_ivp_solve": per["ivp"], "flops_per_newton_iter": per["newton"],
                     "solves_per_launch": (ivp + newt) / world / args.steps},
        "gpu_launches": launches,
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
    ap.add_argument("--cpu-sample", type=int, default=1024)
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
