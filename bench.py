"""Benchmark: distinct finite roots per second on one GB300, chosen configuration vs
plain FP64 (the metric of the mixed-precision tracker).

Workload (default, --workload c5): 1,048,576 paths over 128 tasks, 8,192 paths each.
Task k (seeds 0..127) has its precision points in the unit disk (even k) or along a
random smooth closed curve with 1% jitter (odd k); crank rotations on the unit circle.
Start mechanisms from complex-normal link/pivot values, a random unit-modulus gamma per
task and round, sharpening to 1e-12 at t = 1, canonical cognates, finite-root check
(|Z0|/|Z| >= 1e-8) and per-root residual. A root counts when its path succeeded, it is
finite, its row-scaled residual is <= 1e-10, and it is not a duplicate of a root already
collected for its task in the timed region (one collection per task across all steps,
the reference's cross-round merge, frg.cu:440). Synthetic inputs: the reference ships no
benchmark data; tasks and starts are seeded.

One step = one round of 8 tasks x 8,192 paths (65,536 paths): step s tracks tasks
8 (s mod 16) .. 8 (s mod 16) + 7 with seed 1000003 + s, so 16 steps cover the whole
1,048,576-path workload and later steps run further rounds on the same tasks.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c5|c4|c2] [--impl ours|reference]

value    distinct finite roots / second over K steps of the chosen configuration run through
         frg_track_rounds with --depth rounds in flight (task sets resident in HBM, CUDA events
         on the launching streams). Plain FP64 over the same K steps, seeds and pipelining gives
         plain_fp64, the speed-up and the recall of plain FP64's distinct roots.
e2e      the same through the public C ABI with pinned host buffers: the task upload, tracking,
         the copy of roots/codes/residuals back and the host duplicate merge of every step
--impl reference  the reference's own tracker sources built for the host (oracle/_ref,
         staged reference sources; the oracle restatement where they are missing) on all host
         cores, each step a bounded sample of the same step's tasks, seeds and path streams.
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
DUP_TOL = 1e-6
SEED_BASE = 1000003
WARM_SEED_BASE = 7000001


def _load_tasks_module():
    """The task generator (numpy only), loaded by file path so that the reference arm
    never imports the product package."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "frg_bench_tasks", os.path.join(ROOT, "finite_root_generation_gb300", "tasks.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class Workload:
    """Tasks, their path counts and the tasks of each step.

    c5: 128 tasks (seeds 0..127, disk / curve alternating) x 8,192 paths, 8 tasks per step
    c4: 64 tasks (seeds 0..63, disk / curve alternating) x 8,192 paths, 8 tasks per step
    c2: 1 task (seed 1, disk) x 65,536 paths per step (rounds on one task, the reference's loop)"""

    def __init__(self, name):
        tm = _load_tasks_module()
        self.name = name
        if name == "c5":
            ntasks, self.paths_per_task, self.tasks_per_step = 128, 8192, 8
        elif name == "c4":
            ntasks, self.paths_per_task, self.tasks_per_step = 64, 8192, 8
        elif name == "c2":
            ntasks, self.paths_per_task, self.tasks_per_step = 1, 65536, 1
        else:
            raise SystemExit(f"unknown workload {name}")
        if name == "c2":
            self.tasks = np.stack([tm.precision_point_task(1, "disk")])
        else:
            self.tasks = np.stack([tm.precision_point_task(k, "disk" if k % 2 == 0 else "curve")
                                   for k in range(ntasks)])
        self.ntasks = ntasks
        self.blocks = ntasks // self.tasks_per_step
        self.paths_per_step = self.paths_per_task * self.tasks_per_step

    def step_tasks(self, s):
        """Global task indices of step s."""
        b = s % self.blocks
        return list(range(b * self.tasks_per_step, (b + 1) * self.tasks_per_step))

    def task_sets(self, steps):
        """[len(steps), tasks_per_step, 30] task parameters of the given steps."""
        return np.ascontiguousarray(np.stack([self.tasks[self.step_tasks(s)] for s in steps]))

    def describe(self):
        if self.name == "c2":
            return ("Stephenson II FRG rounds of 65,536 paths on one generic complex precision-point task (seed 1, "
                    "points in the unit disk)")
        total = self.ntasks * self.paths_per_task
        return (f"Stephenson II FRG, {total:,} paths over {self.ntasks} tasks ({self.paths_per_task:,} each; task "
                f"seeds 0..{self.ntasks - 1}, precision points in the unit disk / along a random smooth closed curve "
                f"with 1% jitter, alternating), one step = {self.tasks_per_step} tasks x {self.paths_per_task:,} "
                f"paths, {self.blocks} steps per pass over all tasks")


def workload_config(frg, precision):
    return frg.default_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=INF_TOL,
                              precision=precision)


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
def _chosen_overrides(frg):
    """The chosen configuration on top of the workload's (frg.CHOSEN): mixed precision,
    the FP32 stage also running the endgame and sharpening (double-float points and
    refinement), FP64 for steps whose condition estimate exceeds 1e6 and for finishing
    every root, at most 10,000 FP64 solves per path and launch (a path still going after
    that ends as a step-limit failure; such paths crawl near a singularity and set the
    FP64 tail), paths well conditioned again carried back to FP32 in a later round, the
    rounds launched as one CUDA graph."""
    return dict(frg.CHOSEN)


class TaskCollections:
    """One root collection per task across all steps (the reference merges every round
    into one collection, frg.cu:440); counts distinct finite roots."""

    def __init__(self, make_collection, ntasks):
        self.make = make_collection
        self.colls = {}
        self.ntasks = ntasks

    def merge_step(self, wl, s, roots, codes, resid):
        """roots [P, 21] complex, codes [P], resid [P] of step s (paths_per_task per task)."""
        ppt = wl.paths_per_task if roots.shape[0] == wl.paths_per_step else roots.shape[0] // wl.tasks_per_step
        for i, k in enumerate(wl.step_tasks(s)):
            sl = slice(i * ppt, (i + 1) * ppt)
            good = (codes[sl] == 0) & (resid[sl] <= RESID_MAX)
            c = np.where(good, 0, 5).astype(np.int32)
            if k not in self.colls:
                self.colls[k] = self.make()
            self.colls[k].merge(roots[sl], c)

    def distinct(self):
        return sum(len(c) for c in self.colls.values())

    def roots_of(self, k):
        c = self.colls.get(k)
        return c.roots() if c is not None else np.zeros((0, 21), np.complex128)


def _timed_rounds(torch, tracker, fpm_sets, ppt, seeds, outs, depth, world, dedup=None):
    """K rounds through frg_track_rounds (device buffers, `depth` rounds in flight, one
    task set per round), then, with dedup = (DeviceCollection, keys), the duplicate
    removal of every round's roots on the device; bracketed by a barrier and a
    synchronize on both sides. Returns (stats, ms): the library times the tracking span
    with CUDA events on its launching streams (first launch to the last round's end) and
    the merges are timed with CUDA events on the stream they run on (torch's current
    stream); ms = tracking span + merges."""
    roots, codes, resid = outs
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    st = tracker.track_rounds(fpm_sets, ppt, seeds, roots, codes, resid=resid, depth=depth, per_round_tasks=True)
    merge_ms = 0.0
    if dedup is not None:
        # the merges mark duplicates in a copy of the codes (made by the copy engine), so the
        # tracker's own codes stay available for the host cross-check
        dc, keys, mark = dedup
        n = keys[0].numel()
        mark.copy_(codes)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        stream = torch.cuda.current_stream().cuda_stream
        ev0.record()
        for i in range(len(seeds)):
            sl = slice(i * n, (i + 1) * n)
            dc.merge(roots[sl], mark[sl], keys[i], stream=stream, resid=resid[sl], resid_max=RESID_MAX)
        ev1.record()
        torch.cuda.synchronize()
        merge_ms = ev0.elapsed_time(ev1)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    return st, st["track_ms"] + merge_ms, merge_ms


def _collect(frg, wl, steps, outs, n):
    """Per-task collections of K steps' device outputs, and the outputs on the host."""
    R = outs[0].cpu().numpy().view(np.complex128)
    C = outs[1].cpu().numpy()
    E = outs[2].cpu().numpy()
    tc = TaskCollections(lambda: frg.Collection(DUP_TOL), wl.ntasks)
    for i, s in enumerate(steps):
        sl = slice(i * n, (i + 1) * n)
        tc.merge_step(wl, s, R[sl], C[sl], E[sl])
    tc.host = (R, C, E)
    return tc


def _kept_root_quality(chosen, plain):
    """Residuals of the chosen run's kept roots and, per path, the distance of its root to
    the plain FP64 run's root of the same path (same random stream)."""
    Rc, Cc, Ec = chosen
    Rp, Cp, _ = plain
    kept = (Cc == 0) & (Ec <= RESID_MAX)
    both = kept & (Cp == 0)
    d = np.max(np.abs(Rc[both] - Rp[both]), axis=1) / np.max(np.abs(Rp[both]), axis=1)
    near = d <= 1e-8
    return {"kept_roots": int(kept.sum()),
            "kept_residual_max": float(Ec[kept].max()) if kept.any() else None,
            "kept_residual_median": float(np.median(Ec[kept])) if kept.any() else None,
            "successes_failing_residual": int(((Cc == 0) & ~(Ec <= RESID_MAX)).sum()),
            "paths_kept_by_both": int(both.sum()),
            "within_1e-8_of_fp64_track": round(float(near.mean()), 5) if both.any() else None,
            "distance_to_fp64_track_median": float(np.median(d)) if both.any() else None,
            "distance_to_fp64_track_p99_of_those_within": float(np.quantile(d[near], 0.99)) if near.any() else None}


def run_ours(args, rank, world):
    import torch

    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300 import build as frg_build
    from finite_root_generation_gb300.metrics import recall

    frg_build.build()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    wl = Workload(args.workload)
    n, k, depth = wl.paths_per_step, args.steps, args.depth
    ppt = [wl.paths_per_task] * wl.tasks_per_step
    chosen_cfg = workload_config(frg, frg.PREC_MIXED)
    for key, v in _chosen_overrides(frg).items():
        setattr(chosen_cfg, key, v)
    # the autotuner's recorded choice for this GPU and workload, where there is one
    from finite_root_generation_gb300 import autotune
    tuned = autotune.tuned_setting(torch.cuda.get_device_name(dev), args.workload)
    if tuned:
        depth = int(tuned.pop("depth", depth))
        for key, v in tuned.items():
            setattr(chosen_cfg, key, v)
    chosen = frg.Tracker(chosen_cfg, device=dev)
    plain = frg.Tracker(workload_config(frg, frg.PREC_FP64), device=dev)
    # steps of this rank (ranks take disjoint seeds)
    steps = list(range(k))

    def seed_of(s):
        return SEED_BASE + 1000 * rank + s

    seeds = [seed_of(s) for s in steps]
    sets = wl.task_sets(steps)
    d_sets = torch.from_numpy(sets.view(np.float64).copy()).cuda()
    nbuf = max(k, args.warmup, 1) * n
    outs = (torch.empty((nbuf, 42), dtype=torch.float64, device="cuda"),
            torch.empty(nbuf, dtype=torch.int32, device="cuda"),
            torch.empty(nbuf, dtype=torch.float64, device="cuda"))
    # warm-up: W rounds of the chosen configuration (other seeds) and one small plain round
    wsteps = list(range(args.warmup))
    warm = [WARM_SEED_BASE + 1000 * rank + s for s in wsteps]
    if warm:
        d_wsets = torch.from_numpy(wl.task_sets(wsteps).view(np.float64).copy()).cuda()
        chosen.track_rounds(d_wsets, ppt, warm, outs[0][: len(warm) * n], outs[1][: len(warm) * n],
                            resid=outs[2][: len(warm) * n], depth=depth, per_round_tasks=True)
        plain.track_rounds(d_wsets[:1], [min(c, 1024) for c in ppt], warm[:1], outs[0], outs[1],
                           resid=outs[2], depth=1, per_round_tasks=True)
    torch.cuda.synchronize()

    # device duplicate removal: one collection per global task (key), keys of each step
    keys = [torch.from_numpy(np.repeat(np.asarray(wl.step_tasks(s), np.int32), wl.paths_per_task)).cuda()
            for s in steps]
    capacity = k * n + 1024
    mark = torch.empty(k * n, dtype=torch.int32, device="cuda")

    # ---- chosen configuration, task sets resident in HBM (value): tracking and the
    #      device duplicate removal of every round ----
    c_outs = tuple(o[: k * n] for o in outs)
    c_dc = frg.DeviceCollection(capacity, DUP_TOL, device=dev)
    with ClockSampler(dev) as clk:
        c_st, c_ms, c_merge_ms = _timed_rounds(torch, chosen, d_sets, ppt, seeds, c_outs, depth, world,
                                               dedup=(c_dc, keys, mark))
    clocks = clk.summary()
    c_dev_distinct = len(c_dc)
    c_dc.close()
    c_coll = _collect(frg, wl, steps, c_outs, n)
    if c_dev_distinct != c_coll.distinct():
        raise SystemExit(f"device and host duplicate removal disagree: {c_dev_distinct} vs {c_coll.distinct()}")
    # ---- plain FP64 on the same steps, seeds and pipelining (ratio and recall) ----
    p_dc = frg.DeviceCollection(capacity, DUP_TOL, device=dev)
    p_st, p_ms, _ = _timed_rounds(torch, plain, d_sets, ppt, seeds, c_outs, depth, world, dedup=(p_dc, keys, mark))
    p_dev_distinct = len(p_dc)
    p_dc.close()
    p_coll = _collect(frg, wl, steps, c_outs, n)
    hits = found = 0
    for t in sorted(p_coll.colls):
        a = p_coll.roots_of(t)
        hits += round(recall(a, c_coll.roots_of(t)) * len(a))
        found += len(a)
    rec = hits / max(found, 1)
    quality = _kept_root_quality(c_coll.host, p_coll.host)
    c_coll.host = p_coll.host = None
    # ---- one round of the chosen configuration with nothing else in flight: its FP32 and
    #      FP64 stages' own durations (the pipelined rounds overlap them) ----
    solo_st, _, _ = _timed_rounds(torch, chosen, d_sets[:1], ppt, seeds[:1], tuple(o[:n] for o in outs), 1, world)

    # ---- end to end through the C ABI with pinned host buffers (e2e): the task upload,
    #      tracking, the copy of roots/codes/residuals back, and the host duplicate merge
    #      into the per-task collections ----
    h_sets = torch.from_numpy(sets.view(np.float64).copy()).pin_memory()
    h_roots = torch.empty((k * n, 42), dtype=torch.float64, pin_memory=True)
    h_codes = torch.empty(k * n, dtype=torch.int32, pin_memory=True)
    h_resid = torch.empty(k * n, dtype=torch.float64, pin_memory=True)
    hr, hc, he = h_roots.numpy(), h_codes.numpy(), h_resid.numpy()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    chosen.track_rounds(h_sets.numpy(), ppt, seeds, hr, hc, resid=he, depth=depth, per_round_tasks=True)
    R = hr.view(np.complex128)
    e2e_coll = TaskCollections(lambda: frg.Collection(DUP_TOL), wl.ntasks)
    for i, s in enumerate(steps):
        sl = slice(i * n, (i + 1) * n)
        e2e_coll.merge_step(wl, s, R[sl], hc[sl], he[sl])
    e2e_distinct = e2e_coll.distinct()
    e2e_s = time.perf_counter() - t0

    track_ms = c_ms
    distinct = c_dev_distinct
    p_distinct = p_dev_distinct
    t = torch.tensor([track_ms, e2e_s, distinct, e2e_distinct, p_ms, p_distinct, hits, found],
                     dtype=torch.float64)
    if world > 1:
        tmax, tsum = t.clone().cuda(), t.clone().cuda()
        torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(tsum, op=torch.distributed.ReduceOp.SUM)
        track_ms, e2e_s, p_ms = float(tmax[0]), float(tmax[1]), float(tmax[4])
        distinct, e2e_distinct, p_distinct = float(tsum[2]), float(tsum[3]), float(tsum[5])
        rec = float(tsum[6]) / max(float(tsum[7]), 1.0)
    chosen_rounds = chosen.config.mixed_rounds
    chosen_carry = bool(chosen.config.carry_handback) and chosen_rounds <= 1
    chosen.close()
    plain.close()
    if rank != 0:
        return None

    value = distinct / (track_ms * 1e-3)
    value_plain = p_distinct / (p_ms * 1e-3)
    e2e = e2e_distinct / e2e_s
    peaks = measure_fma_peaks()
    fps = flops_per_solve()
    # roofline of the whole step: the FMA-pipe time its algorithmic FLOPs need at the two
    # measured peaks, over the step's time, (F32 / peak32 + F64 / peak64) / T
    solves = c_st["ivp_solves"] + c_st["newton_iters"]
    fp64_solves = c_st["fp64_solves"]
    fp32_solves = solves - fp64_solves
    F32, F64 = fp32_solves * fps, fp64_solves * fps
    T = track_ms * 1e-3
    frac = (F32 / (peaks["fp32"] * 1e12) + F64 / (peaks["fp64"] * 1e12)) / T
    # per kernel, from the round with nothing else in flight (non-overlapped stage times)
    s_solves = solo_st["ivp_solves"] + solo_st["newton_iters"]
    s64 = solo_st["fp64_solves"]
    s32 = s_solves - s64
    ms32, ms64 = solo_st["stage_ms"]
    kernels = {
        "team_kernel<1, float, df> (FP32 stage)": {
            "bound": "fp32", "achieved": s32 * fps / (ms32 * 1e-3) / 1e12, "peak": peaks["fp32"],
            "ms_per_launch": ms32, "solves_per_launch": s32},
        "team_kernel<2, double, double> (FP64 stage)": {
            "bound": "fp64", "achieved": s64 * fps / (ms64 * 1e-3) / 1e12, "peak": peaks["fp64"],
            "ms_per_launch": ms64, "solves_per_launch": s64},
    }
    for v in kernels.values():
        v["frac"] = v["achieved"] / v["peak"]
    p_solves = p_st["ivp_solves"] + p_st["newton_iters"]
    plain_frac = p_solves * fps / (p_ms * 1e-3) / (peaks["fp64"] * 1e12)
    ntask = wl.tasks_per_step
    h2d = ntask * (16 * 30 + 16 * 3 + 8) + 8  # task parameters, gammas (3 precisions), path offsets
    d2h = n * (16 * 21 + 4 + 8) + FRG_COUNTERS_BYTES
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": k,
        "warmup": args.warmup, "ms_per_step": round(track_ms / k, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded tasks and start mechanisms)",
        "config": {"workload": wl.describe() + "; complex-normal start mechanisms, random unit gamma per task and "
                               "round; FP64 sharpening check, canonical cognates, finite + residual <= 1e-10 "
                               "checks, one duplicate collection per task over the timed steps",
                   "paths_per_step": n, "tasks_per_step": wl.tasks_per_step, "steps_cover_workload": k >= wl.blocks,
                   "rounds_in_flight": depth,
                   "setting_from": "autotuner table (finite_root_generation_gb300/tuned.json)" if tuned
                                   else "frg.CHOSEN",
                   "chosen": "mixed precision: FP32 team kernel (double-float points and refinement, endgame and "
                             "sharpening included), FP64 team kernel for steps with condition estimate > "
                             f"{chosen_cfg.cond_switch:.0e} (at most {chosen_cfg.fp64_budget:,} FP64 solves per "
                             "path and launch) and for finishing; paths well conditioned again carried back to "
                             "FP32 in a later round; rounds as one CUDA graph; duplicate removal on the device",
                   "l2": f"not flushed: per-round state (start values 816 B, hand-off record 1.2 KB, outputs "
                         f"348 B per path: ~{n * 2364 / 1e6:.0f} MB per round, {depth} rounds in flight) exceeds "
                         "the 129 MB L2",
                   "parallelism": f"replicas x{world}"},
        "plain_fp64": {"value": round(value_plain, 2), "unit": UNIT, "steps": k, "rounds_in_flight": depth,
                       "ms_per_step": round(p_ms / k, 3), "distinct": int(p_distinct),
                       "roofline_frac_fp64": round(plain_frac, 4)},
        "speedup_vs_plain_fp64": round(value / value_plain, 3),
        "recall_vs_plain_fp64": round(rec, 5),
        "kept_root_quality": quality,
        "distinct_roots": int(distinct),
        "dedup_ms_per_step": round(c_merge_ms / k, 3),
        "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fma (fp32 + fp64 pipes)", "achieved": round(frac, 5), "peak": 1.0,
                     "unit": "fraction of the step's time the algorithmic FLOPs need at the measured FP32 and "
                             "FP64 FMA peaks: (F32/peak32 + F64/peak64)/T",
                     "frac": round(frac, 5),
                     "traffic": round((TRAFFIC_PER_PATH["fp32_stage"] + TRAFFIC_PER_PATH["fp64_stage"]) * n),
                     "traffic_unit": "bytes per step (both tracking stages, DRAM read + write; ncu capture of a "
                                     "4,096-path round scaled by paths; inputs and outputs are ~1.2 KB per path)",
                     "f32_tflop": round(F32 / 1e12, 3), "f64_tflop": round(F64 / 1e12, 3),
                     "peak_fp32_tflops": round(peaks["fp32"], 2), "peak_fp64_tflops": round(peaks["fp64"], 4),
                     "peak_source": "FMA peaks of measured: bench.py's own chain-free FMA kernels (MEASURED_PEAKS.json "
                                    "has no FP32/FP64 vector figure)",
                     "flops_per_solve": fps,
                     "kernels_one_round_alone": {
                         kk: {x: (round(y, 4) if isinstance(y, float) else y) for x, y in v.items()}
                         for kk, v in kernels.items()}},
        # tracking: with carry hand-back the FP32 and double-float parameter copies once,
        # then per round the start values, the FP32-stage and the FP64-stage kernels;
        # without it all five per round (two per mixed round); dedup: five kernels per round
        "gpu_launches": ((2 + 3 * k) if chosen_carry else (3 + 2 * max(1, chosen_rounds)) * k) + 5 * k,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, wl, steps=[0], paths_per_task=args.cpu_paths)
    return line


FRG_COUNTERS_BYTES = 48 * 8
# DRAM bytes (read + write) per path of the two tracking stages, from one ncu capture of a
# 4,096-path round of the chosen configuration (`bench.py --profile-case`, MemoryWorkloadAnalysis):
# 11.67 MB for the FP32 stage and 29.85 MB for the FP64 stage; a round's traffic is taken to
# grow in proportion to its paths
TRAFFIC_PER_PATH = {"fp32_stage": 11.67e6 / 4096, "fp64_stage": 29.85e6 / 4096}


# ------------------------------------------------------------------- CPU baseline
def _gamma_of(uniform01, seed, k):
    """The random gamma of task k of a call with `seed` (the library's per-task draw:
    stream 2^64 - 1 - k, index 0)."""
    phi = 2 * np.pi * uniform01(seed, 2**64 - 1 - k, 0)
    return complex(np.cos(phi), np.sin(phi))


def cpu_baseline(args, wl, steps, paths_per_task, seed_base=SEED_BASE):
    """The reference tracker on all host cores over a sample of the given steps: for each
    step, the first `paths_per_task` paths of each of its tasks, with the step's seed,
    path streams and gammas. Uses the reference's own sources built for the host
    (oracle/_ref/libfrgref.so, kind "reference") where they were staged, else the oracle's
    C restatement (kind "port"). Duplicates are removed with the oracle's restatement of
    SortingDeletingMerging (pinned to the reference's merge by the golden vectors): the
    reference's own merge reads one element past its local order vector in its fold loop
    (frgsupport.cu:195), which crashed the host process once collections grew past a
    round. Never loads the product library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build(ref=True)
    cores = os.cpu_count() or 1
    use_ref = os.path.exists(oracle.REF_SO)
    lib = oracle.RefLib() if use_ref else oracle.Oracle()
    merger = oracle.Oracle()
    o_cfg = None if use_ref else lib.config(start_dist=1)
    colls = {}
    total_paths = 0
    t0 = time.perf_counter()
    for s in steps:
        seed = seed_base + s
        for i, kt in enumerate(wl.step_tasks(s)):
            fpm = wl.tasks[kt]
            gamma = _gamma_of(lib.uniform01, seed, i)
            stream0 = i * wl.paths_per_task
            if use_ref:
                roots, codes, yf, resid = lib.homotopy_batch_ex(fpm, gamma, seed, stream0, paths_per_task,
                                                                start_normal=True, nthreads=cores)
            else:
                roots, codes, _, yf = lib.homotopy_batch(fpm, gamma, seed, stream0 + np.arange(paths_per_task),
                                                         cfg=o_cfg, nthreads=cores, want_yfinal=True)
                resid = lib.residuals(roots, fpm)
            zmax = np.max(np.abs(yf[:, :21]), axis=1)
            finite = np.abs(yf[:, 21]) >= INF_TOL * zmax
            good = (codes == 0) & finite & (resid <= RESID_MAX)
            c = np.where(good, 0, 5).astype(np.int32)
            coll = colls.get(kt, np.zeros((0, 21), np.complex128))
            colls[kt], _ = merger.sort_merge(coll, roots, c, DUP_TOL)
            total_paths += paths_per_task
    dt = time.perf_counter() - t0
    d = sum(len(c) for c in colls.values())
    return {"value": round(d / dt, 3), "unit": UNIT, "cores": cores, "kind": "reference" if use_ref else "port",
            "distinct": d, "paths": total_paths, "seconds": round(dt, 2),
            "sample": f"first {paths_per_task} paths of each task of step(s) {steps[0]}..{steps[-1]} "
                      f"({total_paths} paths, the GPU arm's seeds and path streams), {dt:.1f} s on {cores} threads; "
                      + ("the reference's own tracker sources built for this host (oracle/_ref/libfrgref.so); "
                         "duplicates by the oracle's restatement of SortingDeletingMerging (the reference's own "
                         "reads past its order vector, frgsupport.cu:195, and crashed on grown collections)"
                         if use_ref else
                         "the oracle's C restatement (the reference's sources were not staged)")}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    wl = Workload(args.workload)
    for s in range(args.warmup):
        cpu_baseline(args, wl, steps=[s], paths_per_task=args.cpu_paths, seed_base=WARM_SEED_BASE)
    res = cpu_baseline(args, wl, steps=list(range(args.steps)), paths_per_task=args.cpu_paths)
    v = res["value"]
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(res["seconds"] / args.steps * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded tasks and start mechanisms)",
            "config": {"workload": wl.describe() + "; complex-normal start mechanisms, random unit gamma per task "
                                   "and round; FP64 sharpening, canonical cognates, finite + residual <= 1e-10 "
                                   "checks, one duplicate collection per task over the timed steps",
                       "paths_per_step": args.cpu_paths * wl.tasks_per_step,
                       "sample_of_gpu_step": f"first {args.cpu_paths} of each task's {wl.paths_per_task} paths",
                       "precision": "plain FP64", "parallelism": "host threads"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": res["cores"], "kind": res["kind"],
                             "sample": res["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ------------------------------------------------------------------ plug-in systems
def _plugin_tasks(name, ntasks):
    """Seeded tasks of a plug-in system: five physical positions (burmester5) or two line
    pairs in general position (conic2), task k from seed k."""
    import importlib
    mod = importlib.import_module(f"finite_root_generation_gb300.systems.{name}")
    out = []
    for k in range(ntasks):
        rng = np.random.default_rng(k)
        if name == "burmester5":
            out.append(mod.physical_task(rng))
        elif name == "conic2":
            out.append(mod.line_pair_task(rng.normal(size=4) + 1j * rng.normal(size=4),
                                          rng.normal(size=4) + 1j * rng.normal(size=4))[0])
        else:
            raise SystemExit(f"no benchmark tasks for system {name}")
    return np.stack(out)


def plugin_flops_per_solve(name, nv, np_):
    """Algorithmic FLOPs of one linear-system step of the thread kernel on a plug-in
    system (complex mul = 6, add = 2, real x complex = 2, FMA = 8, reciprocal = 12):
    q(t), dq/dt (np x 24), the generated rows (their operation counts, in the header),
    row scaling (nz x ny x 2), dense LU of the ny x ny system with its right-hand side
    (sum over pivots of a reciprocal and, per row below, a multiplier and ny - 1 - i
    FMAs plus one for the right-hand side), back substitution and the tangent's norm.
    The tangent step is counted for Newton steps as well (one row fewer eliminated)."""
    import re
    gen = open(os.path.join(ROOT, "finite_root_generation_gb300", "csrc", "frg_plugins_gen.cuh")).read()
    i = gen.index(f"struct Sys_{name} ")
    m = re.search(r"ROWS_CMUL = (\d+), ROWS_CADD = (\d+), ROWS_SMUL = (\d+)", gen[i:])
    cm, ca, sm = (int(x) for x in m.groups())
    ny, nz = nv + 2, nv + 1
    f = np_ * 24 + 6 * cm + 2 * ca + 2 * sm + nz * ny * 2
    f += sum(12 + (ny - 1 - i) * (6 + 8 * (ny - 1 - i) + 8) for i in range(ny))
    f += sum(8 * (ny - 1 - i) + 6 for i in range(ny))
    f += ny * 10
    return f


def run_plugin(args):
    """--system NAME: paths/s of a plug-in system on the FP64 thread kernel, rounds of
    --plugin-tasks tasks x --plugin-paths paths through frg_track_rounds (device outputs,
    CUDA-event span), end to end from host buffers, the kernel's FP64 roofline, and the
    oracle's tracker on the host cores (no reference implementation exists for a plug-in)."""
    import torch

    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300 import build as frg_build
    from finite_root_generation_gb300.metrics import distinct_rows

    frg_build.build()
    cfg = frg.plugin_config(args.system, start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=INF_TOL)
    info = frg.system_info(cfg.system)
    T, n, k, depth = args.plugin_tasks, args.plugin_paths, args.steps, 2
    tasks = _plugin_tasks(args.system, T)
    N = T * n
    dev = torch.device("cuda", 0)
    fpm_d = torch.from_numpy(tasks.view(np.float64).copy()).to(dev)
    seeds = [SEED_BASE + s for s in range(k)]
    roots = torch.empty((k * N, info.nv, 2), dtype=torch.float64, device=dev)
    codes = torch.empty(k * N, dtype=torch.int32, device=dev)
    resid = torch.empty(k * N, dtype=torch.float64, device=dev)
    with frg.Tracker(cfg) as t:
        for w in range(args.warmup):
            t.track_rounds(fpm_d, [n] * T, [WARM_SEED_BASE + w], roots[:N], codes[:N], resid[:N], depth=1)
        torch.cuda.synchronize()
        with ClockSampler() as clk:
            st = t.track_rounds(fpm_d, [n] * T, seeds, roots, codes, resid, depth=depth)
        torch.cuda.synchronize()
        # end to end: host task set in, host roots, codes and residuals out
        h_roots = np.zeros((k * N, info.nv), np.complex128)
        h_codes = np.zeros(k * N, np.int32)
        h_resid = np.zeros(k * N)
        t0 = time.perf_counter()
        t.track_rounds(tasks, [n] * T, seeds, h_roots, h_codes, h_resid, depth=depth)
        e2e_s = time.perf_counter() - t0
    # mixed precision on the same rounds: the thread kernel's FP32 stage with hand-off to FP64
    mcfg = frg.plugin_config(args.system, precision=frg.PREC_MIXED, start_dist=frg.START_NORMAL,
                             gamma_mode=frg.GAMMA_RANDOM, inf_tol=INF_TOL)
    m_roots = torch.empty_like(roots)
    m_codes = torch.empty_like(codes)
    m_resid = torch.empty_like(resid)
    with frg.Tracker(mcfg) as tm:
        for w in range(args.warmup):
            tm.track_rounds(fpm_d, [n] * T, [WARM_SEED_BASE + w], m_roots[:N], m_codes[:N], m_resid[:N], depth=1)
        torch.cuda.synchronize()
        st_m = tm.track_rounds(fpm_d, [n] * T, seeds, m_roots, m_codes, m_resid, depth=depth)
        torch.cuda.synchronize()
    ms = st["track_ms"]
    r = roots.cpu().numpy().view(np.complex128).reshape(k * N, info.nv)
    c = codes.cpu().numpy()
    e = resid.cpu().numpy()
    mr = m_roots.cpu().numpy().view(np.complex128).reshape(k * N, info.nv)
    mc = m_codes.cpu().numpy()
    me = m_resid.cpu().numpy()
    # the end-to-end run repeats the device run path for path (failed paths' non-finite
    # roots compare equal); reported, not asserted
    same = (c == h_codes) & np.all((r == h_roots) | (np.isnan(r) & np.isnan(h_roots)), axis=1)
    mismatch = int((~same).sum())
    from finite_root_generation_gb300.metrics import recall

    distinct, m_distinct = [], []
    hits = total = 0
    for j in range(T):
        sel = np.concatenate([np.arange(s * N + j * n, s * N + (j + 1) * n) for s in range(k)])
        a = distinct_rows(r[sel], (c[sel] == 0) & (e[sel] <= RESID_MAX), DUP_TOL, relative=True)
        b = distinct_rows(mr[sel], (mc[sel] == 0) & (me[sel] <= RESID_MAX), DUP_TOL, relative=True)
        distinct.append(len(a))
        m_distinct.append(len(b))
        hits += round(recall(a, b) * len(a))
        total += len(a)
    m_ms = st_m["track_ms"]
    m_solves = st_m["ivp_solves"] + st_m["newton_iters"]
    solves = st["ivp_solves"] + st["newton_iters"]
    fps = plugin_flops_per_solve(args.system, info.nv, info.np)
    peaks = measure_fma_peaks()
    achieved = solves * fps / (ms * 1e-3) / 1e12
    value = k * N / (ms * 1e-3)
    line = {"metric": f"paths tracked/s, plug-in system {args.system} (FP64)", "value": round(value, 1),
            "unit": "paths/s", "n_gpus": 1, "steps": k, "warmup": args.warmup, "ms_per_step": round(ms / k, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded tasks and start points)",
            "config": {"workload": f"{args.system}: {T} tasks x {n} paths per step ({info.nv} unknowns, "
                                   f"{info.np} parameters), complex-normal starts, random gamma per task and step, "
                                   f"{depth} rounds in flight",
                       "paths_per_step": N, "l2": "not flushed: per-step outputs and state are small; the "
                                                  "kernel is compute bound"},
            "codes": [int(x) for x in np.bincount(c, minlength=8)],
            "e2e_paths_differing_from_device_run": mismatch,
            "distinct_roots_per_task": {"min": min(distinct), "max": max(distinct)},
            "e2e": {"value": round(k * N / e2e_s, 1), "unit": "paths/s",
                    "h2d_bytes_per_step": int(tasks.nbytes), "d2h_bytes_per_step": int(N * (info.nv * 16 + 12))},
            "roofline": {"bound": "fp64", "achieved": round(achieved, 4), "peak": round(peaks["fp64"], 4),
                         "unit": "TFLOP/s", "frac": round(achieved / peaks["fp64"], 4), "traffic": None,
                         "flops_per_solve": fps, "solves": int(solves),
                         "peak_source": "of measured: bench.py's own FP64 FMA kernel"},
            "gpu_launches": 3 * k, "clocks": clk.summary(),
            "mixed": {"value": round(k * N / (m_ms * 1e-3), 1), "unit": "paths/s",
                      "speedup_vs_plain_fp64": round(ms / m_ms, 3), "recall_vs_plain_fp64": round(hits / max(total, 1), 5),
                      "distinct_roots_per_task": {"min": min(m_distinct), "max": max(m_distinct)},
                      "fp64_solve_share": round(st_m["fp64_solves"] / max(m_solves, 1), 4),
                      "handoffs": int(st_m["handoffs"]),
                      "codes": [int(x) for x in np.bincount(mc, minlength=8)]}}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        o = oracle.Oracle()
        m = min(n, args.cpu_paths)
        gam = [_gamma_of(o.uniform01, seeds[0], j) for j in range(T)]
        ppt = [m] * T
        t0 = time.perf_counter()
        o_roots, o_codes, _, _ = o.plugin_batch(cfg.system, tasks, gam, seeds[0], ppt,
                                                cfg=o.config(start_dist=1))
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": round(m * T / dt, 1), "unit": "paths/s", "cores": os.cpu_count() or 1,
                                "kind": "port", "sample": f"first {m} paths of each task of step 0 "
                                                          f"({m * T} paths) by the oracle's tracker, {dt:.2f} s"}
    return line


def run_profile_case(args):
    """The ncu target: one round of the chosen configuration (or plain FP64 with
    --profile-plain) on --profile-paths paths of the workload's first two tasks, one
    call, nothing else launched. Prints the call's counters."""
    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300 import build as frg_build

    frg_build.build()
    wl = Workload(args.workload)
    tasks = wl.tasks[:2] if wl.ntasks >= 2 else wl.tasks
    ppt = [args.profile_paths // len(tasks)] * len(tasks)
    cfg = workload_config(frg, frg.PREC_FP64 if args.profile_plain else frg.PREC_MIXED)
    if not args.profile_plain:
        for key, v in _chosen_overrides(frg).items():
            setattr(cfg, key, v)
    with frg.Tracker(cfg) as t:
        r = t.track(tasks, ppt, SEED_BASE, want_resid=True)
    keys = ("ivp_solves", "newton_iters", "fp64_solves", "refine_solves", "refine_warp_steps", "refine_cycles",
            "track_ms", "stage_ms", "kernel_cycles", "codes")
    print(json.dumps({"profile_case": {"paths": sum(ppt), "plain": bool(args.profile_plain)},
                      **{k: r.stats[k] for k in keys}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", choices=["c5", "c4", "c2"], default="c5")
    ap.add_argument("--cpu-paths", type=int, default=128, help="CPU arms: paths per task of each sampled step")
    ap.add_argument("--depth", type=int, default=4, help="rounds in flight")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-case", action="store_true",
                    help="one chosen-configuration round on --profile-paths paths (an ncu target), nothing else")
    ap.add_argument("--profile-paths", type=int, default=4096)
    ap.add_argument("--profile-plain", action="store_true", help="with --profile-case: plain FP64 instead")
    ap.add_argument("--system", default=None, help="measure a plug-in system (its own JSON line) instead")
    ap.add_argument("--plugin-tasks", type=int, default=64)
    ap.add_argument("--plugin-paths", type=int, default=4096)
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    if args.system:
        print(json.dumps(run_plugin(args)))
        return
    if args.warmup < 0 or args.steps < 1:
        raise SystemExit("need --steps >= 1 and --warmup >= 0")
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
