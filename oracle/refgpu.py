"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

The reference's own CUDA tracker on this GPU: its kernels InitRandStates and Homotopy
(frg.cu:30-124) compiled unchanged (``make -C oracle refgpu`` from the staged reference
sources in oracle/_ref/src) and launched by ``oracle/ref_gpu_driver.cu``. Two builds:
``curand`` (the reference's XORWOW streams, as shipped) and ``philox`` (the CUDA
tracker's Philox streams through oracle/ref_stub/curand_kernel.h, so its paths can be
compared with the tracker's path for path).

The reference kernel hard-codes its gamma (frg.cu:41) and draws start mechanisms
uniformly from (-5, 5)^2 (frgkinematics.cu:7-8): the tracker's default configuration.

    python oracle/refgpu.py [--paths 65536] [--seed 1]

runs the 65,536-path single-task comparison (task seed 1, points in the unit disk):
the reference's GPU tracker (both builds) against the CUDA tracker's plain FP64 and
chosen mixed-precision configurations on the same GPU, and prints one JSON line with
throughput, distinct finite roots and path-for-path agreement.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIBS = {"curand": os.path.join(REF_DIR, "librefgpu.so"), "philox": os.path.join(REF_DIR, "librefgpu_philox.so")}


def build(jobs: int | None = None) -> None:
    """Build both GPU libraries from the staged reference sources (make refgpu)."""
    sys.path.insert(0, HERE)
    import oracle
    if not oracle.ref_sources_staged():
        raise RuntimeError("the reference sources are not staged in oracle/_ref/src (make -C oracle stage REF=...)")
    subprocess.run(["make", "-s", "-C", HERE, f"-j{jobs or os.cpu_count() or 1}", "refgpu"], check=True)


class RefGPU:
    """One build of the reference's GPU tracker (``curand`` or ``philox``)."""

    def __init__(self, kind: str = "philox"):
        if not os.path.exists(LIBS[kind]):
            build()
        self.lib = ctypes.CDLL(LIBS[kind])
        self.lib.refgpu_track.restype = ctypes.c_int
        self.lib.refgpu_track.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_longlong, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_char_p,
                                          ctypes.c_int]
        self.kind = kind

    def track(self, fpm, seed: int, npaths: int):
        """roots [n, 21] complex, codes [n], (ms kernels, ms kernels + copies)."""
        fpm = np.ascontiguousarray(np.asarray(fpm, np.complex128).reshape(30))
        roots = np.zeros((npaths, 21), np.complex128)
        codes = np.zeros(npaths, np.int32)
        ms = (ctypes.c_float * 2)()
        err = ctypes.create_string_buffer(128)
        st = self.lib.refgpu_track(fpm.ctypes.data, ctypes.c_ulonglong(seed), ctypes.c_longlong(npaths),
                                   roots.ctypes.data, codes.ctypes.data, ms, err, 128)
        if st != 0:
            raise RuntimeError(f"reference GPU tracker failed: {err.value.decode()} ({st})")
        return roots, codes, (float(ms[0]), float(ms[1]))


def _distinct(roots, codes, resid, dup_tol=1e-6):
    """Distinct finite roots with the oracle's restatement of SortingDeletingMerging (the
    reference's own reads past its order vector, frgsupport.cu:195)."""
    import oracle
    good = (codes == 0) & (resid <= 1e-10)
    c = np.where(good, 0, 5).astype(np.int32)
    coll, _ = oracle.Oracle().sort_merge(np.zeros((0, 21), np.complex128), roots, c, dup_tol)
    return coll


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--paths", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--task-seed", type=int, default=1)
    args = ap.parse_args()
    root = os.path.dirname(HERE)
    sys.path.insert(0, root)
    sys.path.insert(0, HERE)
    import oracle
    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300.metrics import recall
    from finite_root_generation_gb300.tasks import precision_point_task

    oracle.build(ref=True)
    build()
    ref = oracle.RefLib()
    task = precision_point_task(args.task_seed, "disk")
    n = args.paths
    out = {"paths": n, "task": f"precision-point task seed {args.task_seed} (unit disk)", "seed": args.seed,
           "config": "reference kernel: gamma frg.cu:41, starts U(-5,5)^2; tracker: the same (default config)"}
    runs = {}
    for kind in ("curand", "philox"):
        g = RefGPU(kind)
        g.track(task, args.seed, 256)  # warm-up (module load, stack reservation)
        roots, codes, ms = g.track(task, args.seed, n)
        resid = ref.residuals(roots, task)
        coll = _distinct(roots, codes, resid)
        runs[kind] = (roots, codes, resid)
        out[f"reference_gpu_{kind}"] = {
            "ms_kernels": round(ms[0], 1), "ms_with_copies": round(ms[1], 1),
            "paths_per_s": round(n / (ms[1] * 1e-3), 1), "codes": np.bincount(codes, minlength=8).tolist(),
            "distinct": len(coll), "distinct_roots_per_s": round(len(coll) / (ms[1] * 1e-3), 1)}
    r_roots, r_codes, r_resid = runs["philox"]
    for name, cfg in (("plain_fp64", frg.default_config()), ("chosen", frg.chosen_config())):
        with frg.Tracker(cfg) as t:
            t.track(task, [1024], 99)  # warm-up
            t0 = time.perf_counter()
            res = t.track(task, [n], args.seed, want_resid=True)
            dt = time.perf_counter() - t0
        coll = _distinct(res.roots, res.codes, res.resid)
        both = (res.codes == 0) & (r_codes == 0)
        d = np.max(np.abs(res.roots[both] - r_roots[both]), axis=1) / np.max(np.abs(r_roots[both]), axis=1)
        ref_coll = _distinct(r_roots, r_codes, r_resid)
        out[name] = {"ms_track": round(res.stats["track_ms"], 1), "ms_total": round(dt * 1e3, 1),
                     "paths_per_s": round(n / dt, 1), "codes": np.bincount(res.codes, minlength=8).tolist(),
                     "distinct": len(coll), "distinct_roots_per_s": round(len(coll) / dt, 1),
                     "same_code_as_reference_gpu": round(float(np.mean(res.codes == r_codes)), 5),
                     "same_root_1e-8_of_both_successful": round(float(np.mean(d <= 1e-8)), 5),
                     "recall_of_reference_gpu_distinct": round(recall(ref_coll, coll), 5)}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
