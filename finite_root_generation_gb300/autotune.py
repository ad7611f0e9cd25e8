"""Autotuner for the tracker's launch and precision settings.

For one workload (a task set, paths per task, rounds) it times every candidate setting
on a sample of pipelined rounds, keeps those whose distinct finite roots recall at least
`target_recall` of the plain FP64 tracker's on the same seeds (the plain tracker is the
reference point), picks the highest distinct-roots-per-second, re-checks that choice on
fresh seeds, and caches it per GPU model and workload in a JSON file.

Searched dimensions (each a field of frg_config, a bundle of fields, or the rounds in
flight of frg_track_rounds):
  kernel_variant  paths per warp: 4 (8-lane teams) or 32 (one path per thread)
  blocks_per_sm   resident blocks per SM (0 = the occupancy maximum)
  precision       FP64, or mixed with the FP32 stage's point type lo_points 0/1
  cond_switch     the condition estimate above which a step goes to FP64
  fp64_budget     FP64 solves a path may spend before it is ended
  carry_handback  paths well conditioned again return from FP64 to a later round's FP32
  corrector       the FP32 stage's corrector: always refine on double-float residuals, or
                  accept an FP32 update below 1e-6 first (lo_refine 1 / 3)
  depth           rounds in flight
A dimension whose values are dicts is a bundle: each value's fields are set together.

The register cap of the FP32 stage is a compile-time choice (FRG_LO_MIN_BLOCKS); it was
measured once rather than searched: capping it for 5 resident blocks per SM spills ~1.8 KB
per thread and is slower than 4 blocks.

`TUNED` (tuned.json next to this file) holds the entries this tuner wrote on the GPUs the
project measured on; `tuned_setting` reads it, so a benchmark can use the tuner's choice
without re-tuning on every fresh machine.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
import time

import numpy as np

from . import PREC_FP64, PREC_MIXED, KERNEL_TEAM, KERNEL_THREAD, Tracker, default_config
from .metrics import distinct_roots, recall

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED = os.path.join(HERE, "tuned.json")

DEFAULT_SPACE = {
    "kernel_variant": [KERNEL_TEAM],
    "precision": [PREC_MIXED],
    "lo_points": [1],
    "cond_switch": [1e5, 5e5, 1e6],
    "carry_handback": [0, 1],
    "corrector": [{"lo_refine": 1}, {"lo_refine": 3, "newt_tol_lo": 1e-6}],
    "depth": [4],
}


def _cache_path(path=None):
    if path:
        return path
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "frg_gb300", "autotune.json")


def _key(device_name, tasks, n, rounds, base_overrides, space):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(tasks, np.complex128).tobytes())
    h.update(json.dumps(base_overrides, sort_keys=True).encode())
    h.update(json.dumps(space, sort_keys=True, default=str).encode())
    return f"{device_name}|n={n}|rounds={rounds}|{h.hexdigest()[:16]}"


def _run(cfg_kw, tasks, n, seeds, depth, device):
    """Pipelined rounds of the task set (n paths per task); per-round distinct roots per
    task and the tracking time."""
    cfg = default_config(**cfg_kw)
    k, T = len(seeds), len(tasks)
    N = n * T
    roots = np.zeros((k * N, 21), np.complex128)
    codes = np.zeros(k * N, np.int32)
    resid = np.zeros(k * N, np.float64)
    with Tracker(cfg, device=device) as t:
        t.track(tasks, [min(n, 256)] * T, 1)  # warm-up
        st = t.track_rounds(tasks, [n] * T, seeds, roots, codes, resid=resid, depth=depth)
    sets = []
    for i in range(k):
        for j in range(T):
            sl = slice(i * N + j * n, i * N + (j + 1) * n)
            sets.append(distinct_roots(roots[sl], codes[sl], resid[sl]))
    return sets, st["track_ms"]


def _flatten(cand):
    out = {}
    for k, v in cand.items():
        if isinstance(v, dict):
            out.update(v)
        else:
            out[k] = v
    return out


def _recall(ref_sets, sets):
    hits = total = 0
    for a, b in zip(ref_sets, sets):
        hits += round(recall(a, b) * len(a))
        total += len(a)
    return hits / max(total, 1)


def autotune(tasks, n=8192, rounds=2, base=None, space=None, target_recall=0.995, device=0, cache=None,
             device_name=None, retune=False, log=None):
    """Return the best setting (dict of frg_config fields plus 'depth') for the task set
    `tasks` ([T, 30] complex, or one task) at `n` paths per task and round, over `rounds`
    pipelined rounds; `base` holds fixed config fields of the workload."""
    tasks = np.asarray(tasks, np.complex128).reshape(-1, 30)
    base = dict(base or {})
    space = dict(DEFAULT_SPACE if space is None else space)
    if device_name is None:
        try:
            import torch
            device_name = torch.cuda.get_device_name(device)
        except Exception:  # noqa: BLE001 - the name only keys the cache
            device_name = "cuda"
    path = _cache_path(cache)
    key = _key(device_name, tasks, n, rounds, base, space)
    store = {}
    if os.path.exists(path):
        with open(path) as f:
            store = json.load(f)
    if key in store and not retune:
        return store[key]["best"]

    seeds = [1000 + i for i in range(rounds)]
    # plain FP64 with as many rounds in flight as the candidates (the largest depth searched)
    ref_depth = max(space.get("depth", [2]))
    ref_sets, ref_ms = _run(dict(base, precision=PREC_FP64), tasks, n, seeds, ref_depth, device)
    ref_rate = sum(len(s) for s in ref_sets) / (ref_ms * 1e-3)
    names = list(space)
    results = []
    for values in itertools.product(*(space[k] for k in names)):
        cand = _flatten(dict(zip(names, values)))
        mixed_only = ("lo_points", "cond_switch", "fp64_budget", "carry_handback", "lo_refine", "newt_tol_lo")
        if cand.get("precision") == PREC_FP64 and any(k in cand for k in mixed_only):
            continue  # FP64 ignores the mixed-precision fields
        if cand.get("kernel_variant") == KERNEL_THREAD and (cand.get("lo_points", 0) or cand.get("carry_handback")):
            continue  # these options exist for the team kernels only
        depth = cand.pop("depth", 2)
        t0 = time.perf_counter()
        sets, ms = _run(dict(base, **cand), tasks, n, seeds, depth, device)
        rec = _recall(ref_sets, sets)
        rate = sum(len(s) for s in sets) / (ms * 1e-3)
        entry = {"setting": dict(cand, depth=depth), "roots_per_s": rate, "recall": rec,
                 "speedup_vs_plain_fp64": rate / ref_rate, "wall_s": time.perf_counter() - t0}
        results.append(entry)
        if log:
            log(entry)
    ok = [r for r in results if r["recall"] >= target_recall]
    if not ok:
        best = {"precision": PREC_FP64, "depth": 2}
        check = {"recall": 1.0}
    else:
        best = max(ok, key=lambda r: r["roots_per_s"])["setting"]
        # re-validate the choice on fresh seeds
        fresh = [5000 + i for i in range(rounds)]
        fb = {k: v for k, v in best.items() if k != "depth"}
        r_sets, _ = _run(dict(base, precision=PREC_FP64), tasks, n, fresh, ref_depth, device)
        c_sets, _ = _run(dict(base, **fb), tasks, n, fresh, best["depth"], device)
        check = {"recall": _recall(r_sets, c_sets)}
        if check["recall"] < target_recall:
            best = {"precision": PREC_FP64, "depth": 2}
    store[key] = {"best": best, "plain_fp64_roots_per_s": ref_rate, "candidates": results,
                  "revalidation": check, "target_recall": target_recall}
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(store, f, indent=1)
    return best


def tuned_setting(device_name, workload, path=TUNED):
    """The tuner's recorded choice for `workload` on a GPU named `device_name` (the table
    tuned.json: {gpu name: {workload: {"best": setting, ...}}}), or None."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        table = json.load(f)
    for gpu, entries in table.items():
        if gpu in device_name and workload in entries:
            return dict(entries[workload]["best"])
    return None


def _main(argv=None):
    """Tune the 128-task workload's settings on this GPU and record the choice in tuned.json:
    the first round's task set (task seeds 0..7, points in the unit disk / along a closed
    curve, alternating), --paths-per-task paths each, --rounds pipelined rounds."""
    import argparse

    from . import GAMMA_RANDOM, START_NORMAL
    from .tasks import precision_point_task

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c5")
    ap.add_argument("--paths-per-task", type=int, default=4096)
    ap.add_argument("--rounds", type=int, default=8)
    ap.add_argument("--table", default=TUNED)
    ap.add_argument("--space", default=None, help="search space as JSON (default: DEFAULT_SPACE)")
    ap.add_argument("--target", type=float, default=0.995, help="recall target against plain FP64")
    args = ap.parse_args(argv)
    space = json.loads(args.space) if args.space else None
    import torch

    tasks = np.stack([precision_point_task(k, "disk" if k % 2 == 0 else "curve") for k in range(8)])
    base = dict(start_dist=START_NORMAL, gamma_mode=GAMMA_RANDOM, inf_tol=1e-8, mixed_rounds=1, lo_endgame=1,
                fp64_budget=10000, handback_good=32, fp64_segment=256, round_graph=1)
    seen = []
    best = autotune(tasks, n=args.paths_per_task, rounds=args.rounds, base=base, space=space,
                    target_recall=args.target, cache=args.table + ".cache", retune=True,
                    log=lambda e: (seen.append(e), print(json.dumps(e), flush=True)))
    gpu = torch.cuda.get_device_name(0)
    table = {}
    if os.path.exists(args.table):
        with open(args.table) as f:
            table = json.load(f)
    table.setdefault(gpu, {})[args.workload] = {
        "best": best, "base": base, "paths_per_task": args.paths_per_task, "rounds": args.rounds,
        "target_recall": args.target,
        "tasks": "seeds 0..7, unit disk / closed curve alternating", "candidates": seen}
    with open(args.table, "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps({"gpu": gpu, "best": best}))


if __name__ == "__main__":
    _main()
