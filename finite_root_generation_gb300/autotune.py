"""Autotuner for the tracker's launch and precision settings.

For one workload (a task and a round size) it times every candidate setting on a
sample of rounds, keeps those whose distinct finite roots recall at least
`target_recall` of the plain FP64 tracker's on the same seeds (the plain tracker is
the reference point), picks the highest distinct-roots-per-second, re-checks that choice on
fresh seeds, and caches it per GPU model and workload in a JSON file.

Searched dimensions (each a field of frg_config, or the rounds in flight of
frg_track_rounds):
  kernel_variant  paths per warp: 4 (8-lane teams) or 32 (one path per thread)
  blocks_per_sm   resident blocks per SM (0 = the occupancy maximum)
  precision       FP64, or mixed with the FP32 stage's point type lo_points 0/1
  cond_switch     the condition estimate above which a step goes to FP64
  fp64_budget     FP64 solves a path may spend before it is ended
  depth           rounds in flight
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

DEFAULT_SPACE = {
    "kernel_variant": [KERNEL_TEAM],
    "blocks_per_sm": [0],
    "precision": [PREC_MIXED],
    "lo_points": [0, 1],
    "cond_switch": [1e5, 1e6],
    "fp64_budget": [0, 10000],
    "depth": [2, 4],
}


def _cache_path(path=None):
    if path:
        return path
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "frg_gb300", "autotune.json")


def _key(device_name, task, n, base_overrides):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(task, np.complex128).tobytes())
    h.update(json.dumps(base_overrides, sort_keys=True).encode())
    return f"{device_name}|n={n}|{h.hexdigest()[:16]}"


def _run(cfg_kw, task, n, seeds, depth, device):
    cfg = default_config(**cfg_kw)
    k = len(seeds)
    roots = np.zeros((k * n, 21), np.complex128)
    codes = np.zeros(k * n, np.int32)
    resid = np.zeros(k * n, np.float64)
    with Tracker(cfg, device=device) as t:
        t.track(task, [min(n, 1024)], 1)  # warm-up
        st = t.track_rounds(task, [n], seeds, roots, codes, resid=resid, depth=depth)
    sets = [distinct_roots(roots[i * n:(i + 1) * n], codes[i * n:(i + 1) * n], resid[i * n:(i + 1) * n])
            for i in range(k)]
    return sets, st["track_ms"]


def autotune(task, n=8192, rounds=2, base=None, space=None, target_recall=0.995, device=0, cache=None,
             device_name=None, retune=False, log=None):
    """Return the best setting (dict of frg_config fields plus 'depth') for `task` at
    `n` paths per round; `base` holds fixed config fields of the workload."""
    base = dict(base or {})
    space = dict(DEFAULT_SPACE if space is None else space)
    if device_name is None:
        try:
            import torch
            device_name = torch.cuda.get_device_name(device)
        except Exception:  # noqa: BLE001 - the name only keys the cache
            device_name = "cuda"
    path = _cache_path(cache)
    key = _key(device_name, task, n, base)
    store = {}
    if os.path.exists(path):
        with open(path) as f:
            store = json.load(f)
    if key in store and not retune:
        return store[key]["best"]

    seeds = [1000 + i for i in range(rounds)]
    ref_sets, ref_ms = _run(dict(base, precision=PREC_FP64), task, n, seeds, 2, device)
    ref_rate = sum(len(s) for s in ref_sets) / (ref_ms * 1e-3)
    names = list(space)
    results = []
    for values in itertools.product(*(space[k] for k in names)):
        cand = dict(zip(names, values))
        if cand.get("precision") == PREC_FP64 and (cand.get("lo_points", 0) or cand.get("cond_switch", 1e5) != 1e5
                                                  or cand.get("fp64_budget", 0)):
            continue  # FP64 ignores the mixed-precision fields
        if cand.get("kernel_variant") == KERNEL_THREAD and cand.get("lo_points", 0):
            continue  # the point type option exists for the team kernels only
        depth = cand.pop("depth", 2)
        t0 = time.perf_counter()
        sets, ms = _run(dict(base, **cand), task, n, seeds, depth, device)
        rec = min(recall(ref_sets[i], sets[i]) for i in range(rounds))
        rate = sum(len(s) for s in sets) / (ms * 1e-3)
        entry = {"setting": dict(cand, depth=depth), "roots_per_s": rate, "recall": rec,
                 "wall_s": time.perf_counter() - t0}
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
        r_sets, _ = _run(dict(base, precision=PREC_FP64), task, n, fresh, 2, device)
        c_sets, _ = _run(dict(base, **fb), task, n, fresh, best["depth"], device)
        check = {"recall": min(recall(r_sets[i], c_sets[i]) for i in range(rounds))}
        if check["recall"] < target_recall:
            best = {"precision": PREC_FP64, "depth": 2}
    store[key] = {"best": best, "plain_fp64_roots_per_s": ref_rate, "candidates": results,
                  "revalidation": check, "target_recall": target_recall}
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(store, f, indent=1)
    return best
