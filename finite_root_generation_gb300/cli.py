"""Multi-round driver: the reference's `frg <nRounds>` program (frg.cu:128-553) on top of
the C ABI.

Each round tracks N paths from fresh random start mechanisms, merges the roots into the
sorted root collection (duplicates marked code 6), rewrites `fptColl`, appends the
round's codes to `errorCodesAgr` and appends the round's statistics to `progress`, in
the reference's file formats and progress-file sections (frg.cu:440-512). An existing
`fptColl` / `errorCodesAgr` in the output directory is resumed (frg.cu:295-336).
Additions: rounds are tracked `--depth` at a time with frg_track_rounds (pipelined),
the precision and task are options, and `--stop-at` ends the run once the Lambert-W
estimate of the share of roots collected (frg.cu:463-464) reaches it.

    python -m finite_root_generation_gb300.cli --rounds 10 --paths 65536 --dir run1
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

from . import (PREC_FP64, PREC_MIXED, START_NORMAL, START_UNIFORM, GAMMA_FIXED, GAMMA_RANDOM, Collection,
               codes_append, default_config, estimate_collected, Tracker)
from .tasks import REFERENCE_TARGET, precision_point_task


class Totals:
    """Running code counts (successes 0, tracking errors 1..5, duplicates 6)."""

    def __init__(self):
        self.counts = np.zeros(8, np.int64)

    def add(self, codes):
        self.counts += np.bincount(np.clip(np.asarray(codes, np.int64), 0, 7), minlength=8)

    @property
    def successes(self):
        return int(self.counts[0])

    @property
    def duplicates(self):
        return int(self.counts[6])

    @property
    def errors(self):
        return [int(c) for c in self.counts[1:6]]

    @property
    def trials(self):
        return int(self.counts.sum())


def progress_block(rnd, total, per_round, n, t_track, t_merge, t_write):
    """One round's section of the progress file (the reference's layout, frg.cu:486-511)."""
    s = total.successes
    d = total.duplicates
    ratio = s / (s + d) if s + d > 0 else 1.0
    est = estimate_collected(s, d)
    e, er = total.errors, per_round.errors
    lines = [f"-----Progress statistics for round {rnd}-----", "",
             "---In Total---",
             f"Roots collected:{s:>10}",
             f"Duplicates:     {d:>10}",
             f"Trials:         {total.trials:>10}",
             f"Tracking errors:{sum(e):>10}    ({' '.join(str(x) for x in e)})", "",
             "---Per Round---",
             f"Roots collected:{per_round.successes:>10}",
             f"Duplicates:     {per_round.duplicates:>10}",
             f"Trials:         {n:>10}",
             f"Tracking errors:{sum(er):>10}    ({' '.join(str(x) for x in er)})", "",
             "---Progress---",
             f"Success ratio:          {ratio:>10.6g}",
             f"Roots collected (est.): {est * 100:>10.6g}%", "",
             "--- Timing ---",
             f"Tracking:                   {t_track:>10.6g} sec",
             f"Sorting, del. dup., merging:{t_merge:>10.6g} sec",
             f"Writing to disk:            {t_write:>10.6g} sec", "", ""]
    return "\n".join(lines) + "\n", est


def run(track_rounds, n, rounds, outdir, first_round=1, seed0=None, depth=2, stop_at=None, dup_tol=1e-6,
        log=print):
    """Drive `rounds` rounds. track_rounds(seeds) -> (roots [k*n, 21], codes [k*n]) tracks one
    batch of rounds. Returns the number of rounds done."""
    os.makedirs(outdir, exist_ok=True)
    coll_path = os.path.join(outdir, "fptColl")
    codes_path = os.path.join(outdir, "errorCodesAgr")
    prog_path = os.path.join(outdir, "progress")
    coll = Collection(dup_tol)
    total = Totals()
    done_before = 0
    if os.path.exists(coll_path):
        coll.load(coll_path)
    if os.path.exists(codes_path):
        prior = np.fromfile(codes_path, dtype=np.int32)
        total.add(prior)
        done_before = len(prior) // n if n else 0
    if seed0 is None:
        seed0 = time.time_ns() & 0xFFFFFFFF
    r = 0
    while r < rounds:
        k = min(depth, rounds - r)
        seeds = [seed0 + done_before + r + i for i in range(k)]
        t0 = time.perf_counter()
        roots, codes = track_rounds(seeds)
        t_track = (time.perf_counter() - t0) / k
        for i in range(k):
            t1 = time.perf_counter()
            c = coll.merge(roots[i * n:(i + 1) * n], codes[i * n:(i + 1) * n])
            t_merge = time.perf_counter() - t1
            t2 = time.perf_counter()
            coll.save(coll_path)
            codes_append(codes_path, c)
            t_write = time.perf_counter() - t2
            per = Totals()
            per.add(c)
            total.add(c)
            block, est = progress_block(first_round + done_before + r + i, total, per, n, t_track, t_merge, t_write)
            with open(prog_path, "a") as f:
                f.write(block)
            if log:
                log(f"round {first_round + done_before + r + i}: {len(coll)} roots collected, "
                    f"estimated {est * 100:.2f}% of all")
            if stop_at is not None and est >= stop_at:
                return r + i + 1
        r += k
    return rounds


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--rounds", type=int, required=True)
    ap.add_argument("--paths", type=int, default=20480, help="paths per round (the reference: 80 x 256)")
    ap.add_argument("--dir", default=".")
    ap.add_argument("--task-seed", type=int, default=None, help="generic task from this seed (default: the "
                                                                "reference's hard-coded target)")
    ap.add_argument("--task-kind", default="disk")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--normal-starts", action="store_true", help="complex-normal start values")
    ap.add_argument("--random-gamma", action="store_true")
    ap.add_argument("--seed", type=int, default=None, help="first round's seed (default: the clock)")
    ap.add_argument("--depth", type=int, default=2, help="rounds tracked at a time")
    ap.add_argument("--stop-at", type=float, default=None, help="stop at this estimated share collected")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    task = REFERENCE_TARGET if a.task_seed is None else precision_point_task(a.task_seed, a.task_kind)
    kw = dict(start_dist=START_NORMAL if a.normal_starts else START_UNIFORM,
              gamma_mode=GAMMA_RANDOM if a.random_gamma else GAMMA_FIXED)
    if a.precision == "mixed":
        kw.update(precision=PREC_MIXED, lo_endgame=1, lo_points=1, fp64_budget=10000)
    else:
        kw.update(precision=PREC_FP64)
    n = a.paths
    with Tracker(default_config(**kw), device=a.device) as t:
        def track_rounds(seeds):
            roots = np.zeros((len(seeds) * n, 21), np.complex128)
            codes = np.zeros(len(seeds) * n, np.int32)
            t.track_rounds(task, [n], seeds, roots, codes, depth=len(seeds))
            return roots, codes

        done = run(track_rounds, n, a.rounds, a.dir, seed0=a.seed, depth=a.depth, stop_at=a.stop_at)
    print(f"{done} rounds done")


if __name__ == "__main__":
    main()
