"""Parity of the chosen mixed-precision configuration (frg.CHOSEN, the setting the
benchmark measures) at the workload configurations, and of the finite/infinite
classification.

Bars (numerical, written here):
  * a root counts (is kept) only when its path succeeded (code 0) and its row-scaled FP64
    residual is <= 1e-10, so every kept root meets the residual bar; the residual filter
    discards at most 1e-4 of the successful paths;
  * recall of the plain FP64 tracker's distinct finite roots >= 0.995 on the 65,536-path
    and 262,144-path configurations (two exact FP64 trackers already disagree on ~0.4 % of
    paths, those that jump between nearby path branches, so small samples get the looser
    bar 0.99);
  * distance of each kept root to the FP64 track of the same path (same random stream):
    the max-norm relative distance of the two endpoints; >= 99 % of the paths that both
    finish lie within 1e-8 (the rest jumped to another root in one of the two runs).
The oracle (C restatement of the reference tracker) is the FP64 track on the 1,024-path
configuration; the library's plain FP64 kernel, itself pinned path for path to the
oracle and the reference (test_track_gpu.py), is the FP64 track on the larger ones.
"""
import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.metrics import distinct_roots, recall
from finite_root_generation_gb300.tasks import precision_point_task

pytestmark = pytest.mark.gpu

RESID_MAX = 1e-10
ROOT_RTOL = 1e-8
INF_TOL = 1e-8


def _workload(**kw):
    return dict(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=INF_TOL, **kw)


def _gamma(oracle, seed, k):
    """The library's random gamma of task k of a call with `seed`."""
    phi = 2 * np.pi * oracle.uniform01(seed, 2**64 - 1 - k, 0)
    return complex(np.cos(phi), np.sin(phi))


def _distance(a_roots, a_codes, b_roots, b_codes):
    """Relative max-norm distance between the endpoints of the paths both runs finish."""
    both = (a_codes == 0) & (b_codes == 0)
    d = np.max(np.abs(a_roots[both] - b_roots[both]), axis=1) / np.max(np.abs(b_roots[both]), axis=1)
    return both, d


def _residual_filter_ok(res, label):
    """At most 1e-4 of the successful paths fail the residual test (and are not kept)."""
    ok = res.codes == 0
    bad = int(np.sum(~(res.resid[ok] <= RESID_MAX)))
    print(f"{label}: {bad} of {int(ok.sum())} successful paths above the residual bar")
    assert bad <= 1e-4 * ok.sum() + 1, bad


def _track(cfg, tasks, ppt, seed):
    with frg.Tracker(cfg) as t:
        return t.track(tasks, ppt, seed, want_resid=True)


@pytest.fixture(scope="module", autouse=True)
def _built():
    frg_build.build()


def test_c1_chosen_matches_oracle(oracle):
    """1,024 paths on task seed 0, complex-normal starts, random gamma: the chosen
    configuration against the oracle's FP64 tracks on the same Philox streams."""
    task = precision_point_task(0, "disk")
    n, seed = 1024, 2024
    res = _track(frg.chosen_config(**_workload()), task, [n], seed)
    roots, codes, _, yf = oracle.homotopy_batch(task, _gamma(oracle, seed, 0), seed, np.arange(n),
                                                cfg=oracle.config(start_dist=1), want_yfinal=True)
    zmax = np.max(np.abs(yf[:, :21]), axis=1)
    codes = np.where((codes == 0) & (np.abs(yf[:, 21]) < INF_TOL * zmax), 7, codes)
    o_resid = oracle.residuals(roots, task)
    ok = res.codes == 0
    assert ok.mean() > 0.9
    _residual_filter_ok(res, "C1")
    a = distinct_roots(roots, codes, o_resid, RESID_MAX)
    b = distinct_roots(res.roots, res.codes, res.resid, RESID_MAX)
    assert recall(a, b) >= 0.99, recall(a, b)
    both, d = _distance(res.roots, res.codes, roots, codes)
    assert both.sum() > 0.9 * n
    assert np.mean(d <= ROOT_RTOL) >= 0.99, np.sort(d)[-10:]


@pytest.fixture(scope="module")
def c2_runs():
    """65,536 paths on task seed 1 (points in the unit disk), one round, chosen and plain."""
    task = precision_point_task(1, "disk")
    n, seed = 65536, 1
    return (task, _track(frg.chosen_config(**_workload()), task, [n], seed),
            _track(frg.default_config(**_workload()), task, [n], seed))


def test_c2_chosen_recall_and_residuals(c2_runs):
    task, ch, pl = c2_runs
    _residual_filter_ok(ch, "C2")
    a = distinct_roots(pl.roots, pl.codes, pl.resid, RESID_MAX)
    b = distinct_roots(ch.roots, ch.codes, ch.resid, RESID_MAX)
    r = recall(a, b)
    print(f"C2: plain {len(a)} distinct, chosen {len(b)}, recall {r:.5f}")
    assert r >= 0.995, r


def test_c2_distance_to_fp64_track(c2_runs):
    """Each kept root against the FP64 track of the same path."""
    task, ch, pl = c2_runs
    both, d = _distance(ch.roots, ch.codes, pl.roots, pl.codes)
    near = d <= ROOT_RTOL
    print(f"C2: {both.sum()} paths finish in both; {near.mean():.5f} within 1e-8 of the FP64 track, "
          f"median distance {np.median(d):.2e}, 99th percentile of those within {np.quantile(d[near], 0.99):.2e}")
    assert both.sum() > 0.9 * len(ch.codes)
    assert near.mean() >= 0.99


def test_c3_near_degenerate_tasks():
    """262,144 paths over 10 tasks, one of them near-degenerate (precision points within
    1e-3 of a centre): recall of plain FP64's distinct roots and residuals, per task kind."""
    tasks = np.stack([precision_point_task(300, "degenerate")] + [precision_point_task(301 + k, "disk")
                                                                  for k in range(9)])
    ppt = [26215, 26215] + [26214] * 8
    seed = 33
    ch = _track(frg.chosen_config(**_workload()), tasks, ppt, seed)
    pl = _track(frg.default_config(**_workload()), tasks, ppt, seed)
    _residual_filter_ok(ch, "C3")
    starts = np.concatenate([[0], np.cumsum(ppt)])
    hits = total = 0
    for k in range(len(ppt)):
        sl = slice(starts[k], starts[k + 1])
        a = distinct_roots(pl.roots[sl], pl.codes[sl], pl.resid[sl], RESID_MAX)
        b = distinct_roots(ch.roots[sl], ch.codes[sl], ch.resid[sl], RESID_MAX)
        r = recall(a, b)
        if k == 0:
            print(f"C3 near-degenerate task: plain {len(a)} distinct, chosen {len(b)}, recall {r:.5f}")
        hits += round(r * len(a))
        total += len(a)
    print(f"C3 all tasks: recall {hits / total:.5f} of {total}")
    assert hits / total >= 0.995


@pytest.mark.parametrize("variant", [frg.KERNEL_TEAM, frg.KERNEL_THREAD], ids=["team", "thread"])
def test_infinite_root_classification(oracle, variant):
    """Code 7 (infinite root) exactly when |Z0| < inf_tol max|Z| at the tracked endpoint of
    a successful path, on the device's own endpoints, and the same decisions as the
    oracle's endpoints of the same paths. On this system a path that runs to infinity
    (|Z0| -> 0) nearly always fails sharpening (code 5) first -- the oracle ends 154 of 512
    paths of this physical-mechanism task (Pc = conj(P), |Q| = 1) that way -- so the test
    uses inf_tol = 0.02, which splits the successful endpoints (|Z0|/max|Z| from 0.0024
    up), to exercise the decision itself."""
    tol = 0.02
    task = precision_point_task(7, "real")
    n, seed = 512, 91
    cfg = frg.default_config(inf_tol=tol, kernel_variant=variant)
    with frg.Tracker(cfg) as t:
        res = t.track(task, [n], seed, want_yfinal=True)
    yf = res.yfinal
    rule = np.abs(yf[:, 21]) < tol * np.max(np.abs(yf[:, :21]), axis=1)
    fin = np.isin(res.codes, [0, 7])
    assert np.array_equal(res.codes[fin] == 7, rule[fin])
    assert (res.codes == 7).sum() > 0 and (res.codes == 0).sum() > 0
    _, o_codes, _, o_yf = oracle.homotopy_batch(task, complex(cfg.gamma_re, cfg.gamma_im), seed, np.arange(n),
                                                want_yfinal=True)
    o_rule = np.abs(o_yf[:, 21]) < tol * np.max(np.abs(o_yf[:, :21]), axis=1)
    both = fin & (o_codes == 0)
    agree = (res.codes[both] == 7) == o_rule[both]
    assert both.sum() > 0.5 * (o_codes == 0).sum()
    assert agree.mean() >= 0.99, (agree.mean(), both.sum())
