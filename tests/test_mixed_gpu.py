"""Mixed precision (FP32 stage, FP64 endgame/sharpening) against plain FP64 on the
same tasks and seeds: recall of distinct finite roots, residuals, FP64 share."""
import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.metrics import distinct_roots, recall
from finite_root_generation_gb300.tasks import REFERENCE_TARGET, precision_point_task

pytestmark = pytest.mark.gpu


def _cfg(precision, **kw):
    return frg.default_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8,
                              precision=precision, **kw)


@pytest.fixture(scope="module", params=[frg.KERNEL_TEAM, frg.KERNEL_THREAD], ids=["team", "thread"])
def runs(request):
    frg_build.build()
    task = precision_point_task(1, "disk")
    n = 4096 if request.param == frg.KERNEL_TEAM else 1024
    out = {"n": n}
    for name, prec in (("fp64", frg.PREC_FP64), ("mixed", frg.PREC_MIXED)):
        with frg.Tracker(_cfg(prec, kernel_variant=request.param)) as t:
            out[name] = t.track(task, [n], 4242, want_resid=True)
    return out


def test_mixed_recall_vs_fp64(runs):
    a = distinct_roots(runs["fp64"].roots, runs["fp64"].codes, runs["fp64"].resid)
    b = distinct_roots(runs["mixed"].roots, runs["mixed"].codes, runs["mixed"].resid)
    assert len(a) > 0.9 * runs["n"]
    r = recall(a, b)
    # bench.py reports the full-size recall against the 99.5% target; small samples
    # here only guard against regressions
    assert r >= 0.985, r
    assert len(b) >= 0.985 * len(a)


def test_mixed_residuals(runs):
    res = runs["mixed"]
    ok = res.codes == 0
    assert ok.mean() > 0.9
    assert np.all(res.resid[ok] <= 1e-10)


def test_mixed_uses_fp32_for_most_solves(runs):
    s = runs["mixed"].stats
    total = s["ivp_solves"] + s["newton_iters"]
    # a path may be handed to FP64 and back a bounded number of times (at most 8
    # hand-backs), so hand-offs can exceed the path count but not 9x it
    assert 0 < s["handoffs"] <= 9 * s["paths"]
    assert s["handbacks"] <= 8 * s["paths"]
    assert s["fp64_solves"] < 0.5 * total
    assert runs["fp64"].stats["fp64_solves"] == runs["fp64"].stats["ivp_solves"] + runs["fp64"].stats["newton_iters"]


def test_mixed_reference_target():
    """Mixed precision on the reference's own target and gamma finds the reference's roots."""
    with frg.Tracker(frg.default_config(precision=frg.PREC_MIXED)) as t:
        m = t.track(REFERENCE_TARGET, [512], 1234, want_resid=True)
    with frg.Tracker(frg.default_config()) as t:
        p = t.track(REFERENCE_TARGET, [512], 1234, want_resid=True)
    r = recall(distinct_roots(p.roots, p.codes, p.resid), distinct_roots(m.roots, m.codes, m.resid))
    assert r >= 0.98, r
