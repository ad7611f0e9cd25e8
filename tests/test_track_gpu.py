"""Parity of the CUDA tracker with the oracle and the reference's golden paths.

Numerical bar: codes equal path for path; successful roots equal within 1e-8
relative (the reference's FP64 trajectories and ours differ only by rounding);
residual of every successful root <= 1e-10 (row-scaled, Z0 = 1)."""
import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.tasks import REFERENCE_GAMMA, REFERENCE_TARGET, precision_point_task

pytestmark = pytest.mark.gpu

ROOT_RTOL = 1e-8


@pytest.fixture(scope="module", params=[frg.KERNEL_TEAM, frg.KERNEL_THREAD], ids=["team", "thread"])
def tracker(request):
    frg_build.build()
    t = frg.Tracker(frg.default_config(kernel_variant=request.param))
    t.variant = request.param
    yield t
    t.close()


def _rel(a, b):
    return np.max(np.abs(a - b), axis=-1) / np.maximum(np.max(np.abs(b), axis=-1), 1e-300)


def test_reference_paths_path_for_path(tracker, golden):
    """The reference's own paths (host build of its sources, golden vectors)."""
    seed = int(golden["path_seed"][0])
    n = len(golden["path_codes"])
    res = tracker.track(REFERENCE_TARGET, [n], seed, want_yfinal=True, want_resid=True)
    want = golden["path_codes"]
    ok = want == 0
    if tracker.variant == frg.KERNEL_THREAD:
        # the reference's dense LU restated: same codes everywhere
        assert np.array_equal(res.codes, want)
        assert np.all(_rel(res.roots[ok], golden["path_roots"][ok]) < ROOT_RTOL)
    else:
        # structured elimination: rounding differs, the tracked roots do not
        same = (res.codes[ok] == 0) & (_rel(res.roots[ok], golden["path_roots"][ok]) < ROOT_RTOL)
        assert same.mean() >= 0.99
        assert (res.codes == want).mean() >= 0.97
    assert np.all(res.resid[res.codes == 0] <= 1e-10)


def test_random_task_matches_oracle(tracker, oracle):
    fpm = precision_point_task(11, "disk")
    n = 384
    res = tracker.track(fpm, [n], 77, want_resid=True)
    roots, codes, _, _ = oracle.homotopy_batch(fpm, complex(*[0.39231132891081666, 1.0062265257923928]), 77,
                                               np.arange(n))
    # paths the oracle tracks to a root: same root (failing paths near singular
    # endpoints may fail with a different code after rounding-level differences)
    ok = codes == 0
    same = (res.codes[ok] == 0) & (_rel(res.roots[ok], roots[ok]) < ROOT_RTOL)
    assert same.mean() >= 0.99
    assert (res.codes == codes).mean() >= 0.97
    assert np.all(res.resid[res.codes == 0] <= 1e-10)


def test_multi_task_streams(tracker, oracle):
    """Path i of task k uses stream (paths of earlier tasks) + i, each task its own fpm."""
    fpms = np.stack([precision_point_task(s, "disk") for s in (3, 4, 5)])
    ppt = [40, 0, 24]
    res = tracker.track(fpms, ppt, 9)
    assert len(res.codes) == 64
    start = 0
    for k, n in enumerate(ppt):
        if n == 0:
            continue
        r, c, _, _ = oracle.homotopy_batch(fpms[k], REFERENCE_GAMMA, 9, np.arange(start, start + n))
        assert (res.codes[start:start + n] == c).mean() >= 0.95
        ok = (c == 0) & (res.codes[start:start + n] == 0)
        assert (_rel(res.roots[start:start + n][ok], r[ok]) < ROOT_RTOL).mean() >= 0.95
        start += n


def test_device_buffers_match_host(tracker):
    torch = pytest.importorskip("torch")
    n = 64
    host = tracker.track(REFERENCE_TARGET, [n], 5)
    fpm = torch.from_numpy(REFERENCE_TARGET.view(np.float64).copy()).cuda()
    roots = torch.zeros((n, 42), dtype=torch.float64, device="cuda")
    codes = torch.zeros(n, dtype=torch.int32, device="cuda")
    tracker.track_into(fpm, [n], 5, roots, codes)
    assert np.array_equal(codes.cpu().numpy(), host.codes)
    assert np.array_equal(roots.cpu().numpy().view(np.complex128), host.roots)


def test_deterministic(tracker):
    a = tracker.track(REFERENCE_TARGET, [48], 21)
    b = tracker.track(REFERENCE_TARGET, [48], 21)
    assert np.array_equal(a.codes, b.codes) and np.array_equal(a.roots, b.roots)


def test_empty_and_limits(tracker):
    r = tracker.track(REFERENCE_TARGET, [0], 1)
    assert r.roots.shape == (0, 21) and r.stats["paths"] == 0
    v = tracker.variant
    t = frg.Tracker(frg.default_config(max_steps=0, kernel_variant=v))
    assert np.all(t.track(REFERENCE_TARGET, [16], 1).codes == 1)
    t.set_config(frg.default_config(max_ministeps=3, kernel_variant=v))
    assert np.all(t.track(REFERENCE_TARGET, [16], 1).codes == 2)
    for prec in (frg.PREC_MIXED,):
        t.set_config(frg.default_config(max_ministeps=3, kernel_variant=v, precision=prec))
        assert np.all(t.track(REFERENCE_TARGET, [16], 1).codes == 2)
    t.close()


def test_oracle_config_knobs_match(tracker, oracle):
    """Non-default tracker settings (residual type |H|, normal starts) still match the oracle."""
    cfg = frg.default_config(newt_residual=0, start_dist=frg.START_NORMAL, start_range=1.0,
                             kernel_variant=tracker.variant)
    t = frg.Tracker(cfg)
    n = 96
    res = t.track(REFERENCE_TARGET, [n], 3)
    ocfg = oracle.config(newt_residual=0, start_dist=1, start_range=1.0)
    r, c, _, _ = oracle.homotopy_batch(REFERENCE_TARGET, REFERENCE_GAMMA, 3, np.arange(n), cfg=ocfg)
    ok = c == 0
    same = (res.codes[ok] == 0) & (_rel(res.roots[ok], r[ok]) < ROOT_RTOL)
    assert same.mean() >= 0.97
    assert (res.codes == c).mean() >= 0.95
    t.close()


def test_stats_counters(tracker):
    res = tracker.track(REFERENCE_TARGET, [64], 8)
    s = res.stats
    assert s["paths"] == 64 and sum(s["codes"]) == 64
    assert np.bincount(res.codes, minlength=8).tolist() == s["codes"]
    assert s["ivp_solves"] > 64 * 100 and s["newton_iters"] > 0 and s["track_ms"] > 0


def test_team_matches_thread_kernel():
    """The two FP64 kernels (dense LU per thread, structured LU per 8-lane team)
    track the same paths to the same roots."""
    fpm = precision_point_task(12, "disk")
    n = 512
    with frg.Tracker(frg.default_config(kernel_variant=frg.KERNEL_THREAD)) as t:
        a = t.track(fpm, [n], 31, want_resid=True)
    with frg.Tracker(frg.default_config(kernel_variant=frg.KERNEL_TEAM)) as t:
        b = t.track(fpm, [n], 31, want_resid=True)
    ok = a.codes == 0
    same = (b.codes[ok] == 0) & (_rel(b.roots[ok], a.roots[ok]) < ROOT_RTOL)
    assert same.mean() >= 0.99
    assert np.all(b.resid[b.codes == 0] <= 1e-10)


def test_sharded_round_matches_single(tracker):
    """A round split into path ranges (path_offset = the range's first global index,
    every task kept at its global index) reproduces the single round path for path."""
    from finite_root_generation_gb300 import shard

    fpm = np.stack([precision_point_task(5, "disk"), precision_point_task(6, "curve")])
    ppt = [40, 56]
    whole = tracker.track(fpm, ppt, 77)
    cfg0 = tracker.config
    parts = []
    try:
        for r in range(3):
            _, res = shard.track_shard(tracker, fpm, ppt, 77, r, 3, want_resid=False)
            parts.append(res)
    finally:
        cfg0.path_offset = 0
        tracker.set_config(cfg0)
    codes = np.concatenate([p.codes for p in parts])
    roots = np.concatenate([p.roots for p in parts])
    assert np.array_equal(codes, whole.codes)
    assert np.array_equal(roots, whole.roots)
