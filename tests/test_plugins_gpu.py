"""System plug-ins on the GPU: the CUDA thread kernel instantiated on the generated
systems against the oracle's tracker on the same random streams, path for path, and the
plug-ins' known answers.

Bars: codes equal on >= 99 % of the paths; where both succeed, roots within 1e-8
relative on >= 99 % of the paths (the oracle and the kernel round differently: FMA
contraction and the order of the complex products); every successful root's row-scaled
FP64 residual <= 1e-10 but at most 1e-3 of them; the known roots found. Endpoints with
|Z0| < 1e-8 max|Z| are infinite roots (code 7; the oracle's endpoints classified by the
same rule): burmester5's physical tasks have solutions at infinity, which sharpening
reaches in homogeneous coordinates (|Z0| / max|Z| ~ 1e-34) and which are no finite roots.
"""
import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.metrics import distinct_rows, recall
from finite_root_generation_gb300.systems import burmester5, conic2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    frg_build.build()


def _gammas(oracle, seed, ntasks):
    """The library's random gamma of each task of a call with `seed`."""
    phi = 2 * np.pi * np.array([oracle.uniform01(seed, 2**64 - 1 - k, 0) for k in range(ntasks)])
    return np.exp(1j * phi)


INF_TOL = 1e-8


def _compare(oracle, name, tasks, ppt, seed, start_dist):
    cfg = frg.plugin_config(name, start_dist=start_dist, gamma_mode=frg.GAMMA_RANDOM, inf_tol=INF_TOL)
    sid = cfg.system
    with frg.Tracker(cfg) as t:
        res = t.track(tasks, ppt, seed, want_resid=True)
    o_roots, o_codes, o_resid, o_yf = oracle.plugin_batch(sid, tasks, _gammas(oracle, seed, len(ppt)), seed, ppt,
                                                          cfg=oracle.config(start_dist=start_dist), want_yfinal=True)
    nv = o_roots.shape[1]
    at_inf = np.abs(o_yf[:, nv]) < INF_TOL * np.max(np.abs(o_yf[:, :nv]), axis=1)
    o_codes = np.where((o_codes == 0) & at_inf, 7, o_codes)
    agree = np.mean(res.codes == o_codes)
    both = (res.codes == 0) & (o_codes == 0)
    rel = np.max(np.abs(res.roots[both] - o_roots[both]), axis=1) / np.max(np.abs(o_roots[both]), axis=1)
    ok = res.codes == 0
    bad = int(np.sum(~(res.resid[ok] <= 1e-10)))
    print(f"{name}: {len(res.codes)} paths, codes agree {agree:.4f}, {both.sum()} both succeed, "
          f"{np.mean(rel <= 1e-8):.4f} within 1e-8 (max {rel.max():.2e}), {bad} above the residual bar, "
          f"track {res.stats['track_ms']:.1f} ms")
    assert agree >= 0.99
    assert np.mean(rel <= 1e-8) >= 0.99
    assert bad <= 1e-3 * ok.sum()
    return res, o_roots, o_codes


@pytest.mark.parametrize("start_dist", [frg.START_UNIFORM, frg.START_NORMAL])
def test_conic2_matches_oracle_and_known_roots(oracle, start_dist):
    rng = np.random.default_rng(21)
    q_known, known = conic2.line_pair_task(rng.normal(size=4) + 1j * rng.normal(size=4),
                                           rng.normal(size=4) + 1j * rng.normal(size=4))
    q_rand = rng.normal(size=12) + 1j * rng.normal(size=12)
    tasks = np.stack([q_known, q_rand])
    res, _, _ = _compare(oracle, "conic2", tasks, [512, 512], 5, start_dist)
    ok = res.codes[:512] == 0
    found = distinct_rows(res.roots[:512], ok)
    assert len(found) == 4
    for r in found:
        assert np.min(np.max(np.abs(known - r), axis=1)) <= 1e-10


def test_burmester5_matches_oracle_and_finds_four_dyads(oracle):
    tasks = np.stack([burmester5.physical_task(np.random.default_rng(s)) for s in (5, 6)])
    res, _, _ = _compare(oracle, "burmester5", tasks, [2048, 2048], 17, frg.START_NORMAL)
    for k in range(2):
        sl = slice(2048 * k, 2048 * (k + 1))
        dyads = distinct_rows(res.roots[sl], (res.codes[sl] == 0) & (res.resid[sl] <= 1e-10))
        assert len(dyads) == 4, dyads


def test_plugin_rounds_match_single_calls():
    """frg_track_rounds on a plug-in: each round equals frg_track with that round's seed."""
    cfg = frg.plugin_config("burmester5", start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM)
    task = burmester5.physical_task(np.random.default_rng(9))
    n, seeds = 1024, [3, 4, 5]
    roots = np.zeros((len(seeds) * n, 5), np.complex128)
    codes = np.zeros(len(seeds) * n, np.int32)
    with frg.Tracker(cfg) as t:
        t.track_rounds(task, [n], seeds, roots, codes, depth=2)
        for r, s in enumerate(seeds):
            single = t.track(task, [n], s)
            assert np.array_equal(codes[r * n:(r + 1) * n], single.codes)
            assert np.array_equal(roots[r * n:(r + 1) * n], single.roots, equal_nan=True)


@pytest.mark.parametrize("name", ["conic2", "burmester5"])
def test_plugin_mixed_precision_finds_the_plain_roots(name):
    """Mixed precision on a plug-in (the thread kernel's FP32 stage handing ill-conditioned
    steps, the endgame and the finish to FP64) finds every distinct finite root plain FP64
    finds on the same paths, each with residual <= 1e-10 (at most 1e-3 of the successes
    filtered)."""
    if name == "conic2":
        rng = np.random.default_rng(31)
        tasks = np.stack([conic2.line_pair_task(rng.normal(size=4) + 1j * rng.normal(size=4),
                                                rng.normal(size=4) + 1j * rng.normal(size=4))[0] for _ in range(2)])
    else:
        tasks = np.stack([burmester5.physical_task(np.random.default_rng(s)) for s in (11, 12)])
    n = 2048
    kw = dict(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=INF_TOL)
    with frg.Tracker(frg.plugin_config(name, **kw)) as t:
        plain = t.track(tasks, [n, n], 23, want_resid=True)
    with frg.Tracker(frg.plugin_config(name, precision=frg.PREC_MIXED, **kw)) as t:
        mixed = t.track(tasks, [n, n], 23, want_resid=True)
    ok = mixed.codes == 0
    bad = int(np.sum(~(mixed.resid[ok] <= 1e-10)))
    print(f"{name} mixed: codes {np.bincount(mixed.codes, minlength=8)}, {mixed.stats['handoffs']} hand-offs, "
          f"{bad} above the residual bar, track {mixed.stats['track_ms']:.1f} ms vs plain "
          f"{plain.stats['track_ms']:.1f} ms")
    assert bad <= 1e-3 * ok.sum() + 1
    for k in range(2):
        sl = slice(k * n, (k + 1) * n)
        a = distinct_rows(plain.roots[sl], (plain.codes[sl] == 0) & (plain.resid[sl] <= 1e-10), relative=True)
        b = distinct_rows(mixed.roots[sl], (mixed.codes[sl] == 0) & (mixed.resid[sl] <= 1e-10), relative=True)
        assert len(a) == 4 and recall(a, b) == 1.0, (len(a), len(b))
