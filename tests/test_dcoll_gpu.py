"""Device-resident root collection (frg_dcoll) against the host collection
(frg_coll_merge, pinned to the reference's SortingDeletingMerging by the golden merge
vectors): the same duplicate marks, merge after merge, per key, and the same collected
sets. Bar: codes equal exactly; collected roots equal as sets (bit for bit)."""
import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.tasks import precision_point_task

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _batch(rng, prev, n):
    """n roots: fresh random ones, exact and near copies of earlier roots (within and
    beyond tol), near copies inside the batch and chains of near copies."""
    roots = (rng.normal(size=(n, 21)) + 1j * rng.normal(size=(n, 21))) * 3.0
    for i in range(n):
        kind = int(rng.integers(0, 8))
        src = None
        if kind in (1, 2, 3) and len(prev):
            src = prev[rng.integers(0, len(prev))]
        elif kind in (4, 5) and i > 0:
            src = roots[rng.integers(0, i)]
        if src is None:
            continue
        jitter = {1: 0.0, 2: 0.5e-6, 3: 2e-6, 4: 0.5e-6, 5: 0.9e-6}[kind]
        d = rng.uniform(-jitter, jitter, size=(21, 2))
        roots[i] = src + d[:, 0] + 1j * d[:, 1]
    return roots


def _host_merge(colls, roots, codes, keys):
    out = codes.copy()
    for k in np.unique(keys):
        idx = np.nonzero(keys == k)[0]
        if k not in colls:
            colls[k] = frg.Collection(TOL)
        out[idx] = colls[k].merge(roots[idx], codes[idx])
    return out


def _canon(r):
    v = np.ascontiguousarray(r).view(np.float64).reshape(len(r), 42)
    return v[np.lexsort(v.T[::-1])]


def test_device_collection_matches_host_merge():
    torch = pytest.importorskip("torch")
    frg_build.build()
    rng = np.random.default_rng(5)
    dc = frg.DeviceCollection(20000, TOL)
    colls = {}
    prev = np.zeros((0, 21), np.complex128)
    for rnd in range(4):
        n = 3000
        roots = _batch(rng, prev, n)
        codes = np.where(rng.uniform(size=n) < 0.9, 0, rng.integers(1, 6, size=n)).astype(np.int32)
        keys = rng.integers(0, 3, size=n).astype(np.int32)
        want = _host_merge(colls, roots, codes, keys)
        d_codes = torch.from_numpy(codes.copy()).cuda()
        dc.merge(torch.from_numpy(roots.view(np.float64).copy()).cuda(), d_codes, torch.from_numpy(keys).cuda())
        got = d_codes.cpu().numpy()
        assert np.array_equal(got, want), (rnd, np.nonzero(got != want)[0][:10])
        assert (want == 6).sum() > 50
        prev = np.concatenate([prev, roots])
    assert len(dc) == sum(len(c) for c in colls.values())
    d_roots, d_keys = dc.roots()
    for k, c in colls.items():
        assert np.array_equal(_canon(d_roots[d_keys == k]), _canon(c.roots()))
    dc.close()


def test_device_collection_on_tracked_roots():
    """Three rounds of real roots of two tasks (the second round repeats the first's
    paths): the same marks as the host merge per task."""
    torch = pytest.importorskip("torch")
    frg_build.build()
    tasks = np.stack([precision_point_task(3, "disk"), precision_point_task(4, "curve")])
    cfg = frg.default_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8)
    dc = frg.DeviceCollection(10000, TOL)
    colls = {}
    with frg.Tracker(cfg) as t:
        for seed in (8, 8, 9):
            res = t.track(tasks, [1024, 1024], seed, want_resid=True)
            codes = np.where((res.codes == 0) & (res.resid <= 1e-10), 0, 5).astype(np.int32)
            keys = np.repeat(np.array([0, 1], np.int32), 1024)
            want = _host_merge(colls, res.roots, codes, keys)
            d_codes = torch.from_numpy(codes.copy()).cuda()
            dc.merge(torch.from_numpy(res.roots.view(np.float64).copy()).cuda(), d_codes,
                     torch.from_numpy(keys).cuda())
            assert np.array_equal(d_codes.cpu().numpy(), want)
    assert len(dc) == sum(len(c) for c in colls.values())
    dc.close()


def test_device_collection_residual_filter():
    """With residuals given, a success whose residual exceeds resid_max (or is NaN) takes no
    part: it is not collected, not compared, and its code is left as it is."""
    torch = pytest.importorskip("torch")
    frg_build.build()
    rng = np.random.default_rng(9)
    n = 4000
    roots = _batch(rng, np.zeros((0, 21), np.complex128), n)
    codes = np.zeros(n, np.int32)
    resid = rng.uniform(0, 2e-10, size=n)
    resid[::97] = np.nan
    want_codes = np.where(resid <= 1e-10, 0, 5).astype(np.int32)
    want = _host_merge({}, roots, want_codes, np.zeros(n, np.int32))
    dc = frg.DeviceCollection(n, TOL)
    d_codes = torch.from_numpy(codes.copy()).cuda()
    dc.merge(torch.from_numpy(roots.view(np.float64).copy()).cuda(), d_codes, None,
             resid=torch.from_numpy(resid).cuda(), resid_max=1e-10)
    got = d_codes.cpu().numpy()
    part = resid <= 1e-10
    assert np.array_equal(got[part], want[part])
    assert np.all(got[~part] == 0)
    assert len(dc) == int((want == 0).sum())
    dc.close()
