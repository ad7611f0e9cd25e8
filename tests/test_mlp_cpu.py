"""The float64 network oracle (oracle/mlp_oracle.py) against central finite differences,
its BF16 rounding, and the library's parameter layout (CPU only)."""
import sys
import os

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import mlp_oracle as mo  # noqa: E402


def _net(seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(size=mo.NPARAM) * 0.3
    X = rng.normal(size=(24, mo.NIN))
    y = rng.integers(0, 3, size=24)
    return p, X, y


def test_gradient_matches_finite_differences():
    p, X, y = _net(1)
    cw = np.array([1.0, 3.0, 0.5])
    loss, g = mo.loss_grad(p, X, y, cw)
    assert np.isfinite(loss) and loss > 0
    rng = np.random.default_rng(2)
    for k in rng.choice(mo.NPARAM, size=60, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mo.loss_grad(pp, X, y, cw)[0] - mo.loss_grad(pm, X, y, cw)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding():
    # BF16 keeps 7 fraction bits: steps of 2^-7 just above 1
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 3 * 2 ** -8, -2.5, 3.1415926, 1e-3], np.float32)
    r = mo.bf16_round(v)
    assert r[0] == 1.0 and r[4] == -2.5
    assert r[1] == 1.0                    # tie between 1 and 1 + 2^-7 goes to the even one
    assert r[2] == 1.0 + 2 ** -7          # nearest
    assert r[3] == 1.0 + 2 ** -6          # tie between 1 + 2^-7 and 1 + 2^-6: even
    assert np.all(np.abs(r - v) <= np.abs(v) * 2 ** -8)  # half a unit in the last of 8 bits


def test_layout_matches_library_count():
    import finite_root_generation_gb300.retire as rt

    assert rt.param_count() == mo.NPARAM == 6467
    d = mo.unpack(np.arange(mo.NPARAM, dtype=np.float64))
    assert d["W1"][1, 0] == 32 and d["b1"][0] == 2048 and d["W2"][0, 0] == 2112 and d["b3"][2] == 6466
    assert np.array_equal(mo.pack(d), np.arange(mo.NPARAM))


def test_path_labels():
    import finite_root_generation_gb300.retire as rt

    rng = np.random.default_rng(3)
    roots = rng.normal(size=(6, 21)) + 1j * rng.normal(size=(6, 21))
    roots[4] = roots[1] + 1e-9  # duplicate of path 1
    codes = np.array([0, 0, 3, 0, 0, 0], np.int32)
    resid = np.array([1e-14, 1e-14, 1e-14, 1e-8, 1e-14, 1e-14])
    y = rt.path_labels(roots, codes, resid)
    assert y[2] == 1 and y[3] == 1            # failure code, residual too large
    assert sorted([y[1], y[4]]) == [0, 2]     # one of the pair is the duplicate
    assert y[0] == 0 and y[5] == 0
