"""System plug-ins on the CPU: the generated code is current, the oracle's generated rows
and starts agree with the symbolic systems (evaluated independently by numpy, with
derivatives by central differences), the oracle's tracker finds the known answers of
both plug-ins, and the C ABI describes and validates them without a GPU.

Known answers:
  * conic2 with two line pairs y = m_i x + k_i: exactly the four intersection points;
  * burmester5 with five physical positions: four dyads (Burmester's theorem: at most
    four circle-point / centre-point pairs; 2 real and one conjugate pair here), each with
    Gc = conj(G), zc = conj(z), R real for the real ones.
"""
import ctypes

import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300.metrics import distinct_rows

sp = pytest.importorskip("sympy")  # the plug-in modules state their systems in sympy

from finite_root_generation_gb300.systems import PLUGINS, burmester5, conic2  # noqa: E402

MODULES = {"conic2": conic2, "burmester5": burmester5}


def _numeric_system(mod):
    """F^h(Z, Z0; q) = Z0^deg F(Z / Z0; q) as a numpy function of (Z, Z0, q)."""
    f = sp.lambdify([mod.UNKNOWNS, mod.PARAMS], mod.EQUATIONS, "numpy")
    deg = [sp.Poly(e, *mod.UNKNOWNS).total_degree() for e in mod.EQUATIONS]

    def Fh(Z, z0, q):
        vals = np.array(f(list(Z / z0), list(q)), np.complex128)
        return vals * z0 ** np.array(deg)

    return Fh


def test_generated_code_is_current():
    from finite_root_generation_gb300.gen import gen_plugins

    assert gen_plugins.main(check=True), "run finite_root_generation_gb300/gen/gen_plugins.py"


@pytest.mark.parametrize("name", PLUGINS)
def test_oracle_rows_match_the_symbolic_system(oracle, name):
    mod = MODULES[name]
    sid = PLUGINS.index(name) + 1
    nv, np_ = oracle.plugin_info(sid)
    assert (nv, np_) == (len(mod.UNKNOWNS), len(mod.PARAMS))
    Fh = _numeric_system(mod)
    rng = np.random.default_rng(sid)
    for _ in range(3):
        Z = rng.normal(size=nv) + 1j * rng.normal(size=nv)
        z0 = complex(rng.normal(), rng.normal())
        q = rng.normal(size=np_) + 1j * rng.normal(size=np_)
        dq = rng.normal(size=np_) + 1j * rng.normal(size=np_)
        Y = np.concatenate([Z, [z0, 0.37]])
        M, F = oracle.plugin_rows(sid, Y, q, dq)
        np.testing.assert_allclose(F, Fh(Z, z0, q), rtol=1e-13, atol=1e-13)
        h = 1e-6
        for c in range(nv + 1):
            e = np.zeros(nv + 1, np.complex128)
            e[c] = h
            fd = (Fh(Z + e[:nv], z0 + e[nv], q) - Fh(Z - e[:nv], z0 - e[nv], q)) / (2 * h)
            np.testing.assert_allclose(M[:, c], fd, rtol=1e-7, atol=1e-7)
        fd_t = (Fh(Z, z0, q + h * dq) - Fh(Z, z0, q - h * dq)) / (2 * h)
        np.testing.assert_allclose(M[:, nv + 1], fd_t, rtol=1e-7, atol=1e-7)


@pytest.mark.parametrize("name", PLUGINS)
@pytest.mark.parametrize("dist", [0, 1])
def test_oracle_start_is_an_exact_root(oracle, name, dist):
    mod = MODULES[name]
    sid = PLUGINS.index(name) + 1
    Fh = _numeric_system(mod)
    cfg = oracle.config(start_dist=dist)
    for stream in range(5):
        spt, spm = oracle.plugin_start(sid, 77, stream, cfg)
        f = Fh(spt, 1.0, spm)
        assert np.max(np.abs(f)) <= 1e-12 * max(1.0, np.max(np.abs(spm)) ** 2 * np.max(np.abs(spt)) ** 2)


def test_oracle_conic2_finds_the_four_known_roots(oracle):
    rng = np.random.default_rng(3)
    q, known = conic2.line_pair_task(rng.normal(size=4) + 1j * rng.normal(size=4),
                                     rng.normal(size=4) + 1j * rng.normal(size=4))
    roots, codes, resid, _ = oracle.plugin_batch(1, q, [np.exp(0.7j)], 11, [64])
    ok = codes == 0
    assert ok.mean() >= 0.95
    assert np.all(resid[ok] <= 1e-12)
    for r in roots[ok]:
        assert np.min(np.max(np.abs(known - r), axis=1)) <= 1e-10
    found = distinct_rows(roots, ok)
    assert len(found) == 4


def test_oracle_burmester5_finds_four_dyads(oracle):
    task = burmester5.physical_task(np.random.default_rng(5))
    roots, codes, resid, yf = oracle.plugin_batch(2, task, [np.exp(0.3j)], 11, [512], want_yfinal=True)
    ok = codes == 0
    assert ok.mean() > 0.5
    assert np.all(resid[ok] <= 1e-12)
    dyads = distinct_rows(roots, ok)
    assert len(dyads) == 4, dyads
    real = [r for r in dyads if abs(r[1] - np.conj(r[0])) < 1e-9 and abs(r[3] - np.conj(r[2])) < 1e-9]
    assert len(real) % 2 == 0 and all(abs(r[4].imag) < 1e-9 for r in real)
    # the others come in conjugate pairs (G, Gc, z, zc, R) -> (conj Gc, conj G, conj zc, conj z, conj R)
    for r in dyads:
        mirror = np.conj(r[[1, 0, 3, 2, 4]])
        assert np.min(np.max(np.abs(dyads - mirror), axis=1)) < 1e-9


def test_capi_describes_the_systems():
    infos = frg.list_systems()
    assert infos[0].name == "stephenson2" and (infos[0].nv, infos[0].np) == (frg.NV, frg.NP)
    assert [s.name for s in infos[1:]] == PLUGINS
    for s in infos[1:]:
        mod = MODULES[s.name]
        assert (s.nv, s.np) == (len(mod.UNKNOWNS), len(mod.PARAMS))
    with pytest.raises(frg.FrgError):
        frg.system_info(len(infos))
    with pytest.raises(frg.FrgError):
        frg.system_info(-1)


def test_capi_rejects_unsupported_plugin_configs_without_a_gpu():
    lib = frg.load()
    lib.frg_track_noalloc.restype = ctypes.c_int
    ppt = (ctypes.c_int64 * 1)(4)
    buf = (ctypes.c_double * 64)()
    bad = [dict(system=len(frg.list_systems())), dict(system=-1),
           dict(system=1),                                            # the team kernel
           dict(system=1, kernel_variant=frg.KERNEL_THREAD, precision=frg.PREC_MIXED),
           dict(system=2, kernel_variant=frg.KERNEL_THREAD)]          # no-alloc holds Stephenson II tasks
    for kw in bad:
        c = frg.default_config(**kw)
        assert lib.frg_track_noalloc(ctypes.byref(c), buf, 1, ppt, ctypes.c_uint64(1), buf, buf, None,
                                     None) == -1, kw


def test_distinct_rows_relative_tolerance():
    """Absolute tolerance keeps near copies of a large root apart; the relative option
    merges them, and never merges distinct small roots."""
    big = np.array([5e4 + 1j, 3.0, 2.0 - 1j])
    rows = np.stack([big, big * (1 + 3e-11), big * (1 - 2e-11), np.array([0.1, 0.2, 0.3]),
                     np.array([0.1 + 2e-6, 0.2, 0.3])])
    assert len(distinct_rows(rows)) == 5
    assert len(distinct_rows(rows, relative=True)) == 3
    assert len(distinct_rows(rows, keep=[True, False, False, True, True], relative=True)) == 3


def test_generator_rejects_malformed_systems():
    """A plug-in needs one polynomial equation per unknown and one solved parameter per
    equation in which the system is linear."""
    import types

    from finite_root_generation_gb300.gen import gen_plugins

    x, y, a, b, c = sp.symbols("x y a b c")

    def spec(eqs, solved, unknowns=(x, y), params=(a, b, c)):
        return types.SimpleNamespace(NAME="bad", UNKNOWNS=list(unknowns), PARAMS=list(params), EQUATIONS=eqs,
                                     SOLVED=solved)

    good = spec([a * x**2 + y - b, x * y - c], [b, c])
    info = gen_plugins.analyse(good)
    assert (info["nv"], info["np"], info["ns"]) == (2, 3, 2)
    with pytest.raises(ValueError, match="one equation per unknown"):
        gen_plugins.analyse(spec([x - a], [a]))
    with pytest.raises(ValueError, match="SOLVED"):
        gen_plugins.analyse(spec([x - a, y - b], [a]))
    with pytest.raises(ValueError, match="linear in SOLVED"):
        gen_plugins.analyse(spec([x - b**2, y - c], [b, c]))
    with pytest.raises(sp.PolynomialError):
        gen_plugins.analyse(spec([x - 1 / y + b, y - c], [b, c]))
