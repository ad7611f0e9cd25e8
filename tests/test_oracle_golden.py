"""Pin the C restatement of the reference (the oracle) against golden vectors
recorded from the reference's own sources (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from conftest import rel_err
from oracle import GAMMA_REF, T_REF


def test_philox_known_answers(oracle):
    """Philox4x32-10 known-answer vectors published with Random123 (Salmon et al.)."""
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in kat:
        assert oracle.philox_block(ctr, key) == want


def test_uniform_draws_in_unit_interval(oracle):
    u = np.array([oracle.uniform01(7, 3, k) for k in range(2000)])
    assert u.min() > 0.0 and u.max() <= 1.0
    assert abs(u.mean() - 0.5) < 0.03


@pytest.mark.parametrize("name", ["fsys", "jvar", "jpar"])
def test_system_matches_reference(oracle, golden, name):
    for Z, q, want in zip(golden["sys_Z"], golden["sys_q"], golden[name]):
        got = getattr(oracle, name)(Z, q)
        assert rel_err(got, want) < 1e-13


def test_jacobian_sparsity_matches_reference(oracle, golden):
    for Z, q, want in zip(golden["sys_Z"], golden["sys_q"], golden["jvar"]):
        assert np.array_equal(oracle.jvar(Z, q) != 0, want != 0)
    for Z, q, want in zip(golden["sys_Z"], golden["sys_q"], golden["jpar"]):
        assert np.array_equal(oracle.jpar(Z, q) != 0, want != 0)


def test_jacobian_finite_differences(oracle, golden):
    """Central differences of FSYS along each unknown (F is holomorphic)."""
    Z, q = golden["sys_Z"][0], golden["sys_q"][0]
    J = oracle.jvar(Z, q)
    h = 1e-6
    for c in range(22):
        e = np.zeros(22, complex); e[c] = h
        fd = (oracle.fsys(Z + e, q) - oracle.fsys(Z - e, q)) / (2 * h)
        assert np.max(np.abs(fd - J[:, c])) < 1e-6 * max(1.0, np.max(np.abs(J)))
    P = oracle.jpar(Z, q)
    for c in range(30):
        e = np.zeros(30, complex); e[c] = h
        fd = (oracle.fsys(Z, q + e) - oracle.fsys(Z, q - e)) / (2 * h)
        assert np.max(np.abs(fd - P[:, c])) < 1e-6 * max(1.0, np.max(np.abs(P)))


def test_homotopy_pieces_match_reference(oracle, golden):
    for k in range(len(golden["hs_t"])):
        t, spm = golden["hs_t"][k], golden["hs_spm"][k]
        Y, u, V = golden["hs_Y"][k], golden["hs_u"][k], golden["hs_V"][k]
        assert rel_err(oracle.q(t, spm, T_REF, GAMMA_REF), golden["hs_q"][k]) < 1e-14
        assert rel_err(oracle.dqdt(t, spm, T_REF, GAMMA_REF), golden["hs_dqdt"][k]) < 1e-14
        assert rel_err(oracle.h(Y, u, spm, T_REF, GAMMA_REF), golden["hs_h"][k]) < 1e-13
        assert rel_err(oracle.jh(Y, u, spm, T_REF, GAMMA_REF), golden["hs_jh"][k]) < 1e-13
        assert rel_err(oracle.switch_patch(u, Y), golden["hs_switch"][k]) < 1e-14
        assert rel_err(oracle.ivp(0, Y, V, u, spm, T_REF, GAMMA_REF), golden["hs_ivp0"][k]) < 1e-9
        assert rel_err(oracle.ivp(1, Y, V, u, spm, T_REF, GAMMA_REF), golden["hs_ivp1"][k]) < 1e-9


def test_q_endpoints(oracle, golden):
    spm = golden["hs_spm"][0]
    assert rel_err(oracle.q(0.0, spm, T_REF, GAMMA_REF), spm) < 1e-15
    assert rel_err(oracle.q(1.0, spm, T_REF, GAMMA_REF), T_REF) < 1e-15


def test_dp65_step_matches_reference(oracle, golden):
    for k in range(len(golden["dp_Y"])):
        want = golden["dp_out"][k]
        s = want[-1].real
        Yn, Vn, err, sc = oracle.dp65(s, 1e-3, 0, golden["dp_Y"][k], golden["dp_V"][k], golden["dp_u"][k],
                                      golden["dp_spm"][k], T_REF, GAMMA_REF)
        assert rel_err(Yn, want[:23]) < 1e-10
        assert rel_err(Vn, want[23:46]) < 1e-9
        # err is a norm of cancelling stage sums: compare it absolutely at the
        # rounding level of s*|k| (|k| = 1), and the step factor through it.
        assert abs(err - want[46].real) <= 1e-7 * abs(want[46].real) + 1e-13 * max(s, 1.0)
        assert abs(sc - want[47].real) <= 1e-6 * abs(want[47].real) + abs(sc) * abs(err - want[46].real) / max(err, 1e-300)


def test_newton_matches_reference(oracle, golden):
    for k in range(len(golden["nw_Y0"])):
        Y0 = golden["nw_Y0"][k]
        YN, res = oracle.newton(Y0[22].real, golden["dp_out"][k][23:46], golden["dp_u"][k],
                                golden["dp_spm"][k], T_REF, GAMMA_REF, 10, 1e-8, 1, Y0)
        assert rel_err(YN, golden["nw_out"][k]) < 1e-10
        assert (res < 1e-8) == (golden["nw_res"][k] < 1e-8)
        sh = golden["nw_sh"][k]
        YS, rs = oracle.newton(0.0, golden["dp_V"][k], golden["dp_u"][k], golden["dp_spm"][k], T_REF, GAMMA_REF,
                               30, 1e-12, 1, sh[:23])
        assert rel_err(YS, sh[23:]) < 1e-10
        assert (rs < 1e-12) == (golden["nw_shres"][k] < 1e-12)


def test_generate_start_matches_reference(oracle, golden):
    seed = int(golden["path_seed"][0])
    for s in range(len(golden["gs_spt"])):
        spt, spm = oracle.generate_start(seed, s)
        # two quadratic solves per j (frgkinematics.cu:63-107) lose a few digits to cancellation
        assert rel_err(spt, golden["gs_spt"][s]) < 1e-10
        assert rel_err(spm, golden["gs_spm"][s]) < 1e-10


def test_generate_start_is_exact_root(oracle):
    """Known answer: the start point solves the start system, F(spt, 1; spm) = 0."""
    for s in range(8):
        spt, spm = oracle.generate_start(99, s)
        f = oracle.fsys(np.concatenate([spt, [1.0]]), spm)
        assert np.max(np.abs(f)) < 1e-9 * max(1.0, np.max(np.abs(spt)) ** 3)


def test_full_paths_match_reference(oracle, golden):
    """Path for path on the reference target: same code, same canonical root."""
    seed = int(golden["path_seed"][0])
    n = len(golden["path_codes"])
    roots, codes, _, _ = oracle.homotopy_batch(T_REF, GAMMA_REF, seed, np.arange(n))
    want_codes = golden["path_codes"]
    assert np.array_equal(codes, want_codes)
    for i in range(n):
        if want_codes[i] == 0:
            assert rel_err(roots[i], golden["path_roots"][i]) < 1e-8


def test_batch_residuals_are_per_root(oracle, golden):
    """Residuals of many roots in one call equal the roots' residuals one at a time (and,
    where the reference's host build exists, the reference's own FSYS/JVAR residuals)."""
    roots = golden["path_roots"][golden["path_codes"] == 0]
    batch = oracle.residuals(roots, T_REF)
    single = np.array([oracle.residuals(r[None], T_REF)[0] for r in roots])
    assert len(roots) > 10
    assert np.array_equal(batch, single)
    assert np.all(batch < 1e-10)
    import oracle as oracle_mod
    if os.path.exists(oracle_mod.REF_SO):
        ref = oracle_mod.RefLib().residuals(roots, T_REF)
        # both are round-off (~1e-16) at these roots; they agree to that level
        np.testing.assert_allclose(batch, ref, rtol=0, atol=1e-13)


def test_cognate_matches_reference(oracle, golden):
    for z, want in zip(golden["cog_in"], golden["cog_out"]):
        assert rel_err(oracle.cognate(z, T_REF), want) < 1e-12


def test_cognate_is_root(oracle, golden):
    """Known answer: the 1/2 cognate of a root is again a root of the target system."""
    for z, pair in zip(golden["cog_in"], golden["cog_out"]):
        for r in pair:
            f = oracle.fsys(np.concatenate([r, [1.0]]), T_REF)
            assert np.max(np.abs(f)) < 1e-6 * max(1.0, np.max(np.abs(r)) ** 3)


def test_sort_merge_matches_reference(oracle, golden):
    merged, codes = oracle.sort_merge(golden["dd_coll"], golden["dd_new"], golden["dd_codes_in"])
    assert np.array_equal(codes, golden["dd_codes_out"])
    assert np.array_equal(merged, golden["dd_merged"])
    m2, c2 = oracle.sort_merge(np.zeros((0, 21), complex), golden["dd_new"], golden["dd_codes_in"])
    assert np.array_equal(c2, golden["dd_codes_empty"])
    assert np.array_equal(m2, golden["dd_merged_empty"])


def test_lambertw_matches_reference(oracle, golden):
    for z, w in zip(golden["lw_z"], golden["lw_w"]):
        assert abs(oracle.lambertw0(z) - w) < 1e-12 * max(1.0, abs(w))
