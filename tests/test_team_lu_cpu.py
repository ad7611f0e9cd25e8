"""The structured elimination the team kernels use for the 23 x 23 tangent system
(csrc/frg_team.cuh, linear_step), restated in numpy float64 and checked on the
oracle's Jacobians (CPU only): it solves the same system as a dense solve, and its
condition estimate (pivot ratio of the re-scaled dense phase, group amplification)
follows the reference's dense partial-pivoting pivot ratio.

The restatement mirrors the kernel step by step: row scaling by max(|re|, |im|); per
equation group j, partial pivoting on the U_j column among its three rows and
elimination of U_j from the other two; folding of every group's pivot row into the two
patch rows; re-scaling of the 16 remaining rows; a dense 16 x 16 solve with partial
pivoting; U_j recovered from its group's pivot row."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import oracle as orc  # noqa: E402

DENSE = list(range(14)) + [21, 22]


def _rowmax(R):
    return np.maximum(np.abs(R.real), np.abs(R.imag)).max(axis=-1)


def gepp(A, b):
    """Dense partial pivoting (first maximum of |a|^2); returns x and the pivots."""
    A = A.copy()
    b = b.copy()
    n = len(b)
    piv = []
    for k in range(n):
        i = k + int(np.argmax(np.abs(A[k:, k]) ** 2))
        A[[k, i]] = A[[i, k]]
        b[[k, i]] = b[[i, k]]
        piv.append(A[k, k])
        l = A[k + 1:, k] / A[k, k]
        A[k + 1:, k:] -= np.outer(l, A[k, k:])
        b[k + 1:] -= l * b[k]
    x = np.zeros(n, complex)
    for k in range(n - 1, -1, -1):
        x[k] = (b[k] - A[k, k + 1:] @ x[k + 1:]) / A[k, k]
    return x, np.abs(np.array(piv))


def team_solve(M, b):
    M = M.copy()
    b = b.copy()
    s = 1.0 / _rowmax(M[:22])
    M[:22] *= s[:, None]
    b[:22] *= s
    rows, rhs, pivots, amp = [], [], {}, 1.0
    patch, prhs = M[[21, 22]].copy(), b[[21, 22]].copy()
    for j in range(1, 8):
        r, cu = [j - 1, j + 6, j + 13], 13 + j
        G, g = M[r], b[r]
        a = np.abs(G[:, cu]) ** 2
        p = 0 if (a[0] >= a[1] and a[0] >= a[2]) else (1 if a[1] >= a[2] else 2)
        pr, prb = G[p], g[p]
        amp = max(amp, 1.0 / abs(pr[cu]))
        for q in range(3):
            if q != p:
                m = G[q, cu] / pr[cu]
                rows.append((G[q] - m * pr)[DENSE])
                rhs.append(g[q] - m * prb)
        m = patch[:, cu] / pr[cu]
        patch = patch - np.outer(m, pr)
        prhs = prhs - m * prb
        pivots[j] = (pr, prb)
    D = np.array(rows + [patch[0][DENSE], patch[1][DENSE]])
    d = np.array(rhs + [prhs[0], prhs[1]])
    sc = 1.0 / _rowmax(D)
    xd, piv = gepp(D * sc[:, None], d * sc)
    x = np.zeros(23, complex)
    x[DENSE] = xd
    for j, (pr, prb) in pivots.items():
        cu = 13 + j
        rest = [c for c in range(23) if c != cu]
        x[cu] = (prb - pr[rest] @ x[rest]) / pr[cu]
    return x, max(piv.max() / piv.min(), amp)


def _tangent_systems(count=40, seed=5):
    o = orc.Oracle()
    rng = np.random.default_rng(seed)
    fpm = rng.uniform(-1, 1, 30) + 1j * rng.uniform(-1, 1, 30)
    cfg = o.config(start_dist=1)
    out = []
    for i in range(count):
        spt, spm = o.generate_start(seed, i, cfg)
        Y = np.concatenate([spt, [1.0, rng.uniform(0.0, 0.9)]])
        u = rng.uniform(-2, 2, 23) + 1j * rng.uniform(-2, 2, 23)
        V = rng.uniform(-2, 2, 23) + 1j * rng.uniform(-2, 2, 23)
        gamma = np.exp(2j * np.pi * rng.random())
        M = np.vstack([o.jh(Y, u, spm, fpm, gamma), V[None, :]])
        b = np.zeros(23, complex)
        b[22] = 1.0
        out.append((M, b))
    return out


def test_structured_solve_equals_dense_solve():
    for M, b in _tangent_systems():
        x, _ = team_solve(M, b)
        ref = np.linalg.solve(M, b)
        assert np.max(np.abs(x - ref)) <= 1e-9 * np.max(np.abs(ref))


def test_condition_estimate_tracks_dense_pivot_ratio():
    ratios = []
    for M, b in _tangent_systems(seed=6):
        Ms = M.copy()
        Ms[:22] /= _rowmax(M[:22])[:, None]
        _, piv = gepp(Ms, b)
        _, est = team_solve(M, b)
        ratios.append(est / (piv.max() / piv.min()))
    ratios = np.array(ratios)
    # the same scale of conditioning: within a factor of 20 of the reference's estimate
    assert np.all(ratios > 0.05) and np.all(ratios < 20), ratios
