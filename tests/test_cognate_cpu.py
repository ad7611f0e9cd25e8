"""Why the canonical form uses the 1/2 cognate only (the reference's CognateSolns,
frgkinematics.cu:227-285, with its Cognate34 calls commented out at :262-266).

A root's 1/2 cognate is again a root of the same task (the same coupler path with the
same prescribed crank rotations), so two paths can land on the two members of a pair:
the canonical form picks one of them. The 3/4 cognate linkage (Cognate34,
frgkinematics.cu:140-182) draws the same coupler curve but cannot meet the prescribed
rotations: no choice of the rotations U_j makes it a root (least squares over all seven
U_j from four starting guesses leaves |F| >= 1e-3), so it never duplicates a collected
root and a 4-cognate canonical form would change nothing. Checked on the reference's own
tracked roots (golden vectors), CPU only."""
import numpy as np
import pytest

from finite_root_generation_gb300.tasks import REFERENCE_TARGET


def _roots(golden):
    ok = golden["path_codes"] == 0
    return golden["path_roots"][ok][:12]


def test_half_cognate_is_a_root(oracle, golden):
    import oracle as om
    for z in _roots(golden):
        c = om.cognate12_root(z, REFERENCE_TARGET)
        assert oracle.residuals(c[None], REFERENCE_TARGET)[0] < 1e-10


def test_three_quarter_cognate_is_never_a_root(oracle, golden):
    optimize = pytest.importorskip("scipy.optimize")
    import oracle as om
    q = REFERENCE_TARGET

    def fvec(u, z):
        y = z.copy()
        y[14:21] = u[:7] + 1j * u[7:]
        f = oracle.fsys(np.concatenate([y, [1.0]]), q)
        return np.concatenate([f.real, f.imag])

    for z in _roots(golden):
        z34 = z.copy()
        z34[0:7] = om.cognate34_linkage(z[0:7], q[0])
        z34[7:14] = om.cognate34_linkage(z[7:14], q[8])
        u_down = om.cognate12_root(z, q)[14:21]
        best = np.inf
        for u0 in (z[14:21], u_down, 1 / z[14:21], 1 / u_down):
            sol = optimize.least_squares(fvec, np.concatenate([u0.real, u0.imag]), args=(z34,), xtol=1e-14,
                                         ftol=1e-14, gtol=1e-14)
            best = min(best, float(np.max(np.abs(sol.fun))))
        assert best > 1e-3, best
