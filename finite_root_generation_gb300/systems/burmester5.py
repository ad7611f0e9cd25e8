"""Five-position Burmester problem: the dyads that guide a rigid body through five
prescribed positions.

A position j is the body's displacement d_j and rotation T_j; a dyad is a ground pivot
G and a moving pivot at z in the body frame, whose distance stays constant:
|d_j + T_j z - G|^2 = R for j = 0..4. In isotropic coordinates every point p has an
independent conjugate pc (|p|^2 = p pc), so the system is polynomial over the complex
numbers: unknowns G, Gc, z, zc, R; parameters d_j, dc_j, T_j, Tc_j. A physical task
has dc_j = conj(d_j) and Tc_j = conj(T_j) = 1 / T_j (`physical_task`); a generic
complex task (random parameters) has more roots. Each equation is linear in its own
d_j, which the start generation solves for.
"""
import numpy as np
import sympy as sp

NAME = "burmester5"
G, Gc, z, zc, R = sp.symbols("G Gc z zc R")
d = sp.symbols("d0:5")
dc = sp.symbols("dc0:5")
T = sp.symbols("T0:5")
Tc = sp.symbols("Tc0:5")
UNKNOWNS = [G, Gc, z, zc, R]
PARAMS = list(d) + list(dc) + list(T) + list(Tc)
EQUATIONS = [(d[j] + T[j] * z - G) * (dc[j] + Tc[j] * zc - Gc) - R for j in range(5)]
SOLVED = list(d)


def physical_task(rng):
    """Parameters of five random planar positions: displacements in the unit disk,
    rotation angles within +-60 degrees, conjugates as a real task has them."""
    r = np.sqrt(rng.uniform(0, 1, 5))
    phi = rng.uniform(0, 2 * np.pi, 5)
    dd = r * np.exp(1j * phi)
    th = np.exp(1j * rng.uniform(-np.pi / 3, np.pi / 3, 5))
    return np.concatenate([dd, np.conj(dd), th, np.conj(th)]).astype(np.complex128)
