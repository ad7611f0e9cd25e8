"""Two plane conics in the unknowns (x, y).

The smallest plug-in, with a known answer: when each conic is a pair of lines,
y = m1 x + k1 and y = m2 x + k2 for the first, y = m3 x + k3 and y = m4 x + k4 for the
second, the system has exactly the four finite roots where a line of one pair meets a
line of the other (`line_pair_task`). The start generation solves for the constant
terms f1, f2.
"""
import numpy as np
import sympy as sp

NAME = "conic2"
x, y = sp.symbols("x y")
a1, b1, c1, d1, e1, f1 = sp.symbols("a1 b1 c1 d1 e1 f1")
a2, b2, c2, d2, e2, f2 = sp.symbols("a2 b2 c2 d2 e2 f2")
UNKNOWNS = [x, y]
PARAMS = [a1, b1, c1, d1, e1, f1, a2, b2, c2, d2, e2, f2]
EQUATIONS = [
    a1 * x**2 + b1 * x * y + c1 * y**2 + d1 * x + e1 * y + f1,
    a2 * x**2 + b2 * x * y + c2 * y**2 + d2 * x + e2 * y + f2,
]
SOLVED = [f1, f2]


def line_pair_task(m, k):
    """Parameters of the two line pairs y = m[i] x + k[i] (i = 0, 1 the first conic,
    2, 3 the second), and the four roots (x, y), one per line of the first pair and
    line of the second."""
    m = np.asarray(m, np.complex128)
    k = np.asarray(k, np.complex128)
    q = []
    for i, j in ((0, 1), (2, 3)):
        # (y - m_i x - k_i)(y - m_j x - k_j)
        q += [m[i] * m[j], -(m[i] + m[j]), 1.0, m[i] * k[j] + m[j] * k[i], -(k[i] + k[j]), k[i] * k[j]]
    roots = []
    for i in (0, 1):
        for j in (2, 3):
            xx = (k[j] - k[i]) / (m[i] - m[j])
            roots.append([xx, m[i] * xx + k[i]])
    return np.array(q, np.complex128), np.array(roots, np.complex128)
