"""Tasks: target parameter sets q = [P0..P7, Pc0..Pc7, Q1..Q7, Qc1..Qc7] (30 complex).

The reference tracks to one hard-coded generic complex target (frg.cu:147-178): every
parameter an independent complex number. K = 8 precision points P0..P7 are fixed by
the system (nP = 30, htpykinematics.cuh:9).

Generators (seeded with numpy's Philox bit generator):
  disk        generic complex target like the reference's: P_k and their isotropic
              partners Pc_k independent and uniform in the unit disk, crank rotations
              Q_j and Qc_j independent and uniform on the unit circle
  degenerate  as disk, with the points clustered: P_k = c + 1e-3 w_k, Pc_k = cc + 1e-3 wc_k
  curve       P_k on a random smooth closed curve sum_{m=-2..2} a_m e^{i m theta},
              a_m ~ CN(0, 1/(1+m^2)), scaled into the unit disk, theta_k = 2 pi k/8 +
              U(-pi/16, pi/16), plus complex Gaussian jitter of 1% of the curve's
              diameter; Pc_k from an independent curve the same way; Q, Qc as disk
  real        a physical mechanism task: P_k uniform in the disk with Pc_k = conj(P_k)
              and Q_j = e^{i theta_j}, Qc_j = 1/Q_j. Such targets lie on the special
              subfamily Q Qc = 1 of the start systems (frgkinematics.cu:115), where a
              large share of the generic family's paths diverge or end singular
              (sharpening failures, code 5); the benchmark therefore uses generic
              targets, as the reference does.
"""
from __future__ import annotations

import numpy as np

# The reference target (frg.cu:149-178) and its gamma (frg.cu:41).
REFERENCE_TARGET = np.array([
    4.241713408139979 - 4.925334736425448j, 1.448005491494222 - 2.686249989236069j,
    2.287911194543938 - 0.9123108488455074j, -1.870502483790705 - 0.5778077414588303j,
    -0.7625329418400497 + 0.9043788195368165j, -4.142822753796651 + 1.697671322829592j,
    1.023004534182935 - 3.026210035710708j, -2.522295755933046 + 3.942421532145637j,
    -3.769870484797034 + 0.7972377857916531j, -4.285631161563732 - 0.5650246890525263j,
    -2.166030800874488 + 0.8836055774820508j, 4.579260949000442 - 2.074013737196861j,
    4.801289733755713 - 1.460721841824302j, 2.041266673362720 + 2.962149232597863j,
    3.989999692714399 - 0.2328295911150420j, -3.996448356004510 + 4.426854856711802j,
    2.315936719955769 - 0.5527803857724418j, -3.018911857947673 + 0.9692384144638879j,
    -0.4906347357049512 + 2.994316903874402j, 0.2397118512793472 - 1.341440197750693j,
    4.942917423339324 - 2.415216683074435j, 1.599536873563615 + 2.367319121024760j,
    4.229853181495468 - 1.149104287738972j, -0.2180298061101595 + 3.585004213517870j,
    4.311063203842579 - 0.03375595047392820j, 4.938148066901551 + 4.551701974206413j,
    -4.271214442569748 + 0.1355349863802999j, -0.7377434797048270 + 1.831738837919296j,
    0.8894614668331116 + 0.8657473695398501j, 4.036757863569754 + 1.461164684969592j,
], dtype=np.complex128)
REFERENCE_GAMMA = 0.39231132891081666 + 1.0062265257923928j

KINDS = ("disk", "degenerate", "curve", "real")


def _disk(rng, n):
    r = np.sqrt(rng.uniform(0, 1, n))
    th = rng.uniform(0, 2 * np.pi, n)
    return r * np.exp(1j * th)


def _circle(rng, n):
    return np.exp(1j * rng.uniform(0, 2 * np.pi, n))


def _curve_points(rng):
    m = np.arange(-2, 3)
    a = (rng.normal(size=5) + 1j * rng.normal(size=5)) * np.sqrt(0.5 / (1 + m**2))
    th = 2 * np.pi * np.arange(8) / 8 + rng.uniform(-np.pi / 16, np.pi / 16, 8)
    dense = np.linspace(0, 2 * np.pi, 256, endpoint=False)

    def curve(t):
        return (a[None, :] * np.exp(1j * np.outer(t, m))).sum(axis=1)

    pts = curve(dense)
    scale = 0.9 / max(np.max(np.abs(pts)), 1e-12)
    diam = np.max(np.abs(pts[:, None] - pts[None, :])) * scale
    return curve(th) * scale + 0.01 * diam * (rng.normal(size=8) + 1j * rng.normal(size=8)) / np.sqrt(2)


def precision_point_task(seed: int, kind: str = "disk") -> np.ndarray:
    """One task (30 complex) from `seed`; kind in KINDS."""
    rng = np.random.Generator(np.random.Philox(seed))
    q = np.zeros(30, np.complex128)
    if kind == "disk":
        q[0:8], q[8:16] = _disk(rng, 8), _disk(rng, 8)
        q[16:23], q[23:30] = _circle(rng, 7), _circle(rng, 7)
    elif kind == "degenerate":
        c, cc = _disk(rng, 1)[0], _disk(rng, 1)[0]
        q[0:8], q[8:16] = c + 1e-3 * _disk(rng, 8), cc + 1e-3 * _disk(rng, 8)
        q[16:23], q[23:30] = _circle(rng, 7), _circle(rng, 7)
    elif kind == "curve":
        q[0:8], q[8:16] = _curve_points(rng), _curve_points(rng)
        q[16:23], q[23:30] = _circle(rng, 7), _circle(rng, 7)
    elif kind == "real":
        P = _disk(rng, 8)
        Q = _circle(rng, 7)
        q[0:8], q[8:16], q[16:23], q[23:30] = P, np.conj(P), Q, 1.0 / Q
    else:
        raise ValueError(f"unknown task kind {kind!r}; expected one of {KINDS}")
    return q


def task_batch(seeds, kinds) -> np.ndarray:
    """[len(seeds), 30] tasks, one per (seed, kind)."""
    return np.stack([precision_point_task(int(s), k) for s, k in zip(seeds, kinds)])
