"""Root-set metrics: distinct finite roots and recall between two runs.

A root counts as *distinct finite* when its path succeeded (code 0, so not an
infinite root, code 7), its row-scaled residual is at most `resid_max`, and it is
not a duplicate of another counted root. Duplicates are found with the library's
collection merge (the reference's SortingDeletingMerging rule, frgsupport.cu:69-172:
every real component within `dup_tol`).

Recall of run B against run A is the fraction of A's distinct roots that B also
found, matching roots within `rtol` relative (max-norm over the 21 components).
"""
from __future__ import annotations

import numpy as np

from . import Collection


def distinct_roots(roots, codes, resid=None, resid_max=1e-10, dup_tol=1e-6):
    """Sorted array of distinct finite roots ([k, 21] complex)."""
    roots = np.asarray(roots, np.complex128).reshape(-1, 21)
    codes = np.asarray(codes, np.int32)
    good = codes == 0
    if resid is not None:
        good &= np.asarray(resid) <= resid_max
    c = np.where(good, 0, 5).astype(np.int32)
    coll = Collection(dup_tol)
    coll.merge(roots, c)
    return coll.roots()


def recall(reference_roots, found_roots, rtol=1e-8):
    """Fraction of `reference_roots` present in `found_roots` (both [k, 21]).

    Roots with a non-finite component never match. Candidates are found by a binary
    search on the first component's real part, so the cost is O((n + m) log m) plus
    the candidates inside each tolerance window, each window checked vectorised.
    """
    a = np.asarray(reference_roots, np.complex128).reshape(-1, 21)
    b = np.asarray(found_roots, np.complex128).reshape(-1, 21)
    if len(a) == 0:
        return 1.0
    b = b[np.all(np.isfinite(b), axis=1)]
    if len(b) == 0:
        return 0.0
    order = np.argsort(b[:, 0].real, kind="stable")
    bs = b[order]
    keys = bs[:, 0].real
    scale_b = np.max(np.abs(bs), axis=1)
    fin = np.all(np.isfinite(a), axis=1)
    s = np.where(fin, np.max(np.abs(np.where(fin[:, None], a, 0)), axis=1), 0.0)
    # a match within rtol * max(|a|, |b|) has |b| <= |a| (1 + rtol) / (1 - rtol)
    tol = rtol * np.maximum(s, 1e-300) / (1.0 - rtol)
    lo = np.searchsorted(keys, a[:, 0].real - tol, side="left")
    hi = np.searchsorted(keys, a[:, 0].real + tol, side="right")
    hit = 0
    for i in np.nonzero(fin & (hi > lo))[0]:
        cand = bs[lo[i]:hi[i]]
        err = np.max(np.abs(cand - a[i]), axis=1)
        if np.any(err <= rtol * np.maximum(s[i], scale_b[lo[i]:hi[i]])):
            hit += 1
    return hit / len(a)
