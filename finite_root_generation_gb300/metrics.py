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


def distinct_rows(roots, keep=None, dup_tol=1e-6, relative=False):
    """Distinct rows of `roots` ([n, nv] complex, any nv: the plug-in systems' roots),
    among those with `keep` true, by the collection's duplicate rule (every real
    component within dup_tol); the first of a group of duplicates in Re(root[0]) order
    stays. Returns [k, nv] sorted by Re(root[0]). With `relative`, the tolerance of a
    pair is dup_tol x max(1, the larger max-norm of the two), for roots large enough
    that their last digits differ by more than dup_tol between paths."""
    r = np.asarray(roots, np.complex128)
    r = r.reshape(len(r), -1) if r.size else r.reshape(0, max(r.shape[-1] if r.ndim == 2 else 1, 1))
    if keep is not None:
        r = r[np.asarray(keep, bool)]
    r = r[np.all(np.isfinite(r), axis=1)]
    r = r[np.argsort(r[:, 0].real, kind="stable")]
    parts = np.concatenate([r.real, r.imag], axis=1)
    scale = np.maximum(1.0, np.max(np.abs(parts), axis=1)) if relative else np.ones(len(r))
    window = dup_tol * (scale.max() if len(r) else 1.0)
    kept = []
    for i in range(len(r)):
        dup = False
        for j in reversed(kept):
            if parts[i, 0] - parts[j, 0] > window:
                break
            if np.max(np.abs(parts[i] - parts[j])) <= dup_tol * max(scale[i], scale[j]):
                dup = True
                break
        if not dup:
            kept.append(i)
    return r[kept]


def recall(reference_roots, found_roots, rtol=1e-8):
    """Fraction of `reference_roots` present in `found_roots` (both [k, nv]; nv = 21 for
    Stephenson II, a plug-in system's unknowns otherwise).

    Roots with a non-finite component never match. Candidates are found by a binary
    search on the first component's real part, so the cost is O((n + m) log m) plus
    the candidates inside each tolerance window, each window checked vectorised.
    """
    a = np.asarray(reference_roots, np.complex128)
    b = np.asarray(found_roots, np.complex128)
    nv = a.shape[-1] if a.ndim == 2 else (b.shape[-1] if b.ndim == 2 else 21)
    a = a.reshape(-1, nv)
    b = b.reshape(-1, nv)
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
