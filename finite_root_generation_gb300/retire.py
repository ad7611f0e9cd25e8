"""Learned early retirement: data, training and use of the tracker's retirement network.

The plain FP64 tracker is the teacher. `training_set` tracks rounds with checkpoint
features recorded (`Tracker.track_features`) and labels every checkpoint of a path with
the path's outcome: 0 it ends at a new finite root, 1 it fails (non-zero code, an
infinite root, or a residual above 1e-10), 2 it ends at a root that another path of the
round also reaches (the collection merge marks it a duplicate). `train` fits the
network with the library's CUDA kernels (frg_mlp_train); `Retirement.apply` loads it
into a Tracker, which then ends a path at a checkpoint once the network gives it a
failure probability of at least `threshold` (code 2). Paths below the threshold are
tracked as without it: the plain tracker remains the fallback.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import Collection, FrgError, load

NFEAT = 32
NCLASS = 3
RESID_MAX = 1e-10

_F = ctypes.POINTER(ctypes.c_float)
_I32 = ctypes.POINTER(ctypes.c_int32)


def param_count() -> int:
    return int(load().frg_mlp_param_count())


def path_labels(roots, codes, resid, dup_tol=1e-6):
    """Outcome class of every path of one round (see the module docstring)."""
    codes = np.asarray(codes, np.int32)
    good = (codes == 0) & (np.asarray(resid) <= RESID_MAX)
    c = np.where(good, 0, 5).astype(np.int32)
    merged = Collection(dup_tol).merge(roots, c)
    y = np.where(good, 0, 1).astype(np.int32)
    y[good & (merged == 6)] = 2
    return y


def training_set(tracker, fpm, paths_per_task, seeds, max_checkpoints=64, every=32):
    """Checkpoint features X [m, 32], labels y [m] and the path of every checkpoint
    (groups [m], unique across rounds) from rounds tracked by `tracker` (the plain FP64
    tracker for teaching), one round per seed."""
    xs, ys, gs = [], [], []
    base = 0
    for sd in seeds:
        res, feats, nfeat = tracker.track_features(fpm, paths_per_task, sd, max_checkpoints, every)
        lab = path_labels(res.roots, res.codes, res.resid)
        mask = np.arange(max_checkpoints)[None, :] < nfeat[:, None]
        xs.append(feats[mask])
        ys.append(np.repeat(lab, nfeat))
        gs.append(np.repeat(np.arange(len(nfeat), dtype=np.int64) + base, nfeat))
        base += len(nfeat)
    return (np.concatenate(xs).astype(np.float32), np.concatenate(ys).astype(np.int32),
            np.concatenate(gs))


def calibrate(model, X, y, groups, max_good_frac=1e-3):
    """Smallest threshold at which at most `max_good_frac` of the paths that do not fail
    (classes 0 and 2) would be retired at some checkpoint, from held-out checkpoints;
    1.0 (never retire) when no threshold below it qualifies."""
    p1 = model.predict(X)[:, 1].astype(np.float64)
    paths, inv = np.unique(groups, return_inverse=True)
    pmax = np.zeros(len(paths))
    np.maximum.at(pmax, inv, p1)
    fails = np.zeros(len(paths), bool)
    fails[inv[y == 1]] = True
    good = np.sort(pmax[~fails])
    if len(good) == 0:
        return 1.0
    k = int(np.floor(max_good_frac * len(good)))
    thr = float(np.nextafter(good[len(good) - 1 - k], np.inf)) if k < len(good) else 0.0
    return min(max(thr, 0.5), 1.0)


@dataclass
class Retirement:
    params: np.ndarray  # FP32 weights, param_count() values
    mu: np.ndarray
    inv_sigma: np.ndarray
    threshold: float = 0.99
    every: int = 32

    def standardise(self, X):
        return ((np.asarray(X, np.float32) - self.mu) * self.inv_sigma).astype(np.float32)

    def predict(self, X):
        """Class probabilities [n, 3] of raw features, computed on the GPU."""
        Xs = np.ascontiguousarray(self.standardise(X))
        out = np.zeros((len(Xs), NCLASS), np.float32)
        p = np.ascontiguousarray(self.params, np.float32)
        st = load().frg_mlp_predict(Xs.ctypes.data_as(_F), len(Xs), p.ctypes.data_as(_F), out.ctypes.data_as(_F))
        if st != 0:
            raise FrgError(f"frg_mlp_predict failed ({st})")
        return out

    def apply(self, tracker):
        tracker.set_mlp(self.params, self.mu, self.inv_sigma, self.threshold, self.every)


def standardisation(X):
    X = np.nan_to_num(np.asarray(X, np.float64), nan=100.0, posinf=100.0, neginf=-100.0)
    mu = X.mean(axis=0)
    sd = X.std(axis=0)
    inv = np.where(sd > 1e-12, 1.0 / np.maximum(sd, 1e-12), 0.0)
    return mu.astype(np.float32), inv.astype(np.float32)


def class_weights(y):
    counts = np.bincount(y, minlength=NCLASS).astype(np.float64)
    w = np.where(counts > 0, len(y) / (NCLASS * np.maximum(counts, 1)), 0.0)
    return w.astype(np.float32)


def grad(Xs, y, params, class_w):
    """Mean loss and gradient on the GPU (frg_mlp_grad), for standardised features."""
    Xs = np.ascontiguousarray(Xs, np.float32)
    y = np.ascontiguousarray(y, np.int32)
    p = np.ascontiguousarray(params, np.float32)
    cw = np.ascontiguousarray(class_w, np.float32)
    g = np.zeros(param_count(), np.float32)
    loss = ctypes.c_double()
    st = load().frg_mlp_grad(Xs.ctypes.data_as(_F), y.ctypes.data_as(_I32), len(y), p.ctypes.data_as(_F),
                             cw.ctypes.data_as(_F), g.ctypes.data_as(_F), ctypes.byref(loss))
    if st != 0:
        raise FrgError(f"frg_mlp_grad failed ({st})")
    return loss.value, g


def train(X, y, epochs=8, batch=4096, lr=2e-3, seed=0, threshold=0.99, every=32, class_w=None, params=None):
    """Fit the network on raw features X and labels y; returns (Retirement, epoch losses)."""
    mu, inv = standardisation(X)
    Xs = np.ascontiguousarray(((np.asarray(X, np.float32) - mu) * inv).astype(np.float32))
    y = np.ascontiguousarray(y, np.int32)
    cw = np.ascontiguousarray(class_weights(y) if class_w is None else class_w, np.float32)
    p = np.zeros(param_count(), np.float32) if params is None else np.array(params, np.float32)
    losses = np.zeros(epochs, np.float64)
    st = load().frg_mlp_train(Xs.ctypes.data_as(_F), y.ctypes.data_as(_I32), len(y), cw.ctypes.data_as(_F),
                              int(epochs), int(batch), ctypes.c_float(lr), ctypes.c_uint64(seed),
                              p.ctypes.data_as(_F), losses.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if st != 0:
        raise FrgError(f"frg_mlp_train failed ({st})")
    return Retirement(p, mu, inv, threshold, every), losses
