"""Learned early retirement on the GPU: the CUDA forward/backward against the float64
oracle, training with the CUDA Adam loop, and what the trained network gains over the
same tracker without it (work done, distinct roots kept)."""
import os
import sys

import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300 import retire
from finite_root_generation_gb300.metrics import distinct_roots, recall
from finite_root_generation_gb300.tasks import precision_point_task

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import mlp_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu


def _random_problem(seed, n=512):
    rng = np.random.default_rng(seed)
    p = (rng.normal(size=mo.NPARAM) * 0.25).astype(np.float32)
    X = rng.normal(size=(n, mo.NIN)).astype(np.float32)
    y = rng.integers(0, 3, size=n).astype(np.int32)
    return p, X, y


def test_gradient_matches_float64_oracle():
    frg_build.build()
    p, X, y = _random_problem(7)
    cw = np.array([1.0, 4.0, 0.5], np.float32)
    loss, g = retire.grad(X, y, p, cw)
    # the oracle differentiates with respect to the same BF16-rounded weights
    ref_loss, ref_g = mo.loss_grad(mo.bf16_round(p), X, y, cw)
    assert abs(loss - ref_loss) <= 1e-4 * max(1.0, abs(ref_loss))
    err = np.abs(g - ref_g)
    assert np.linalg.norm(err) <= 2e-3 * np.linalg.norm(ref_g)
    assert np.max(err) <= 2e-3 * np.max(np.abs(ref_g)) + 1e-6


def test_predict_matches_oracle():
    frg_build.build()
    p, X, _ = _random_problem(8, n=256)
    r = retire.Retirement(p, np.zeros(32, np.float32), np.ones(32, np.float32))
    got = r.predict(X)
    ref = mo.probs(mo.bf16_round(p), X)
    assert np.max(np.abs(got - ref)) <= 1e-4


def test_training_learns_a_separable_rule():
    frg_build.build()
    rng = np.random.default_rng(9)
    X = rng.normal(size=(20000, 32)).astype(np.float32)
    y = np.where(X[:, 0] + 0.5 * X[:, 3] > 1.0, 1, np.where(X[:, 5] > 1.2, 2, 0)).astype(np.int32)
    model, losses = retire.train(X, y, epochs=6, batch=1024, lr=3e-3, seed=1, class_w=np.ones(3, np.float32))
    assert losses[-1] < 0.5 * losses[0]
    acc = (model.predict(X).argmax(axis=1) == y).mean()
    assert acc > 0.95


def test_retirement_gain_over_plain_tracker():
    """Train on plain-FP64 tracks of three rounds, calibrate the threshold on a fourth
    (at most 0.1 % of the paths that do not fail would be retired), then track a fifth
    round with and without retirement: the network must cut work and keep the roots."""
    frg_build.build()
    task = precision_point_task(1, "disk")
    base = dict(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8)
    n, every = 16384, 32
    with frg.Tracker(frg.default_config(**base)) as t:
        X, y, _ = retire.training_set(t, task, [n], seeds=[101, 102, 103], max_checkpoints=64, every=every)
        Xc, yc, gc = retire.training_set(t, task, [n], seeds=[104], max_checkpoints=64, every=every)
    assert np.all(np.isfinite(X)) and (y == 1).sum() > 50 and (y == 0).sum() > 10000
    model, losses = retire.train(X, y, epochs=12, batch=2048, lr=2e-3, seed=3, every=every,
                                 class_w=np.array([1.0, 2.0, 1.0], np.float32))
    assert losses[-1] < losses[0]
    model.threshold = retire.calibrate(model, Xc, yc, gc, max_good_frac=1e-3)
    assert model.threshold < 1.0
    with frg.Tracker(frg.default_config(**base)) as t:
        plain = t.track(task, [n], 777, want_resid=True)
        model.apply(t)
        ret = t.track(task, [n], 777, want_resid=True)
    a = distinct_roots(plain.roots, plain.codes, plain.resid)
    b = distinct_roots(ret.roots, ret.codes, ret.resid)
    work_plain = plain.stats["ivp_solves"] + plain.stats["newton_iters"]
    work_ret = ret.stats["ivp_solves"] + ret.stats["newton_iters"]
    print(f"retired {ret.stats['retired']} paths at threshold {model.threshold:.4f}; solves {work_ret} vs "
          f"{work_plain}; time {ret.stats['track_ms']:.0f} vs {plain.stats['track_ms']:.0f} ms; "
          f"recall {recall(a, b):.5f}")
    assert ret.stats["retired"] > 0
    assert work_ret < work_plain
    assert recall(a, b) >= 0.995
