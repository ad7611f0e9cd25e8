"""Pipelined rounds (frg_track_rounds) against one frg_track call per round: the same
roots and codes path for path, whatever the number of rounds in flight."""
import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.tasks import precision_point_task

pytestmark = pytest.mark.gpu


def _cfg(precision):
    return frg.default_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8,
                              precision=precision, lo_endgame=1)


@pytest.mark.parametrize("precision", [frg.PREC_FP64, frg.PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("depth", [1, 2, 3])
def test_rounds_match_single_calls(precision, depth):
    frg_build.build()
    task = precision_point_task(3, "disk")
    n, seeds = 1024, [11, 12, 13]
    with frg.Tracker(_cfg(precision)) as t:
        single = [t.track(task, [n], sd, want_resid=True) for sd in seeds]
        roots = np.zeros((len(seeds) * n, 21), np.complex128)
        codes = np.zeros(len(seeds) * n, np.int32)
        resid = np.zeros(len(seeds) * n, np.float64)
        st = t.track_rounds(task, [n], seeds, roots, codes, resid=resid, depth=depth)
    assert np.array_equal(codes, np.concatenate([r.codes for r in single]))
    assert np.array_equal(roots, np.concatenate([r.roots for r in single]))
    assert np.array_equal(resid, np.concatenate([r.resid for r in single]))
    assert st["paths"] == len(seeds) * n
    assert st["codes"] == [sum(r.stats["codes"][k] for r in single) for k in range(8)]
    assert st["ivp_solves"] == sum(r.stats["ivp_solves"] for r in single)
    assert st["track_ms"] > 0


def test_rounds_device_buffers():
    torch = pytest.importorskip("torch")
    frg_build.build()
    task = precision_point_task(4, "disk")
    n, seeds = 512, [5, 6]
    with frg.Tracker(_cfg(frg.PREC_MIXED)) as t:
        ref = [t.track(task, [n], sd) for sd in seeds]
        d_fpm = torch.from_numpy(task.view(np.float64).copy()).cuda()
        d_roots = torch.zeros((len(seeds) * n, 42), dtype=torch.float64, device="cuda")
        d_codes = torch.zeros(len(seeds) * n, dtype=torch.int32, device="cuda")
        t.track_rounds(d_fpm, [n], seeds, d_roots, d_codes, depth=2)
    got = d_roots.cpu().numpy().view(np.complex128)
    assert np.array_equal(d_codes.cpu().numpy(), np.concatenate([r.codes for r in ref]))
    assert np.array_equal(got, np.concatenate([r.roots for r in ref]))


def test_rounds_per_round_task_sets():
    """Each round tracks its own task set (a batch of tasks split into rounds): the same
    results as one frg_track call per round on that round's tasks."""
    frg_build.build()
    sets = np.stack([np.stack([precision_point_task(8 * r + k, "disk" if k % 2 == 0 else "curve")
                               for k in range(2)]) for r in range(3)])
    ppt, seeds = [256, 256], [21, 22, 23]
    n = sum(ppt)
    with frg.Tracker(_cfg(frg.PREC_MIXED)) as t:
        single = [t.track(sets[r], ppt, sd, want_resid=True) for r, sd in enumerate(seeds)]
        roots = np.zeros((len(seeds) * n, 21), np.complex128)
        codes = np.zeros(len(seeds) * n, np.int32)
        resid = np.zeros(len(seeds) * n, np.float64)
        t.track_rounds(sets, ppt, seeds, roots, codes, resid=resid, depth=2, per_round_tasks=True)
    assert np.array_equal(codes, np.concatenate([r.codes for r in single]))
    assert np.array_equal(roots, np.concatenate([r.roots for r in single]))
    assert np.array_equal(resid, np.concatenate([r.resid for r in single]))
