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


def test_carry_handback_matches_single_calls():
    """carry_handback: a path handed back by round r's FP64 launch continues in round
    r + depth's FP32 launch. Per path this is frg_track with mixed_rounds = the number of
    rounds left on the path's stream (r, r + depth, ...), so the results are equal bit for
    bit. Short FP64 segments force many hand-backs."""
    frg_build.build()
    nrounds, depth = 5, 2
    sets = np.stack([np.stack([precision_point_task(40 + 2 * r + k, "disk" if k % 2 == 0 else "curve")
                               for k in range(2)]) for r in range(nrounds)])
    ppt, seeds = [512, 512], [61, 62, 63, 64, 65]
    n = sum(ppt)
    kw = dict(handback_good=4, fp64_segment=16, cond_switch=1e4)
    cfg = frg.chosen_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8,
                            carry_handback=1, **kw)
    with frg.Tracker(cfg) as t:
        roots = np.zeros((nrounds * n, 21), np.complex128)
        codes = np.zeros(nrounds * n, np.int32)
        resid = np.zeros(nrounds * n, np.float64)
        st = t.track_rounds(sets, ppt, seeds, roots, codes, resid=resid, depth=depth, per_round_tasks=True)
    assert st["handbacks"] > 0
    for r in range(nrounds):
        m = (nrounds - 1 - r) // depth + 1
        single_cfg = frg.chosen_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8,
                                       mixed_rounds=m, **kw)
        with frg.Tracker(single_cfg) as t:
            want = t.track(sets[r], ppt, seeds[r], want_resid=True)
        sl = slice(r * n, (r + 1) * n)
        assert np.array_equal(codes[sl], want.codes), r
        assert np.array_equal(roots[sl], want.roots), r
        assert np.array_equal(resid[sl], want.resid), r


def test_round_graph_matches_stream_launches():
    """round_graph: the carried rounds captured into one CUDA graph give the results of
    the same rounds launched one by one, bit for bit, with the same counters."""
    frg_build.build()
    nrounds, depth = 6, 3
    sets = np.stack([np.stack([precision_point_task(70 + r, "disk")]) for r in range(nrounds)])
    ppt, seeds = [768], [81, 82, 83, 84, 85, 86]
    out = {}
    for graph in (0, 1):
        cfg = frg.chosen_config(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8,
                                carry_handback=1, round_graph=graph, handback_good=8, fp64_segment=32)
        with frg.Tracker(cfg) as t:
            roots = np.zeros((nrounds * 768, 21), np.complex128)
            codes = np.zeros(nrounds * 768, np.int32)
            resid = np.zeros(nrounds * 768, np.float64)
            st = t.track_rounds(sets, ppt, seeds, roots, codes, resid=resid, depth=depth, per_round_tasks=True)
        out[graph] = (roots, codes, resid, st)
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][2], out[1][2])
    for key in ("codes", "ivp_solves", "newton_iters", "fp64_solves", "handbacks"):
        assert out[0][3][key] == out[1][3][key], key
    assert out[1][3]["handbacks"] > 0 and out[1][3]["track_ms"] > 0
