"""Autotuner: picks a setting that meets the recall target against plain FP64 on the
same seeds, re-validates it, caches it, and answers from the cache afterwards."""
import json

import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import autotune
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.tasks import precision_point_task

pytestmark = pytest.mark.gpu


def test_autotune_picks_caches_and_reuses(tmp_path, monkeypatch):
    frg_build.build()
    task = precision_point_task(2, "disk")
    base = dict(start_dist=frg.START_NORMAL, gamma_mode=frg.GAMMA_RANDOM, inf_tol=1e-8, lo_endgame=1)
    space = {"precision": [frg.PREC_MIXED], "lo_points": [0, 1], "depth": [1, 2]}
    cache = str(tmp_path / "tune.json")
    seen = []
    best = autotune.autotune(task, n=1024, rounds=1, base=base, space=space, target_recall=0.97, cache=cache,
                             device_name="test-gpu", log=seen.append)
    assert len(seen) == 4
    assert best["depth"] in (1, 2)
    store = json.load(open(cache))
    (entry,) = store.values()
    assert entry["best"] == best
    assert entry["plain_fp64_roots_per_s"] > 0
    if best.get("precision") == frg.PREC_MIXED:
        assert entry["revalidation"]["recall"] >= 0.97
        chosen = [c for c in entry["candidates"] if c["setting"] == best][0]
        assert chosen["recall"] >= 0.97
        assert chosen["roots_per_s"] == max(c["roots_per_s"] for c in entry["candidates"] if c["recall"] >= 0.97)

    def boom(*a, **k):
        raise AssertionError("the cached setting should be reused")

    monkeypatch.setattr(autotune, "_run", boom)
    assert autotune.autotune(task, n=1024, rounds=1, base=base, space=space, target_recall=0.97, cache=cache,
                             device_name="test-gpu") == best
