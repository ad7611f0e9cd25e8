"""The multi-round driver (cli.run) with a stand-in tracker (CPU only): files in the
reference's formats, progress sections, resume from an existing directory, and the
stop on the estimated share of roots collected."""
import os

import numpy as np

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import cli

POOL = np.random.default_rng(0).normal(size=(300, 21)) + 1j * np.random.default_rng(1).normal(size=(300, 21))


def fake_rounds(n):
    def track(seeds):
        roots, codes = [], []
        for sd in seeds:
            rng = np.random.default_rng(sd)
            pick = rng.integers(0, len(POOL), size=n)
            roots.append(POOL[pick])
            c = np.zeros(n, np.int32)
            c[rng.random(n) < 0.05] = 4
            codes.append(c)
        return np.concatenate(roots), np.concatenate(codes)
    return track


def test_rounds_files_and_resume(tmp_path):
    n, d = 64, str(tmp_path)
    assert cli.run(fake_rounds(n), n, 3, d, seed0=10, depth=2, log=None) == 3
    codes = np.fromfile(os.path.join(d, "errorCodesAgr"), dtype=np.int32)
    assert len(codes) == 3 * n
    coll = frg.Collection(1e-6)
    coll.load(os.path.join(d, "fptColl"))
    assert len(coll) == (codes == 0).sum()          # every success is a new root
    assert set(np.unique(codes)) <= {0, 4, 6}
    prog = open(os.path.join(d, "progress")).read()
    assert prog.count("-----Progress statistics for round") == 3
    assert "-----Progress statistics for round 3-----" in prog
    assert f"Trials:         {3 * n:>10}" in prog
    # resume: two more rounds continue the totals and the round numbers
    assert cli.run(fake_rounds(n), n, 2, d, seed0=10, depth=1, log=None) == 2
    codes2 = np.fromfile(os.path.join(d, "errorCodesAgr"), dtype=np.int32)
    assert len(codes2) == 5 * n and np.array_equal(codes2[:3 * n], codes)
    prog = open(os.path.join(d, "progress")).read()
    assert "-----Progress statistics for round 5-----" in prog
    coll2 = frg.Collection(1e-6)
    coll2.load(os.path.join(d, "fptColl"))
    assert len(coll2) == (codes2 == 0).sum() and len(coll2) >= len(coll)


def test_stop_on_estimated_coverage(tmp_path):
    n = 256
    done = cli.run(fake_rounds(n), n, 50, str(tmp_path), seed0=3, depth=1, stop_at=0.95, log=None)
    assert done < 50
    coll = frg.Collection(1e-6)
    coll.load(os.path.join(str(tmp_path), "fptColl"))
    assert len(coll) >= 0.9 * len(POOL)
