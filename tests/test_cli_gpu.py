"""The multi-round driver end to end on the GPU: two pipelined rounds on the reference
target, files and progress in the reference's formats, and a resumed third round."""
import os

import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300 import cli

pytestmark = pytest.mark.gpu


def test_cli_rounds_and_resume(tmp_path):
    frg_build.build()
    d = str(tmp_path)
    cli.main(["--rounds", "2", "--paths", "512", "--dir", d, "--seed", "5", "--depth", "2"])
    codes = np.fromfile(os.path.join(d, "errorCodesAgr"), dtype=np.int32)
    assert len(codes) == 1024 and (codes == 0).mean() > 0.9
    coll = frg.Collection(1e-6)
    coll.load(os.path.join(d, "fptColl"))
    assert len(coll) == (codes == 0).sum()
    cli.main(["--rounds", "1", "--paths", "512", "--dir", d, "--seed", "5", "--precision", "mixed"])
    codes2 = np.fromfile(os.path.join(d, "errorCodesAgr"), dtype=np.int32)
    assert len(codes2) == 1536 and np.array_equal(codes2[:1024], codes)
    prog = open(os.path.join(d, "progress")).read()
    assert "-----Progress statistics for round 3-----" in prog and "Roots collected (est.):" in prog
