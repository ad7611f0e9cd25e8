"""The reference's own CUDA tracker (its Homotopy kernel, frg.cu:35-124, compiled
unchanged for this GPU and fed the tracker's Philox streams) against the CUDA tracker,
path for path, on the reference's target and gamma (frg.cu:41, :149-178).

Bar: codes equal on >= 99 % of the paths (the team kernel's structured elimination
rounds differently from the reference's dense LU, which can flip a path that sits on a
failure boundary; the thread kernel restates the dense LU); successful roots within
1e-8 relative on >= 99 % of the paths both finish. Needs the reference's sources staged
in oracle/_ref/src (they travel with the working tree); skipped where they are not.
"""
import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.tasks import REFERENCE_TARGET

pytestmark = pytest.mark.gpu

N = 256  # one block of the reference's 256 threads


@pytest.fixture(scope="module")
def reference_gpu_run():
    import oracle
    import refgpu

    if not oracle.ref_sources_staged():
        pytest.skip("the reference's sources are not staged in oracle/_ref/src")
    refgpu.build()
    g = refgpu.RefGPU("philox")
    roots, codes, _ = g.track(REFERENCE_TARGET, 4321, N)
    return roots, codes


@pytest.mark.parametrize("variant", [frg.KERNEL_TEAM, frg.KERNEL_THREAD], ids=["team", "thread"])
def test_reference_gpu_kernel_path_for_path(reference_gpu_run, variant):
    frg_build.build()
    r_roots, r_codes = reference_gpu_run
    with frg.Tracker(frg.default_config(kernel_variant=variant)) as t:
        res = t.track(REFERENCE_TARGET, [N], 4321, want_resid=True)
    assert (r_codes == 0).mean() > 0.9
    assert np.mean(res.codes == r_codes) >= 0.99, (res.codes, r_codes)
    both = (res.codes == 0) & (r_codes == 0)
    rel = np.max(np.abs(res.roots[both] - r_roots[both]), axis=1) / np.max(np.abs(r_roots[both]), axis=1)
    assert np.mean(rel <= 1e-8) >= 0.99, np.sort(rel)[-5:]
