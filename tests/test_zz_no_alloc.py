"""frg_track_noalloc: tracking for callers that may not allocate device memory.

Such callers (code hosted in a framework that owns all device memory through its
own pool, or loops that cannot afford cudaFree's device-wide synchronisation) own
their input and output buffers; the entry point keeps its small scratch in a static
device array instead of allocating. This test calls it through the C ABI twice in a
row, with both kernel variants, with and without residual output, and checks each
result against frg_track on the same seed, and checks that a call beyond the
scratch's task limit is refused. It runs last (file name) so a
failure here cannot hide the other tests' results, and it needs nothing they set up.
"""
import ctypes

import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build
from finite_root_generation_gb300.tasks import REFERENCE_TARGET, precision_point_task

pytestmark = pytest.mark.gpu

ROOT_RTOL = 1e-8


def _rel(a, b):
    return np.max(np.abs(a - b), axis=-1) / np.maximum(np.max(np.abs(b), axis=-1), 1e-300)


@pytest.mark.parametrize("variant", [frg.KERNEL_TEAM, frg.KERNEL_THREAD], ids=["team", "thread"])
def test_noalloc_matches_frg_track_twice(variant):
    torch = pytest.importorskip("torch")
    frg_build.build()
    lib = frg.load()
    torch.cuda.set_device(0)
    cfg = frg.default_config(kernel_variant=variant)
    fpms = np.stack([REFERENCE_TARGET, precision_point_task(5, "disk")])
    ppt = np.array([48, 40], np.int64)
    n = int(ppt.sum())
    d_fpm = torch.from_numpy(fpms.view(np.float64).copy()).cuda()
    d_roots = torch.zeros((n, 42), dtype=torch.float64, device="cuda")
    d_codes = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    d_resid = torch.zeros(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row share the scratch array; the second one writes no residuals
    for seed, want_resid in ((1234, True), (99, False)):
        with frg.Tracker(cfg) as t:
            want = t.track(fpms, ppt, seed, want_resid=True)
        d_codes.fill_(-1)
        st = lib.frg_track_noalloc(ctypes.byref(cfg), d_fpm.data_ptr(), len(ppt),
                                   ppt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ctypes.c_uint64(seed),
                                   d_roots.data_ptr(), d_codes.data_ptr(),
                                   d_resid.data_ptr() if want_resid else None, ctypes.c_void_p(stream))
        assert st == 0
        torch.cuda.synchronize()
        codes = d_codes.cpu().numpy()
        roots = d_roots.cpu().numpy().view(np.complex128)
        assert np.array_equal(codes, want.codes)
        ok = want.codes == 0
        assert np.all(_rel(roots[ok], want.roots[ok]) < ROOT_RTOL)
        if want_resid:
            resid = d_resid.cpu().numpy()
            assert np.all(resid[ok] <= 1e-10)


def test_noalloc_rejects_too_many_tasks():
    torch = pytest.importorskip("torch")
    frg_build.build()
    lib = frg.load()
    cfg = frg.default_config()
    ntasks = frg.NOALLOC_MAX_TASKS + 1
    ppt = np.ones(ntasks, np.int64)
    d_fpm = torch.zeros((ntasks, 60), dtype=torch.float64, device="cuda")
    d_roots = torch.zeros((ntasks, 42), dtype=torch.float64, device="cuda")
    d_codes = torch.zeros(ntasks, dtype=torch.int32, device="cuda")
    st = lib.frg_track_noalloc(ctypes.byref(cfg), d_fpm.data_ptr(), ntasks,
                               ppt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ctypes.c_uint64(1),
                               d_roots.data_ptr(), d_codes.data_ptr(), None, None)
    assert st == -1  # FRG_ERR_ARG
    mixed = frg.default_config(precision=frg.PREC_MIXED)
    st = lib.frg_track_noalloc(ctypes.byref(mixed), d_fpm.data_ptr(), 1,
                               ppt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ctypes.c_uint64(1),
                               d_roots.data_ptr(), d_codes.data_ptr(), None, None)
    assert st == -1
