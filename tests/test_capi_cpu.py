"""CPU-side checks of the C-ABI library: it loads, exports every symbol that
include/frg_gb300.h declares, and its host-only parts (collection, Lambert W,
file formats) agree with the oracle and the reference's golden vectors."""
import os
import re

import numpy as np
import pytest

import finite_root_generation_gb300 as frg
from finite_root_generation_gb300 import build as frg_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="session")
def lib():
    frg_build.build()
    return frg.load()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "frg_gb300.h")).read()
    return sorted(set(re.findall(r"\b(frg_[a-z0-9_]+)\s*\(", text)))


def test_exports_match_header(lib):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", frg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (frg_[a-z0-9_]+)", out))
    declared = declared_functions()
    assert declared, "no declarations found"
    missing = [f for f in declared if f not in exported]
    assert not missing, f"declared but not exported: {missing}"
    assert sorted(frg.EXPORTS) == declared


def test_config_defaults_are_reference_constants(lib):
    c = frg.default_config()
    assert (c.s_init, c.s_max, c.s_min, c.rk_tol, c.caution_steps) == (1.0, 100.0, 1e-6, 1e-3, 2)
    assert (c.newt_its, c.newt_tol, c.newt_residual, c.newt_attempts) == (10, 1e-8, 1, 3)
    assert (c.sharp_its, c.sharp_tol, c.sharp_residual, c.sharp_attempts) == (30, 1e-12, 1, 3)
    assert (c.sharp_trigger, c.nudge_trigger, c.max_steps, c.max_ministeps) == (1e-5, 1e-5, 2000, 3000)
    assert (c.patch_range, c.start_range, c.dup_tol) == (2.0, 5.0, 1e-6)
    assert (c.gamma_re, c.gamma_im) == (0.39231132891081666, 1.0062265257923928)


def test_lambertw_matches_reference(lib, golden):
    for z, w in zip(golden["lw_z"], golden["lw_w"]):
        assert abs(frg.lambertw0(z) - w) < 1e-12 * max(1.0, abs(w))


def test_estimate_collected(lib):
    assert frg.estimate_collected(100, 0) == pytest.approx(0.0, abs=1e-12)
    # s = 1/2: 0.5 W(-2 e^-2) + 1 = 0.5 * (-2 + W-correction) ... value from the definition
    s = 0.5
    want = s * frg.lambertw0(-(1 / s) * np.exp(-1 / s)) + 1
    assert frg.estimate_collected(1, 1) == pytest.approx(want)
    assert 0.0 < want < 1.0


def test_collection_matches_reference_merge(lib, golden):
    coll = frg.Collection(1e-6)
    # seed the collection with the golden collection (a round of all-success roots)
    codes0 = coll.merge(golden["dd_coll"], np.zeros(len(golden["dd_coll"]), np.int32))
    assert np.all(codes0 == 0)
    codes = coll.merge(golden["dd_new"], golden["dd_codes_in"])
    assert np.array_equal(codes, golden["dd_codes_out"])
    assert np.array_equal(coll.roots(), golden["dd_merged"])


def test_collection_on_empty_and_matches_oracle(lib, oracle, golden):
    coll = frg.Collection(1e-6)
    codes = coll.merge(golden["dd_new"], golden["dd_codes_in"])
    assert np.array_equal(codes, golden["dd_codes_empty"])
    assert np.array_equal(coll.roots(), golden["dd_merged_empty"])
    # random rounds with planted duplicates: library and oracle agree
    rng = np.random.default_rng(5)
    coll2 = frg.Collection(1e-6)
    ocoll = np.zeros((0, 21), complex)
    for r in range(4):
        new = rng.uniform(-1, 1, (300, 21)) + 1j * rng.uniform(-1, 1, (300, 21))
        new[::7] = new[1::7][: len(new[::7])] + 3e-7
        if len(ocoll):
            new[5:40] = ocoll[: 35] + 1e-7
        codes = rng.choice([0, 0, 0, 0, 1, 5], size=300).astype(np.int32)
        got = coll2.merge(new, codes)
        ocoll, want = oracle.sort_merge(ocoll, new, codes)
        assert np.array_equal(got, want)
        assert np.array_equal(coll2.roots(), ocoll)


def test_empty_round(lib):
    coll = frg.Collection(1e-6)
    out = coll.merge(np.zeros((0, 21), complex), np.zeros(0, np.int32))
    assert len(out) == 0 and len(coll) == 0


def test_file_formats_roundtrip(lib, tmp_path):
    rng = np.random.default_rng(1)
    coll = frg.Collection(1e-6)
    new = rng.normal(size=(50, 21)) + 1j * rng.normal(size=(50, 21))
    coll.merge(new, np.zeros(50, np.int32))
    path = str(tmp_path / "fptColl")
    coll.save(path)
    assert os.path.getsize(path) == 50 * 336  # Vect<21> of cuDoubleComplex, frg.cu:472-476
    c2 = frg.Collection(1e-6)
    c2.load(path)
    assert np.array_equal(c2.roots(), coll.roots())
    # truncated file is rejected
    with open(path, "r+b") as f:
        f.truncate(50 * 336 - 8)
    with pytest.raises(frg.FrgError):
        frg.Collection(1e-6).load(path)
    # error codes append in int32 (frg.cu:478-480)
    cpath = str(tmp_path / "errorCodesAgr")
    frg.codes_append(cpath, [0, 6, 2])
    frg.codes_append(cpath, [5])
    assert np.array_equal(np.fromfile(cpath, np.int32), [0, 6, 2, 5])


def test_tracker_without_gpu_raises(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(frg.FrgError):
        frg.Tracker()


def test_invalid_configs_rejected_before_any_cuda_call():
    """frg_create checks the configuration first, so bad settings fail with FRG_ERR_ARG
    (-1) even on a machine without a GPU."""
    import ctypes

    lib = frg.load()
    bad = [dict(lo_refine=4), dict(lo_points=2), dict(fp64_budget=-1), dict(mixed_rounds=65), dict(path_offset=-1),
           dict(lo_final=2), dict(fp64_segment=-5), dict(handback_good=-1), dict(precision=7),
           dict(kernel_variant=9), dict(rk_tol=0.0), dict(newt_attempts=0),
           dict(precision=frg.PREC_MIXED, cond_switch=0.5)]
    for kw in bad:
        cfg = frg.default_config(**kw)
        ctx = ctypes.c_void_p()
        assert lib.frg_create(ctypes.byref(ctx), ctypes.byref(cfg), 0) == -1, kw
        assert not ctx.value


def test_noalloc_rejects_bad_arguments_without_a_gpu():
    import ctypes

    lib = frg.load()
    lib.frg_track_noalloc.restype = ctypes.c_int
    cfg = frg.default_config()
    ppt = (ctypes.c_int64 * 1)(4)
    assert lib.frg_track_noalloc(ctypes.byref(cfg), None, 1, ppt, ctypes.c_uint64(1), None, None, None, None) == -1
    many = frg.NOALLOC_MAX_TASKS + 1
    ppt_many = (ctypes.c_int64 * many)(*([1] * many))
    buf = (ctypes.c_double * 8)()
    assert lib.frg_track_noalloc(ctypes.byref(cfg), buf, many, ppt_many, ctypes.c_uint64(1), buf, buf, None,
                                 None) == -1
    # configurations frg_create refuses are refused before any GPU work (a negative
    # ministep limit would never end a rejecting path)
    for bad in (dict(max_ministeps=-1), dict(max_steps=-1), dict(s_min=0.0), dict(rk_tol=0.0),
                dict(gamma_mode=7), dict(start_dist=3), dict(path_offset=-5), dict(newt_attempts=0)):
        c = frg.default_config(**bad)
        assert lib.frg_track_noalloc(ctypes.byref(c), buf, 1, ppt, ctypes.c_uint64(1), buf, buf, None,
                                     None) == -1, bad
