"""The benchmark's workload definition and its kept-root quality summary (CPU only)."""
import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("frg_bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_c5_steps_cover_every_task_once_per_pass():
    b = _bench()
    wl = b.Workload("c5")
    assert wl.ntasks == 128 and wl.paths_per_task == 8192 and wl.paths_per_step == 65536
    seen = [t for s in range(wl.blocks) for t in wl.step_tasks(s)]
    assert sorted(seen) == list(range(128))
    assert wl.step_tasks(16) == wl.step_tasks(0)  # the second pass repeats the tasks with new seeds
    sets = wl.task_sets([0, 1])
    assert sets.shape == (2, 8, 30) and np.array_equal(sets[1, 0], wl.tasks[8])
    # disk and curve tasks alternate; a disk task's points lie in the unit disk
    assert np.all(np.abs(wl.tasks[0][:16]) <= 1.0)


def test_kept_root_quality_summary():
    b = _bench()
    R = np.ones((5, 21), np.complex128)
    Rp = R.copy()
    Rp[4] *= 1.1
    C = np.array([0, 0, 0, 5, 0], np.int32)
    E = np.array([1e-12, 2e-10, 1e-13, 1e-12, 1e-12])
    q = b._kept_root_quality((R, C, E), (Rp, C, E))
    assert q["kept_roots"] == 3 and q["successes_failing_residual"] == 1
    assert q["kept_residual_max"] <= 1e-10
    assert q["paths_kept_by_both"] == 3 and abs(q["within_1e-8_of_fp64_track"] - 2 / 3) < 1e-4


def test_chosen_setting_is_the_tuned_one():
    """The benchmark applies frg.CHOSEN, then the autotuner's table entry for the GPU;
    the GPU parity tests run frg.CHOSEN. Every field the table sets agrees with CHOSEN,
    so the tested setting is the measured one."""
    import finite_root_generation_gb300 as frg
    from finite_root_generation_gb300 import autotune

    tuned = autotune.tuned_setting("NVIDIA GB300", "c5")
    assert tuned is not None
    tuned.pop("depth")
    cfg = frg.chosen_config()
    for key, v in tuned.items():
        assert getattr(cfg, key) == v, key
