"""finite_root_generation_gb300: GB300-native finite-root-generation path tracker.

Python binding of the C ABI in ``include/frg_gb300.h`` (``libfrg_gb300.so``, built
in-tree by ``finite_root_generation_gb300.build``). It mirrors the reference's host
flow (frg.cu:351-514): track a round of paths from random start mechanisms to a task
(target precision-point parameters), then merge the round's roots into a collection
that marks duplicates (SortingDeletingMerging, frgsupport.cu:10-215).

The tracking runs only on the CUDA path: there is no CPU fallback, and every call
raises if the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfrg_gb300.so")

NV, NP, NY = 21, 30, 23
CODE_NAMES = {0: "success", 1: "max steps", 2: "max ministeps", 3: "predictor step below s_min",
              4: "corrector failed at s_min", 5: "sharpening failed", 6: "duplicate", 7: "infinite root"}

PREC_FP64, PREC_MIXED = 0, 1
START_UNIFORM, START_NORMAL = 0, 1
GAMMA_FIXED, GAMMA_RANDOM = 0, 1
KERNEL_TEAM, KERNEL_THREAD = 0, 1

_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)


class FrgError(RuntimeError):
    pass


class FrgConfig(ctypes.Structure):
    """``frg_config`` (include/frg_gb300.h)."""

    _fields_ = [
        ("s_init", ctypes.c_double), ("s_max", ctypes.c_double), ("s_min", ctypes.c_double),
        ("rk_tol", ctypes.c_double), ("caution_steps", ctypes.c_int),
        ("newt_its", ctypes.c_int), ("newt_tol", ctypes.c_double), ("newt_residual", ctypes.c_int),
        ("newt_attempts", ctypes.c_int),
        ("sharp_its", ctypes.c_int), ("sharp_tol", ctypes.c_double), ("sharp_residual", ctypes.c_int),
        ("sharp_attempts", ctypes.c_int),
        ("sharp_trigger", ctypes.c_double), ("nudge_trigger", ctypes.c_double),
        ("max_steps", ctypes.c_int), ("max_ministeps", ctypes.c_int),
        ("patch_range", ctypes.c_double),
        ("start_dist", ctypes.c_int), ("start_range", ctypes.c_double),
        ("gamma_mode", ctypes.c_int), ("gamma_re", ctypes.c_double), ("gamma_im", ctypes.c_double),
        ("dup_tol", ctypes.c_double),
        ("precision", ctypes.c_int), ("t_switch", ctypes.c_double), ("cond_switch", ctypes.c_double),
        ("inf_tol", ctypes.c_double),
        ("threads_per_block", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
        ("newt_tol_lo", ctypes.c_double), ("kernel_variant", ctypes.c_int),
        ("mixed_rounds", ctypes.c_int), ("lo_refine", ctypes.c_int), ("lo_endgame", ctypes.c_int),
        ("path_offset", ctypes.c_int64), ("fp64_budget", ctypes.c_int), ("lo_points", ctypes.c_int),
        ("fp64_segment", ctypes.c_int), ("handback_good", ctypes.c_int), ("lo_final", ctypes.c_int),
        ("carry_handback", ctypes.c_int), ("round_graph", ctypes.c_int), ("system", ctypes.c_int),
    ]


class FrgSystemDesc(ctypes.Structure):
    """``frg_system_desc`` (include/frg_gb300.h)."""

    _fields_ = [("name", ctypes.c_char * 32), ("nv", ctypes.c_int), ("np", ctypes.c_int)]


class FrgStats(ctypes.Structure):
    """``frg_stats`` (include/frg_gb300.h)."""

    _fields_ = [
        ("paths", ctypes.c_int64), ("codes", ctypes.c_int64 * 8), ("ivp_solves", ctypes.c_int64),
        ("newton_iters", ctypes.c_int64), ("fp64_solves", ctypes.c_int64), ("steps", ctypes.c_int64),
        ("track_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("handoffs", ctypes.c_int64),
        ("stage_ms", ctypes.c_double * 2), ("handoff_reason", ctypes.c_int64 * 6),
        ("kernel_cycles", ctypes.c_int64 * 12), ("handbacks", ctypes.c_int64),
        ("refine_solves", ctypes.c_int64), ("refine_warp_steps", ctypes.c_int64),
        ("round_ms", ctypes.c_double * 32), ("fp64_segment_hist", ctypes.c_int64 * 6),
        ("fp64_segment_max", ctypes.c_int64), ("retired", ctypes.c_int64), ("refine_cycles", ctypes.c_int64),
    ]

    def as_dict(self) -> dict:
        return {"paths": self.paths, "codes": list(self.codes), "ivp_solves": self.ivp_solves,
                "newton_iters": self.newton_iters, "fp64_solves": self.fp64_solves, "steps": self.steps,
                "track_ms": self.track_ms, "total_ms": self.total_ms, "handoffs": self.handoffs,
                "stage_ms": list(self.stage_ms), "handoff_reason": list(self.handoff_reason),
                "kernel_cycles": list(self.kernel_cycles), "handbacks": self.handbacks,
                "refine_solves": self.refine_solves, "refine_warp_steps": self.refine_warp_steps,
                "round_ms": list(self.round_ms), "fp64_segment_hist": list(self.fp64_segment_hist),
                "fp64_segment_max": self.fp64_segment_max, "retired": self.retired,
                "refine_cycles": self.refine_cycles}


# Exported symbols of libfrg_gb300.so, one per declaration in include/frg_gb300.h.
EXPORTS = [
    "frg_config_default", "frg_create", "frg_destroy", "frg_last_error", "frg_set_config", "frg_track",
    "frg_track_async", "frg_coll_create", "frg_coll_destroy", "frg_coll_size", "frg_coll_get", "frg_coll_merge",
    "frg_coll_save", "frg_coll_load", "frg_codes_append", "frg_lambertw0", "frg_estimate_collected",
    "frg_track_noalloc", "frg_track_rounds", "frg_set_mlp", "frg_track_features", "frg_mlp_param_count",
    "frg_mlp_grad", "frg_mlp_train", "frg_mlp_predict", "frg_dcoll_create", "frg_dcoll_destroy", "frg_dcoll_merge",
    "frg_dcoll_size", "frg_dcoll_get", "frg_system_info", "frg_num_systems",
]
NOALLOC_MAX_TASKS = 1024

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libfrg_gb300.so; raises FrgError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FrgError(f"{path} is missing: build it with `python -m finite_root_generation_gb300.build` "
                       "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    lib.frg_last_error.restype = ctypes.c_char_p
    lib.frg_lambertw0.restype = ctypes.c_double
    lib.frg_lambertw0.argtypes = [ctypes.c_double]
    lib.frg_estimate_collected.restype = ctypes.c_double
    lib.frg_estimate_collected.argtypes = [ctypes.c_int64, ctypes.c_int64]
    lib.frg_coll_size.restype = ctypes.c_int64
    lib.frg_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(FrgConfig), ctypes.c_int]
    lib.frg_track.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _I64, ctypes.c_uint64,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.POINTER(FrgStats)]
    lib.frg_track_async.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _I64, ctypes.c_uint64,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]
    lib.frg_track_rounds.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _I64, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_uint64), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(FrgStats)]
    _F = ctypes.POINTER(ctypes.c_float)
    lib.frg_set_mlp.argtypes = [ctypes.c_void_p, _F, _F, _F, ctypes.c_float, ctypes.c_int]
    lib.frg_track_features.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _I64, ctypes.c_uint64,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _F,
                                       ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(FrgStats)]
    lib.frg_mlp_param_count.restype = ctypes.c_int
    lib.frg_mlp_grad.argtypes = [_F, ctypes.POINTER(ctypes.c_int32), ctypes.c_int64, _F, _F, _F,
                                 ctypes.POINTER(ctypes.c_double)]
    lib.frg_mlp_train.argtypes = [_F, ctypes.POINTER(ctypes.c_int32), ctypes.c_int64, _F, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_float, ctypes.c_uint64, _F, ctypes.POINTER(ctypes.c_double)]
    lib.frg_mlp_predict.argtypes = [_F, ctypes.c_int64, _F, _F]
    lib.frg_destroy.argtypes = [ctypes.c_void_p]
    lib.frg_last_error.argtypes = [ctypes.c_void_p]
    lib.frg_set_config.argtypes = [ctypes.c_void_p, ctypes.POINTER(FrgConfig)]
    for name in ("frg_coll_destroy", "frg_coll_size"):
        getattr(lib, name).argtypes = [ctypes.c_void_p]
    lib.frg_coll_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_double]
    lib.frg_coll_get.argtypes = [ctypes.c_void_p, _D, ctypes.c_int64]
    lib.frg_coll_merge.argtypes = [ctypes.c_void_p, _D, _I32, ctypes.c_int64]
    lib.frg_coll_save.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.frg_coll_load.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.frg_codes_append.argtypes = [ctypes.c_char_p, _I32, ctypes.c_int64]
    lib.frg_dcoll_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int64, ctypes.c_double]
    lib.frg_dcoll_destroy.argtypes = [ctypes.c_void_p]
    lib.frg_dcoll_merge.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_double, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    lib.frg_dcoll_size.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
    lib.frg_dcoll_get.argtypes = [ctypes.c_void_p, _D, _I32, ctypes.c_int64]
    lib.frg_track_noalloc.argtypes = [ctypes.POINTER(FrgConfig), ctypes.c_void_p, ctypes.c_int, _I64,
                                      ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
    lib.frg_system_info.argtypes = [ctypes.c_int, ctypes.POINTER(FrgSystemDesc)]
    lib.frg_num_systems.restype = ctypes.c_int
    _lib = lib
    return lib


@dataclass
class SystemInfo:
    id: int
    name: str
    nv: int   # unknowns of a root
    np: int   # parameters of a task


def system_info(system: int) -> SystemInfo:
    """The system `system` tracks (0 = Stephenson II, k >= 1 = plug-in k, the modules of
    finite_root_generation_gb300/systems in the order of systems.PLUGINS)."""
    d = FrgSystemDesc()
    if load().frg_system_info(int(system), ctypes.byref(d)) != 0:
        raise FrgError(f"unknown system {system}")
    return SystemInfo(int(system), d.name.decode(), d.nv, d.np)


def list_systems() -> list:
    """Every system the library was built with."""
    return [system_info(k) for k in range(load().frg_num_systems())]


def plugin_config(name: str, **overrides) -> FrgConfig:
    """default_config for the plug-in system `name` on the thread kernel (FP64 unless
    `overrides` set precision=PREC_MIXED: the FP32 stage with hand-off to FP64)."""
    for s in list_systems():
        if s.name == name:
            kw = dict(system=s.id, precision=PREC_FP64, kernel_variant=KERNEL_THREAD)
            kw.update(overrides)
            return default_config(**kw)
    raise FrgError(f"no system named {name}")


def default_config(**overrides) -> FrgConfig:
    """The reference's defaults (htpytrack.cu:9-31, frgkinematics.cu:7-8, frg.cu:41, frgsupport.cu:7)."""
    cfg = FrgConfig()
    load().frg_config_default(ctypes.byref(cfg))
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise AttributeError(f"frg_config has no field {k}")
        setattr(cfg, k, v)
    return cfg


# The chosen mixed-precision setting of the benchmark: FP32 team kernel with double-float
# points that also runs the endgame and sharpening; its corrector accepts an FP32 update
# below 1e-5 and otherwise refines on double-float residuals to 1e-8; FP64 for steps whose
# condition estimate exceeds 1e6 and for finishing every root, at most 10,000 FP64 solves
# per path and launch; in frg_track_rounds a path well conditioned again in FP64 (32
# solves below 1e4, or 256 FP64 solves) is carried back to FP32 in a later round, and the
# rounds run as one CUDA graph. The fields the autotuner searches agree with its GB300
# entry for the 128-task workload (tuned.json).
CHOSEN = dict(precision=PREC_MIXED, mixed_rounds=1, lo_endgame=1, cond_switch=1e6, lo_points=1, fp64_budget=10000,
              lo_refine=3, newt_tol_lo=1e-5, carry_handback=1, handback_good=32, fp64_segment=256, round_graph=1)


def chosen_config(**overrides) -> FrgConfig:
    """default_config with the chosen mixed-precision setting (CHOSEN) and `overrides`."""
    kw = dict(CHOSEN)
    kw.update(overrides)
    return default_config(**kw)


def _ptr(a) -> int:
    """Address of a numpy array or torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(type(a))


@dataclass
class TrackResult:
    roots: np.ndarray       # [N, nv] complex128, dehomogenized (Stephenson II: canonical cognate)
    codes: np.ndarray       # [N] int32
    yfinal: np.ndarray | None
    resid: np.ndarray | None
    stats: dict


class Tracker:
    """A tracking context on one GPU (``frg_ctx``)."""

    def __init__(self, config: FrgConfig | None = None, device: int = 0):
        self.lib = load()
        self._ctx = ctypes.c_void_p()
        cfg = config if config is not None else default_config()
        st = self.lib.frg_create(ctypes.byref(self._ctx), ctypes.byref(cfg), device)
        if st != 0:
            raise FrgError(f"frg_create failed with status {st} (no usable CUDA device {device}?)")
        self.config = cfg

    def close(self):
        if self._ctx:
            self.lib.frg_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int, what: str):
        if st != 0:
            msg = self.lib.frg_last_error(self._ctx)
            raise FrgError(f"{what} failed ({st}): {msg.decode() if msg else ''}")

    def set_config(self, cfg: FrgConfig):
        self._check(self.lib.frg_set_config(self._ctx, ctypes.byref(cfg)), "frg_set_config")
        self.config = cfg

    @property
    def dims(self):
        """(unknowns, parameters) of the configured system."""
        if self.config.system == 0:
            return NV, NP
        info = system_info(self.config.system)
        return info.nv, info.np

    def track(self, fpm, paths_per_task, seed: int, want_yfinal: bool = False,
              want_resid: bool = False) -> TrackResult:
        """Track sum(paths_per_task) paths; fpm is [ntasks, np] complex (host; np = 30 for
        Stephenson II). Roots are [N, nv], yfinal [N, nv + 2]."""
        nv, np_ = self.dims
        fpm = np.ascontiguousarray(np.asarray(fpm, dtype=np.complex128).reshape(-1, np_))
        ppt = np.ascontiguousarray(np.atleast_1d(np.asarray(paths_per_task, dtype=np.int64)))
        if len(ppt) != len(fpm):
            raise ValueError("paths_per_task must have one entry per task")
        n = int(ppt.sum())
        roots = np.zeros((n, nv), np.complex128)
        codes = np.zeros(n, np.int32)
        yfinal = np.zeros((n, nv + 2), np.complex128) if want_yfinal else None
        resid = np.zeros(n, np.float64) if want_resid else None
        stats = FrgStats()
        st = self.lib.frg_track(self._ctx, fpm.ctypes.data, len(ppt), ppt.ctypes.data_as(_I64),
                                ctypes.c_uint64(seed), roots.ctypes.data, codes.ctypes.data,
                                _ptr(yfinal), _ptr(resid), ctypes.byref(stats))
        self._check(st, "frg_track")
        return TrackResult(roots, codes, yfinal, resid, stats.as_dict())

    def track_into(self, fpm, paths_per_task, seed: int, roots, codes, yfinal=None, resid=None) -> dict:
        """Track into caller-owned buffers (numpy host arrays or torch CUDA tensors)."""
        ppt = np.ascontiguousarray(np.atleast_1d(np.asarray(paths_per_task, dtype=np.int64)))
        stats = FrgStats()
        st = self.lib.frg_track(self._ctx, _ptr(fpm), len(ppt), ppt.ctypes.data_as(_I64), ctypes.c_uint64(seed),
                                _ptr(roots), _ptr(codes), _ptr(yfinal), _ptr(resid), ctypes.byref(stats))
        self._check(st, "frg_track")
        return stats.as_dict()

    def track_rounds(self, fpm, paths_per_task, seeds, roots, codes, resid=None, depth: int = 2,
                     per_round_tasks: bool = False) -> dict:
        """Track len(seeds) rounds, up to `depth` in flight (frg_track_rounds); outputs are
        [rounds * N, ...] buffers, all numpy host arrays or all torch CUDA tensors. With
        per_round_tasks, fpm holds one task set per round ([rounds, ntasks, 30] complex)."""
        ppt = np.ascontiguousarray(np.atleast_1d(np.asarray(paths_per_task, dtype=np.int64)))
        sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
        stats = FrgStats()
        st = self.lib.frg_track_rounds(self._ctx, _ptr(fpm), len(ppt), ppt.ctypes.data_as(_I64), len(sd),
                                       sd.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                       1 if per_round_tasks else 0, int(depth), _ptr(roots),
                                       _ptr(codes), _ptr(resid), ctypes.byref(stats))
        self._check(st, "frg_track_rounds")
        return stats.as_dict()

    def set_mlp(self, params=None, mu=None, inv_sigma=None, threshold: float = 0.99, every: int = 32):
        """Switch early retirement on (params: frg_mlp_param_count() FP32 weights) or off (None)."""
        if params is None:
            self._check(self.lib.frg_set_mlp(self._ctx, None, None, None, ctypes.c_float(1.0), 1), "frg_set_mlp")
            return
        p = np.ascontiguousarray(params, np.float32)
        m = np.ascontiguousarray(mu, np.float32)
        s = np.ascontiguousarray(inv_sigma, np.float32)
        _F = ctypes.POINTER(ctypes.c_float)
        self._check(self.lib.frg_set_mlp(self._ctx, p.ctypes.data_as(_F), m.ctypes.data_as(_F), s.ctypes.data_as(_F),
                                         ctypes.c_float(threshold), int(every)), "frg_set_mlp")

    def track_features(self, fpm, paths_per_task, seed: int, max_checkpoints: int = 16, every: int = 32):
        """frg_track that also returns every path's checkpoint features
        (features [N, max_checkpoints, 32], nfeat [N])."""
        fpm = np.ascontiguousarray(np.asarray(fpm, dtype=np.complex128).reshape(-1, NP))
        ppt = np.ascontiguousarray(np.atleast_1d(np.asarray(paths_per_task, dtype=np.int64)))
        n = int(ppt.sum())
        roots = np.zeros((n, NV), np.complex128)
        codes = np.zeros(n, np.int32)
        resid = np.zeros(n, np.float64)
        feats = np.zeros((n, max_checkpoints, 32), np.float32)
        nfeat = np.zeros(n, np.int32)
        stats = FrgStats()
        st = self.lib.frg_track_features(self._ctx, fpm.ctypes.data, len(ppt), ppt.ctypes.data_as(_I64),
                                         ctypes.c_uint64(seed), roots.ctypes.data, codes.ctypes.data,
                                         resid.ctypes.data, feats.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                         nfeat.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), int(max_checkpoints),
                                         int(every), ctypes.byref(stats))
        self._check(st, "frg_track_features")
        return TrackResult(roots, codes, None, resid, stats.as_dict()), feats, nfeat

    def track_async(self, fpm, paths_per_task, seed: int, roots, codes, yfinal=None, resid=None, stream=0):
        """Enqueue on a CUDA stream (device buffers only); returns immediately."""
        ppt = np.ascontiguousarray(np.atleast_1d(np.asarray(paths_per_task, dtype=np.int64)))
        st = self.lib.frg_track_async(self._ctx, _ptr(fpm), len(ppt), ppt.ctypes.data_as(_I64),
                                      ctypes.c_uint64(seed), _ptr(roots), _ptr(codes), _ptr(yfinal),
                                      _ptr(resid), ctypes.c_void_p(stream))
        self._check(st, "frg_track_async")


class Collection:
    """Sorted root collection with duplicate marking (``frg_coll``)."""

    def __init__(self, dup_tol: float = 1e-6):
        self.lib = load()
        self._c = ctypes.c_void_p()
        if self.lib.frg_coll_create(ctypes.byref(self._c), ctypes.c_double(dup_tol)) != 0:
            raise FrgError("frg_coll_create failed")

    def __del__(self):
        try:
            if self._c:
                self.lib.frg_coll_destroy(self._c)
        except Exception:
            pass

    def __len__(self) -> int:
        return int(self.lib.frg_coll_size(self._c))

    def roots(self) -> np.ndarray:
        n = len(self)
        out = np.zeros((n, NV), np.complex128)
        if self.lib.frg_coll_get(self._c, out.ctypes.data_as(_D), ctypes.c_int64(n)) != 0:
            raise FrgError("frg_coll_get failed")
        return out

    def merge(self, roots, codes) -> np.ndarray:
        """Merge a round; returns the codes with duplicates marked 6."""
        roots = np.ascontiguousarray(np.asarray(roots, np.complex128).reshape(-1, NV))
        codes = np.ascontiguousarray(np.asarray(codes, np.int32)).copy()
        st = self.lib.frg_coll_merge(self._c, roots.ctypes.data_as(_D), codes.ctypes.data_as(_I32),
                                     ctypes.c_int64(len(codes)))
        if st != 0:
            raise FrgError(f"frg_coll_merge failed ({st})")
        return codes

    def save(self, path: str):
        if self.lib.frg_coll_save(self._c, path.encode()) != 0:
            raise FrgError(f"cannot write {path}")

    def load(self, path: str):
        if self.lib.frg_coll_load(self._c, path.encode()) != 0:
            raise FrgError(f"cannot read {path} (missing, truncated or unsorted)")


class DeviceCollection:
    """Device-resident root collection (``frg_dcoll``): duplicate marking on the GPU with
    the host Collection's rule, one collection per key (e.g. per task)."""

    def __init__(self, capacity: int, dup_tol: float = 1e-6, device: int = 0):
        self.lib = load()
        self._c = ctypes.c_void_p()
        st = self.lib.frg_dcoll_create(ctypes.byref(self._c), int(device), ctypes.c_int64(capacity),
                                       ctypes.c_double(dup_tol))
        if st != 0:
            raise FrgError(f"frg_dcoll_create failed ({st})")

    def close(self):
        if self._c:
            self.lib.frg_dcoll_destroy(self._c)
            self._c = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def merge(self, roots, codes, keys=None, stream=0, resid=None, resid_max=1e-10):
        """Merge device buffers (torch CUDA tensors): roots [n, 42] float64, codes [n]
        int32 (marked 6 in place), keys [n] int32 or None; with resid [n] float64, a success
        whose residual exceeds resid_max takes no part."""
        n = int(codes.numel())
        st = self.lib.frg_dcoll_merge(self._c, _ptr(roots), _ptr(codes), _ptr(resid), ctypes.c_double(resid_max),
                                      _ptr(keys), ctypes.c_int64(n), ctypes.c_void_p(stream))
        if st != 0:
            raise FrgError(f"frg_dcoll_merge failed ({st})")

    def size(self, stream=0) -> int:
        n = ctypes.c_int64()
        st = self.lib.frg_dcoll_size(self._c, ctypes.c_void_p(stream), ctypes.byref(n))
        if st != 0:
            raise FrgError(f"frg_dcoll_size failed ({st})")
        return int(n.value)

    def __len__(self) -> int:
        return self.size()

    def roots(self):
        """(roots [m, 21] complex, keys [m]) in collection order."""
        m = self.size()
        out = np.zeros((m, NV), np.complex128)
        keys = np.zeros(m, np.int32)
        if m and self.lib.frg_dcoll_get(self._c, out.ctypes.data_as(_D), keys.ctypes.data_as(_I32),
                                        ctypes.c_int64(m)) != 0:
            raise FrgError("frg_dcoll_get failed")
        return out, keys


def codes_append(path: str, codes) -> None:
    codes = np.ascontiguousarray(np.asarray(codes, np.int32))
    if load().frg_codes_append(path.encode(), codes.ctypes.data_as(_I32), ctypes.c_int64(len(codes))) != 0:
        raise FrgError(f"cannot append to {path}")


def lambertw0(z: float) -> float:
    return float(load().frg_lambertw0(float(z)))


def estimate_collected(successes: int, duplicates: int) -> float:
    return float(load().frg_estimate_collected(int(successes), int(duplicates)))
