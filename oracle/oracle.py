"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

ctypes binding for the plain-C restatement of the reference tracker
(``oracle/frg_oracle.c`` -> ``oracle/_ref/libfrgoracle.so``) and, where it was built
(only where the reference sources exist), for the host build of the reference's own
sources (``oracle/_ref/libfrgref.so``).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module, and only as the checker.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(REF_DIR, "libfrgoracle.so")
REF_SO = os.path.join(REF_DIR, "libfrgref.so")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U64 = ctypes.POINTER(ctypes.c_uint64)


class OrConfig(ctypes.Structure):
    """Mirror of ``or_config`` in frg_oracle.h (defaults: htpytrack.cu:9-31)."""

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
    ]


class OrStats(ctypes.Structure):
    _fields_ = [("rk_attempts", ctypes.c_int64), ("ivp_solves", ctypes.c_int64),
                ("newton_iters", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("newton_calls", ctypes.c_int64)]


REF_SRC = os.path.join(REF_DIR, "src")


def ref_sources_staged() -> bool:
    """True when the reference's sources were staged into oracle/_ref/src (git-ignored;
    `make -C oracle stage REF=<reference checkout>`), so libfrgref.so can be built here."""
    return os.path.exists(os.path.join(REF_SRC, "htpytrack.cu"))


def stage(ref_dir: str) -> None:
    """Copy the reference sources this build needs from `ref_dir` into oracle/_ref/src."""
    subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF={ref_dir}"], check=True)


def build(ref: bool = False) -> None:
    """Compile the oracle (and, if asked and the staged sources exist, the reference) with make."""
    targets = ["port"]
    if ref and ref_sources_staged():
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _c(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


class Oracle:
    """The C restatement. Complex arguments are numpy complex128 arrays."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        self.lib = ctypes.CDLL(path)
        self.lib.or_lambertw0.restype = ctypes.c_double
        self.lib.or_lambertw0.argtypes = [ctypes.c_double]
        self.lib.or_sort_merge.restype = ctypes.c_int64
        self.prefix = "or_"

    # ---- configuration -------------------------------------------------
    def config(self, **kw) -> OrConfig:
        c = OrConfig()
        self.lib.or_config_default(ctypes.byref(c))
        for k, v in kw.items():
            setattr(c, k, v)
        return c

    # ---- system --------------------------------------------------------
    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def fsys(self, Z, q):
        out = np.zeros(21, np.complex128)
        self._fn("fsys")(_p(_c(Z)), _p(_c(q)), _p(out))
        return out

    def jvar(self, Z, q):
        out = np.zeros((21, 22), np.complex128)
        self._fn("jvar")(_p(_c(Z)), _p(_c(q)), _p(out))
        return out

    def jpar(self, Z, q):
        out = np.zeros((21, 30), np.complex128)
        self._fn("jpar")(_p(_c(Z)), _p(_c(q)), _p(out))
        return out

    def q(self, t, spm, fpm, gamma):
        out = np.zeros(30, np.complex128)
        g = _c([gamma])
        self._fn("q")(ctypes.c_double(t), _p(_c(spm)), _p(_c(fpm)), _p(g), _p(out))
        return out

    def dqdt(self, t, spm, fpm, gamma):
        out = np.zeros(30, np.complex128)
        g = _c([gamma])
        self._fn("dqdt")(ctypes.c_double(t), _p(_c(spm)), _p(_c(fpm)), _p(g), _p(out))
        return out

    def h(self, Y, u, spm, fpm, gamma):
        out = np.zeros(22, np.complex128)
        self._fn("h")(_p(_c(Y)), _p(_c(u)), _p(_c(spm)), _p(_c(fpm)), _p(_c([gamma])), _p(out))
        return out

    def jh(self, Y, u, spm, fpm, gamma):
        out = np.zeros((22, 23), np.complex128)
        self._fn("jh")(_p(_c(Y)), _p(_c(u)), _p(_c(spm)), _p(_c(fpm)), _p(_c([gamma])), _p(out))
        return out

    def switch_patch(self, u, Y):
        out = np.zeros(23, np.complex128)
        self._fn("switch_patch")(_p(_c(u)), _p(_c(Y)), _p(out))
        return out

    def ivp(self, tstepQ, Yc, Vc, u, spm, fpm, gamma):
        out = np.zeros(23, np.complex128)
        self._fn("ivp")(ctypes.c_int(int(tstepQ)), _p(_c(Yc)), _p(_c(Vc)), _p(_c(u)), _p(_c(spm)),
                        _p(_c(fpm)), _p(_c([gamma])), _p(out))
        return out

    def dp65(self, s, tol, tstepQ, Yc, Vc, u, spm, fpm, gamma):
        Yn = np.zeros(23, np.complex128)
        Vn = np.zeros(23, np.complex128)
        err = ctypes.c_double()
        sc = ctypes.c_double()
        self._fn("dp65")(ctypes.c_double(s), ctypes.c_double(tol), ctypes.c_int(int(tstepQ)),
                         _p(_c(Yc)), _p(_c(Vc)), _p(_c(u)), _p(_c(spm)), _p(_c(fpm)),
                         _p(_c([gamma])), _p(Yn), _p(Vn), ctypes.byref(err), ctypes.byref(sc))
        return Yn, Vn, err.value, sc.value

    def newton(self, tgoal, Vn, u, spm, fpm, gamma, maxits, tol, restype, Y0):
        Y = _c(Y0).copy()
        res = ctypes.c_double()
        self._fn("newton")(ctypes.c_double(tgoal), _p(_c(Vn)), _p(_c(u)), _p(_c(spm)), _p(_c(fpm)),
                           _p(_c([gamma])), ctypes.c_int(maxits), ctypes.c_double(tol),
                           ctypes.c_int(restype), _p(Y), ctypes.byref(res))
        return Y, res.value

    def cognate(self, z, q):
        out = np.zeros((2, 21), np.complex128)
        self._fn("cognate")(_p(_c(z)), _p(_c(q)), _p(out))
        return out

    # ---- paths ---------------------------------------------------------
    def generate_start(self, seed, stream, cfg: OrConfig | None = None):
        cfg = cfg or self.config()
        spt = np.zeros(21, np.complex128)
        spm = np.zeros(30, np.complex128)
        self.lib.or_generate_start(ctypes.byref(cfg), ctypes.c_uint64(seed), ctypes.c_uint64(stream),
                                   _p(spt), _p(spm))
        return spt, spm

    def track_path(self, spt, spm, fpm, gamma, seed, stream, cfg: OrConfig | None = None):
        cfg = cfg or self.config()
        Y = np.zeros(23, np.complex128)
        code = ctypes.c_int()
        stt = OrStats()
        self.lib.or_track_path(ctypes.byref(cfg), _p(_c(spt)), _p(_c(spm)), _p(_c(fpm)),
                               _p(_c([gamma])), ctypes.c_uint64(seed), ctypes.c_uint64(stream),
                               _p(Y), ctypes.byref(code), ctypes.byref(stt))
        return Y, code.value, stt

    def homotopy_batch(self, fpm, gamma, seed, streams, cfg: OrConfig | None = None, nthreads=None,
                       want_yfinal=False):
        """Run the reference kernel body (frg.cu:41-68) for each stream; returns
        (roots [n,21] complex, codes [n], work [n,3] = ivp solves, newton iters, steps, yfinal)."""
        cfg = cfg or self.config()
        streams = np.ascontiguousarray(np.asarray(streams, dtype=np.uint64))
        n = len(streams)
        roots = np.zeros((n, 21), np.complex128)
        codes = np.zeros(n, np.int32)
        work = np.zeros((n, 3), np.int64)
        yf = np.zeros((n, 23), np.complex128) if want_yfinal else None
        nthreads = nthreads or os.cpu_count() or 1
        self.lib.or_homotopy_batch(ctypes.byref(cfg), ctypes.c_uint64(seed),
                                   streams.ctypes.data_as(_U64), ctypes.c_int64(n),
                                   _p(_c(fpm)), _p(_c([gamma])), _p(roots), codes.ctypes.data_as(_I),
                                   _p(yf) if yf is not None else None,
                                   work.ctypes.data_as(_I64), ctypes.c_int(nthreads))
        return roots, codes, work, yf

    def residuals(self, roots, q):
        """Row-scaled residual of the target system at dehomogenized roots (Z0 = 1):
        per root, max over rows of |F_r| / max_c max(|Re J_rc|, |Im J_rc|)."""
        roots = _c(roots).reshape(-1, 21)
        out = np.zeros(len(roots))
        for i, r in enumerate(roots):
            Z = np.concatenate([r, [1.0]])
            f = np.abs(self.fsys(Z, q))
            J = self.jvar(Z, q)
            m = np.maximum(np.abs(J.real), np.abs(J.imag)).max(axis=1)
            ratio = f / m
            out[i] = np.inf if np.any(np.isnan(ratio)) else np.max(ratio)
        return out

    def sort_merge(self, coll, fpt, codes, tol=1e-6):
        coll = _c(coll).reshape(-1, 21)
        fpt = _c(fpt).reshape(-1, 21)
        codes = np.ascontiguousarray(np.asarray(codes, dtype=np.int32)).copy()
        out = np.zeros((len(coll) + len(fpt), 21), np.complex128)
        m = self.lib.or_sort_merge(_p(coll), ctypes.c_int64(len(coll)), _p(fpt), codes.ctypes.data_as(_I),
                                   ctypes.c_int64(len(fpt)), ctypes.c_double(tol), _p(out))
        return out[:m], codes

    # ---- plug-in systems (frg_plugins_gen.h; system ids 1..) ----
    def plugin_info(self, system):
        """(nv, np) of plug-in `system`; raises KeyError for an unknown id."""
        nv, np_ = ctypes.c_int(), ctypes.c_int()
        if not self.lib.or_plugin_info(int(system), ctypes.byref(nv), ctypes.byref(np_)):
            raise KeyError(system)
        return nv.value, np_.value

    def plugin_rows(self, system, Y, q, dq):
        """(M [nv, nv + 2], F [nv]): rows of the homotopy Jacobian and F at Y = [Z, Z0, t]."""
        nv, _ = self.plugin_info(system)
        M = np.zeros((nv, nv + 2), np.complex128)
        F = np.zeros(nv, np.complex128)
        self.lib.or_plugin_rows(int(system), _p(_c(Y)), _p(_c(q)), _p(_c(dq)), _p(M), _p(F))
        return M, F

    def plugin_start(self, system, seed, stream, cfg: OrConfig | None = None):
        cfg = cfg or self.config()
        nv, np_ = self.plugin_info(system)
        spt = np.zeros(nv, np.complex128)
        spm = np.zeros(np_, np.complex128)
        self.lib.or_plugin_start(int(system), ctypes.byref(cfg), ctypes.c_uint64(seed), ctypes.c_uint64(stream),
                                 _p(spt), _p(spm))
        return spt, spm

    def plugin_batch(self, system, fpm, gammas, seed, paths_per_task, cfg: OrConfig | None = None, nthreads=None,
                     want_yfinal=False, path_offset=0):
        """Track sum(paths_per_task) paths of plug-in `system`: path i uses random stream
        path_offset + i and belongs to task k (fpm [ntasks, np], gammas [ntasks]);
        returns (roots [n, nv], codes [n], resid [n], yfinal [n, nv + 2] or None)."""
        cfg = cfg or self.config()
        nv, np_ = self.plugin_info(system)
        fpm = _c(fpm).reshape(-1, np_)
        ppt = np.atleast_1d(np.asarray(paths_per_task, np.int64))
        starts = np.ascontiguousarray(np.concatenate([[0], np.cumsum(ppt)]).astype(np.int64))
        n = int(starts[-1])
        streams = np.ascontiguousarray(np.arange(n, dtype=np.uint64) + np.uint64(path_offset))
        roots = np.zeros((n, nv), np.complex128)
        codes = np.zeros(n, np.int32)
        resid = np.zeros(n)
        yf = np.zeros((n, nv + 2), np.complex128) if want_yfinal else None
        nthreads = nthreads or os.cpu_count() or 1
        self.lib.or_plugin_batch(int(system), ctypes.byref(cfg), ctypes.c_uint64(seed), streams.ctypes.data_as(_U64),
                                 ctypes.c_int64(n), ctypes.c_int(len(ppt)), starts.ctypes.data_as(_I64), _p(fpm),
                                 _p(_c(gammas)), _p(roots), codes.ctypes.data_as(_I),
                                 _p(yf) if yf is not None else None, _p(resid), ctypes.c_int(nthreads))
        return roots, codes, resid, yf

    def lambertw0(self, z):
        return self.lib.or_lambertw0(float(z))

    def philox_block(self, ctr, key):
        c = (ctypes.c_uint32 * 4)(*ctr)
        k = (ctypes.c_uint32 * 2)(*key)
        o = (ctypes.c_uint32 * 4)()
        self.lib.or_philox_block(c, k, o)
        return tuple(o)

    def uniform01(self, seed, stream, index):
        f = self.lib.or_uniform01
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        return f(seed, stream, index)


class RefLib:
    """The reference's own sources built for the host (oracle/_ref/libfrgref.so)."""

    def __init__(self, path: str = REF_SO):
        self.lib = ctypes.CDLL(path)
        self.lib.ref_lambertw.restype = ctypes.c_double
        self.lib.ref_lambertw.argtypes = [ctypes.c_double]
        self.lib.ref_sort_merge.restype = ctypes.c_longlong

    def call(self, name, *args):
        return getattr(self.lib, "ref_" + name)(*args)

    fsys = Oracle.fsys
    jvar = Oracle.jvar
    jpar = Oracle.jpar
    q = Oracle.q
    dqdt = Oracle.dqdt
    h = Oracle.h
    jh = Oracle.jh
    switch_patch = Oracle.switch_patch
    ivp = Oracle.ivp
    dp65 = Oracle.dp65
    newton = Oracle.newton
    cognate = Oracle.cognate

    @property
    def prefix(self):
        return "ref_"

    def _fn(self, name):
        return getattr(self.lib, "ref_" + name)

    def generate_start(self, seed, stream):
        spt = np.zeros(21, np.complex128)
        spm = np.zeros(30, np.complex128)
        self.lib.ref_generate_start(ctypes.c_ulonglong(seed), ctypes.c_ulonglong(stream), _p(spt), _p(spm))
        return spt, spm

    def track_path(self, spt, spm, fpm, gamma, seed, stream):
        Y = np.zeros(23, np.complex128)
        code = ctypes.c_int()
        self.lib.ref_track_path(_p(_c(spt)), _p(_c(spm)), _p(_c(fpm)), _p(_c([gamma])),
                                ctypes.c_ulonglong(seed), ctypes.c_ulonglong(stream), _p(Y),
                                ctypes.byref(code))
        return Y, code.value

    def homotopy_path(self, seed, stream, fpm, gamma):
        root = np.zeros(21, np.complex128)
        Y = np.zeros(23, np.complex128)
        code = ctypes.c_int()
        self.lib.ref_homotopy_path(ctypes.c_ulonglong(seed), ctypes.c_ulonglong(stream), _p(_c(fpm)),
                                   _p(_c([gamma])), _p(root), ctypes.byref(code), _p(Y))
        return root, code.value, Y

    def homotopy_batch(self, fpm, gamma, seed, stream0, n, nthreads=None):
        roots = np.zeros((n, 21), np.complex128)
        codes = np.zeros(n, np.int32)
        self.lib.ref_homotopy_batch(ctypes.c_ulonglong(seed), ctypes.c_ulonglong(stream0),
                                    ctypes.c_longlong(n), _p(_c(fpm)), _p(_c([gamma])), _p(roots),
                                    codes.ctypes.data_as(_I), ctypes.c_int(nthreads or os.cpu_count() or 1))
        return roots, codes

    def homotopy_batch_ex(self, fpm, gamma, seed, stream0, n, start_normal=False, nthreads=None,
                          want_yfinal=True):
        """ref_homotopy_batch_ex: roots, codes, Yfinal (or None) and residuals of paths
        stream0 .. stream0 + n - 1, start mechanisms U(-5,5)^2 or complex normal."""
        roots = np.zeros((n, 21), np.complex128)
        codes = np.zeros(n, np.int32)
        yf = np.zeros((n, 23), np.complex128) if want_yfinal else None
        resid = np.zeros(n, np.float64)
        self.lib.ref_homotopy_batch_ex(ctypes.c_ulonglong(seed), ctypes.c_ulonglong(stream0), ctypes.c_longlong(n),
                                       _p(_c(fpm)), _p(_c([gamma])), ctypes.c_int(1 if start_normal else 0),
                                       _p(roots), codes.ctypes.data_as(_I), _p(yf) if yf is not None else None,
                                       _p(resid), ctypes.c_int(nthreads or os.cpu_count() or 1))
        return roots, codes, yf, resid

    def residuals(self, roots, q):
        """Row-scaled residual at dehomogenized roots with the reference's FSYS and JVAR."""
        roots = _c(roots).reshape(-1, 21)
        out = np.zeros(len(roots))
        self.lib.ref_residuals(_p(roots), ctypes.c_longlong(len(roots)), _p(_c(q)), _p(out))
        return out

    def uniform01(self, seed, stream, index):
        f = self.lib.ref_uniform01
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_ulonglong]
        return f(seed, stream, index)

    def sort_merge(self, coll, fpt, codes, order):
        coll = _c(coll).reshape(-1, 21)
        fpt = _c(fpt).reshape(-1, 21)
        codes = np.ascontiguousarray(np.asarray(codes, dtype=np.int32)).copy()
        order = np.ascontiguousarray(np.concatenate([np.asarray(order, np.int32), [0]]).astype(np.int32))
        out = np.zeros((len(coll) + len(fpt), 21), np.complex128)
        m = self.lib.ref_sort_merge(_p(coll), ctypes.c_longlong(len(coll)), _p(fpt),
                                    codes.ctypes.data_as(_I), order.ctypes.data_as(_I), ctypes.c_int(len(fpt)),
                                    _p(out))
        return out[:m], codes

    def lambertw(self, z):
        return self.lib.ref_lambertw(float(z))


def cognate34_linkage(x, P0):
    """The 3/4 cognate of one half of a Stephenson II linkage (A, B, C, D, F, G, H; seven
    complex values) with precision point P0: two similarity maps that keep B and F
    (frgkinematics.cu:140-182, Dijksman's construction; dead code in the reference, its
    calls commented out at :262-266)."""
    A, B, C, D, F, G, H = x
    s = (H - G) / (C - G)
    Ap, Bp, Cp, Gp = s * (A - D) + D, s * (B - D) + D, s * (C - D) + D, D + (H - G)
    s2 = (B - F) / (Bp - F)
    return np.array([s2 * (Ap - F) + F, B, s2 * (Cp - F) + F, s2 * (D - F) + F, F, s2 * (Gp - F) + F,
                     s2 * (H - F) + F])


def cognate12_root(z, q):
    """The 1/2 cognate of a dehomogenized root z (21 complex) of task q: Cognate12 on both
    halves and the rotations U_down (frgkinematics.cu:185-256)."""
    z = np.asarray(z, np.complex128)
    B, F = z[1], z[4]
    P, Pc = q[0:8], q[8:16]
    out = z.copy()
    out[14:21] = ((P[1:8] - B) - z[14:21] * (P[0] - F)) / (F - B)

    def c12(x, p0):
        A, B, C, D, F, G, H = x
        s = (B - F) / (D - F)
        Dp, Gp = s * (D - H) + H, s * (G - H) + H
        s2 = (p0 - F) / (H - F)
        return np.array([s2 * (A - B) + B, B, s2 * (C - B) + B, s2 * (Dp - B) + B, B + (p0 - F), s2 * (Gp - B) + B,
                         s2 * (H - B) + B])

    out[0:7] = c12(z[0:7], P[0])
    out[7:14] = c12(z[7:14], Pc[0])
    return out


# The reference's hard-coded target (frg.cu:149-178) and gamma (frg.cu:41).
T_REF = np.array([
    4.241713408139979 - 4.925334736425448j, 1.448005491494222 - 2.686249989236069j,
    2.287911194543938 - 0.9123108488455074j, -1.870502483790705 - 0.5778077414588303j,
    -0.7625329418400497 + 0.9043788195368165j, -4.142822753796651 + 1.697671322829592j,
    1.023004534182935 - 3.026210035710708j, -2.522295755933046 + 3.942421532145637j,
    -3.769870484797034 + 0.7972377857916531j, -4.285631161563732 - 0.5650246890525263j,
    -2.166030800874488 + 0.8836055774820508j, 4.579260949000442 - 2.074013737196861j,
    4.801289733755713 - 1.460721841824302j, 2.041266673362720 + 2.962149232597863j,
    3.989999692714399 - 0.2328295911150420j, -3.996448356004510 + 4.426854856711802j,
    2.315936719955769 - 0.5527803857724418j, -3.018911857947673 + 0.9692384144638879j,
    -0.4906347357049512 + 2.994316903874402j, 0.2397118512793472 - 1.341440197750693j,
    4.942917423339324 - 2.415216683074435j, 1.599536873563615 + 2.367319121024760j,
    4.229853181495468 - 1.149104287738972j, -0.2180298061101595 + 3.585004213517870j,
    4.311063203842579 - 0.03375595047392820j, 4.938148066901551 + 4.551701974206413j,
    -4.271214442569748 + 0.1355349863802999j, -0.7377434797048270 + 1.831738837919296j,
    0.8894614668331116 + 0.8657473695398501j, 4.036757863569754 + 1.461164684969592j,
], dtype=np.complex128)
GAMMA_REF = 0.39231132891081666 + 1.0062265257923928j
