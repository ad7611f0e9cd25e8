"""Record golden vectors from the reference tracker's own sources.

Builds ``oracle/_ref/libfrgref.so`` from the reference sources (``oracle/Makefile``:
the environment variable REF names the reference checkout; ``make stage`` copies its
sources into the git-ignored ``oracle/_ref/src``, never into tracked files) and
records, on seeded inputs:

* FSYS / JVAR / JPAR        (htpykinematics.cu:8, :129, :1132)
* q(t), dq/dt, H, JH        (htpysupport.cu:37, :51, :64, :89)
* SwitchPatch, IVP          (htpysupport.cu:9, :237)
* one DormandPrince65 step  (rungekutta.cu:3)
* Newton corrector/sharpen  (htpysupport.cu:407)
* GenerateStart             (frgkinematics.cu:13), Philox streams of frg_rng.h
* full kernel-body paths    (frg.cu:41-68) on the reference target (frg.cu:149-178)
* CognateSolns              (frgkinematics.cu:227)
* SortingDeletingMerging    (frgsupport.cu:10) on synthetic collections
* LambertW                  (frgsupport.cu:249)

into ``tests/golden/ref_golden.npz``. Run from the repository root:
``REF=<reference checkout> python tests/golden/make_golden.py``.
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import GAMMA_REF, T_REF, RefLib  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "ref_golden.npz")
SEED = 1234
N_PATHS = 96


def crand(rng, n, r=2.0):
    return rng.uniform(-r, r, n) + 1j * rng.uniform(-r, r, n)


def main() -> None:
    ref_dir = os.environ.get("REF")
    if not ref_dir:
        raise SystemExit("set REF to the reference checkout")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "stage", f"REF={ref_dir}"], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    ref = RefLib()
    rng = np.random.default_rng(20261203)
    g: dict[str, np.ndarray] = {}

    # --- system and Jacobians on random points -----------------------------
    Zs = np.stack([crand(rng, 22) for _ in range(6)])
    qs = np.stack([crand(rng, 30) for _ in range(6)])
    g["sys_Z"], g["sys_q"] = Zs, qs
    g["fsys"] = np.stack([ref.fsys(Z, q) for Z, q in zip(Zs, qs)])
    g["jvar"] = np.stack([ref.jvar(Z, q) for Z, q in zip(Zs, qs)])
    g["jpar"] = np.stack([ref.jpar(Z, q) for Z, q in zip(Zs, qs)])

    # --- homotopy pieces at states taken from real starts -------------------
    starts = [ref.generate_start(SEED, s) for s in range(4)]
    Ys, us, Vs, spms, ts = [], [], [], [], []
    for k, (spt, spm) in enumerate(starts):
        t = [0.0, 0.37, 0.91, 0.999995][k]
        Y = np.concatenate([spt + 0.01 * crand(rng, 21), [1.0 + 0.0j, t]])
        Ys.append(Y); us.append(crand(rng, 23)); Vs.append(crand(rng, 23)); spms.append(spm); ts.append(t)
    Ys, us, Vs, spms = map(np.stack, (Ys, us, Vs, spms))
    g["hs_Y"], g["hs_u"], g["hs_V"], g["hs_spm"] = Ys, us, Vs, spms
    g["hs_t"] = np.array(ts)
    g["hs_q"] = np.stack([ref.q(t, spm, T_REF, GAMMA_REF) for t, spm in zip(ts, spms)])
    g["hs_dqdt"] = np.stack([ref.dqdt(t, spm, T_REF, GAMMA_REF) for t, spm in zip(ts, spms)])
    g["hs_h"] = np.stack([ref.h(Y, u, spm, T_REF, GAMMA_REF) for Y, u, spm in zip(Ys, us, spms)])
    g["hs_jh"] = np.stack([ref.jh(Y, u, spm, T_REF, GAMMA_REF) for Y, u, spm in zip(Ys, us, spms)])
    g["hs_switch"] = np.stack([ref.switch_patch(u, Y) for Y, u in zip(Ys, us)])
    g["hs_ivp0"] = np.stack([ref.ivp(0, Y, V, u, spm, T_REF, GAMMA_REF) for Y, V, u, spm in zip(Ys, Vs, us, spms)])
    g["hs_ivp1"] = np.stack([ref.ivp(1, Y, V, u, spm, T_REF, GAMMA_REF) for Y, V, u, spm in zip(Ys, Vs, us, spms)])

    # --- one DP6(5) step and Newton from exact starts -----------------------
    dp_Y, dp_V, dp_u, dp_spm, dp_out = [], [], [], [], []
    nw_Y0, nw_out, nw_res, nw_sh, nw_shres = [], [], [], [], []
    for k, (spt, spm) in enumerate(starts):
        u = crand(rng, 23)
        Y0 = ref.switch_patch(u, np.concatenate([spt, [1.0, 0.0]]))
        V0 = ref.ivp(0, Y0, crand(rng, 23), u, spm, T_REF, GAMMA_REF)
        s = [0.05, 0.2, 0.01, 0.5][k]
        Yn, Vn, err, sc = ref.dp65(s, 1e-3, 0, Y0, V0, u, spm, T_REF, GAMMA_REF)
        dp_Y.append(Y0); dp_V.append(V0); dp_u.append(u); dp_spm.append(spm)
        dp_out.append(np.concatenate([Yn, Vn, [err, sc, s]]))
        YN, res = ref.newton(Yn[22].real, Vn, u, spm, T_REF, GAMMA_REF, 10, 1e-8, 1, Yn)
        nw_Y0.append(Yn); nw_out.append(YN); nw_res.append(res)
        # sharpening-style Newton at t = t0 from a perturbed exact start
        Yp = Y0 + 1e-4 * crand(rng, 23); Yp[22] = 0.0
        YS, rs = ref.newton(0.0, V0, u, spm, T_REF, GAMMA_REF, 30, 1e-12, 1, Yp)
        nw_sh.append(np.concatenate([Yp, YS])); nw_shres.append(rs)
    g["dp_Y"], g["dp_V"], g["dp_u"], g["dp_spm"] = map(np.stack, (dp_Y, dp_V, dp_u, dp_spm))
    g["dp_out"] = np.stack(dp_out)
    g["nw_Y0"], g["nw_out"], g["nw_res"] = np.stack(nw_Y0), np.stack(nw_out), np.array(nw_res)
    g["nw_sh"], g["nw_shres"] = np.stack(nw_sh), np.array(nw_shres)

    # --- start generation ---------------------------------------------------
    st = [ref.generate_start(SEED, s) for s in range(16)]
    g["gs_spt"] = np.stack([a for a, _ in st])
    g["gs_spm"] = np.stack([b for _, b in st])

    # --- full paths on the reference target --------------------------------
    roots, codes, yfin = [], [], []
    for s in range(N_PATHS):
        r, c, Y = ref.homotopy_path(SEED, s, T_REF, GAMMA_REF)
        roots.append(r); codes.append(c); yfin.append(Y)
    g["path_seed"] = np.array([SEED], np.uint64)
    g["path_roots"], g["path_codes"], g["path_yfinal"] = np.stack(roots), np.array(codes, np.int32), np.stack(yfin)

    # --- cognates -------------------------------------------------------------
    ok = [i for i, c in enumerate(codes) if c == 0][:6]
    g["cog_in"] = np.stack([roots[i] for i in ok])
    g["cog_out"] = np.stack([ref.cognate(roots[i], T_REF) for i in ok])

    # --- dedup / merge --------------------------------------------------------
    base = crand(rng, 21 * 40).reshape(40, 21)
    coll = base[np.argsort(base[:, 0].real, kind="stable")][:25]
    new = [coll[3], coll[3] + 0.5e-6, coll[10] + 2e-6, base[30], base[30] + 0.4e-6 * (1 + 1j),
           base[31], base[32], coll[20], base[33], base[33]]
    new = np.stack(new)
    ncodes = np.array([0, 0, 0, 0, 0, 3, 0, 6, 0, 0], np.int32)
    order = np.argsort(new[:, 0].real, kind="stable").astype(np.int32)
    merged, mcodes = ref.sort_merge(coll, new, ncodes, order)
    g["dd_coll"], g["dd_new"], g["dd_codes_in"] = coll, new, ncodes
    g["dd_merged"], g["dd_codes_out"] = merged, mcodes
    # a second round on an empty collection
    m2, c2 = ref.sort_merge(np.zeros((0, 21), np.complex128), new, ncodes, order)
    g["dd_merged_empty"], g["dd_codes_empty"] = m2, c2

    # --- Lambert W -------------------------------------------------------------
    zs = np.array([-0.36, -0.3, -0.2, -0.05, 0.1, 0.5, 1.0, 2.0, 10.0])
    g["lw_z"] = zs
    g["lw_w"] = np.array([ref.lambertw(z) for z in zs])

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes;", "path codes", np.bincount(g["path_codes"]))


if __name__ == "__main__":
    main()
