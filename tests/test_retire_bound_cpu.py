"""Upper bound on what early retirement can save on the benchmark's task distribution.

Perfect retirement (every path that will not yield a kept root, or whose root another
path of its round already found, ended at zero cost) saves at most the share of linear
solves those paths take. Measured here with the oracle's plain FP64 tracker on a sample
of the 128-task workload (task seeds 0, 8, ..., 120; complex-normal starts, the
benchmark's first seed and gamma): on 32 tasks x 256 paths it is 0.60 % of the solves for
paths without a kept root (0.31 % of the paths) and 0.08 % for duplicates within a
round, so no retirement policy can change the benchmark's throughput by more than
about 0.7 %; the bar below leaves room for sampling noise.
"""
import numpy as np

import bench


def test_retirement_cannot_save_more_than_a_few_percent(oracle):
    wl = bench.Workload("c5")
    cfg = oracle.config(start_dist=1)
    total = lost = dup = 0
    paths = not_kept = 0
    for kt in range(0, 128, 8):
        fpm = wl.tasks[kt]
        gamma = bench._gamma_of(oracle.uniform01, bench.SEED_BASE, 0)
        roots, codes, work, yf = oracle.homotopy_batch(fpm, gamma, bench.SEED_BASE, np.arange(128), cfg=cfg,
                                                       want_yfinal=True)
        resid = oracle.residuals(roots, fpm)
        zmax = np.max(np.abs(yf[:, :21]), axis=1)
        keep = (codes == 0) & (np.abs(yf[:, 21]) >= bench.INF_TOL * zmax) & (resid <= bench.RESID_MAX)
        _, marks = oracle.sort_merge(np.zeros((0, 21), np.complex128), roots,
                                     np.where(keep, 0, 5).astype(np.int32), bench.DUP_TOL)
        w = work[:, 0] + work[:, 1]
        total += w.sum()
        lost += w[~keep].sum()
        dup += w[marks == 6].sum()
        paths += len(w)
        not_kept += int((~keep).sum())
    share = (lost + dup) / total
    print(f"{paths} paths: {not_kept} without a kept root; retirement could save at most {share:.4f} of the solves")
    assert not_kept < 0.02 * paths
    assert share < 0.03
