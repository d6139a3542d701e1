"""Comparing Monte-Carlo tallies (N, sum p, sum p^2)."""

import numpy as np


def chi2_per_dof(t1, t2, min_count=10, n1=None, n2=None):
    """Chi^2/dof between two tallies (3, ...) from independent runs.

    Each run's bin estimate is sum p / n_run with variance sum p^2 / n_run^2
    (n_run = neutrons the run started; equal counts when omitted).  Bins
    with fewer than `min_count` entries in either run are left out.
    Returns (chi2/dof, dof)."""
    t1 = np.asarray(t1).reshape(3, -1)
    t2 = np.asarray(t2).reshape(3, -1)
    a1 = 1.0 / n1 if n1 else 1.0
    a2 = 1.0 / n2 if n2 else 1.0
    m = (t1[0] >= min_count) & (t2[0] >= min_count)
    if not m.any():
        return float("nan"), 0
    d = t1[1][m] * a1 - t2[1][m] * a2
    v = t1[2][m] * a1 * a1 + t2[2][m] * a2 * a2
    return float(np.sum(d * d / v) / m.sum()), int(m.sum())


def z_scores(t1, t2, min_count=10, n1=None, n2=None):
    """Per-bin z = (mean1 - mean2) / sqrt(var1 + var2) over the bins that
    chi2_per_dof uses (same estimates and variances)."""
    t1 = np.asarray(t1).reshape(3, -1)
    t2 = np.asarray(t2).reshape(3, -1)
    a1 = 1.0 / n1 if n1 else 1.0
    a2 = 1.0 / n2 if n2 else 1.0
    m = (t1[0] >= min_count) & (t2[0] >= min_count)
    d = t1[1][m] * a1 - t2[1][m] * a2
    v = t1[2][m] * a1 * a1 + t2[2][m] * a2 * a2
    return d / np.sqrt(v)


def z_summary(t1, t2, **kw):
    """max |z|, the fraction of bins with |z| > 3 (0.27% expected for
    normal z) and the mean and standard deviation of z (0 and 1 expected)."""
    z = z_scores(t1, t2, **kw)
    if z.size == 0:
        return {"bins": 0}
    return {"bins": int(z.size), "max_abs_z": float(np.abs(z).max()),
            "frac_abs_z_gt_3": float((np.abs(z) > 3).mean()),
            "mean_z": float(z.mean()), "std_z": float(z.std())}
