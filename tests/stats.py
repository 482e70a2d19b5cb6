"""Statistical helpers for parity tests (3-standard-error rule of the combined estimate)."""
import math

import numpy as np


def z_threshold(k=1, p=0.0027, df=None):
    """Two-sided |z| threshold at family-wise level p over k comparisons (Bonferroni);
    k=1 gives 3.0 (the 3-sigma rule).  With `df`, the statistic's standard error is itself
    estimated from df+1 batch means, and the threshold is Student's t quantile with df degrees
    of freedom (the same level; the normal quantile would reject too often)."""
    if df is not None:
        from scipy.stats import t
        return float(t.isf(p / (2.0 * max(k, 1)), df))
    from scipy.stats import norm
    return float(norm.isf(p / (2.0 * max(k, 1))))


def binom_sigma(p, n):
    return math.sqrt(max(p * (1 - p), 1e-300) / n)


def zscores(a, sa, b, sb):
    a, sa, b, sb = map(lambda x: np.asarray(x, dtype=np.float64), (a, sa, b, sb))
    s = np.sqrt(sa ** 2 + sb ** 2)
    return np.where(s > 0, (a - b) / np.where(s > 0, s, 1), 0.0)


def batch_means(values):
    """mean and standard error of per-batch values (axis 0 = batch)."""
    v = np.asarray(values, dtype=np.float64)
    return v.mean(axis=0), v.std(axis=0, ddof=1) / math.sqrt(v.shape[0])
