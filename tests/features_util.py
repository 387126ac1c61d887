"""Comparison rule for matrix features (shared by the CPU and GPU tests).

Integer features (counts, minima, maxima) must be equal; floating features
(ratios, variances, P-ratio, Gini, log10 ranges) within 1e-9 relative --
the reference computes them in double (the fixtures come from its double
build) but sums in a different order."""
import numpy as np

INTEGER_FEATURES = [0, 1, 2, 7, 13, 19, 25, 31, 40, 41, 42, 43, 44, 45, 53, 54, 55]


def compare(got, want, rel=1e-9):
    bad = []
    for i, (g, w) in enumerate(zip(got, want)):
        if np.isnan(w) and np.isnan(g):
            continue
        if i in INTEGER_FEATURES:
            if g != w:
                bad.append((i, g, w))
        elif not (g == w or abs(g - w) <= rel * max(1.0, abs(w))):
            bad.append((i, g, w))
    return bad
