"""Statistical checks shared by the sampling tests (test infrastructure)."""

import numpy as np


def chi2_pvalue(counts, probs, shots, min_expected=5.0):
    """Pearson chi-squared p-value of observed counts against exact
    probabilities.  Bins with fewer than `min_expected` expected counts are
    merged, in order of increasing probability, until each merged bin expects
    at least that many."""
    from scipy import stats
    exp = np.asarray(probs, np.float64) * shots
    counts = np.asarray(counts)
    order = np.argsort(exp)
    ce, cc, acc_e, acc_c = [], [], 0.0, 0
    for k in order:
        acc_e += exp[k]
        acc_c += counts[k]
        if acc_e >= min_expected:
            ce.append(acc_e)
            cc.append(acc_c)
            acc_e, acc_c = 0.0, 0
    if acc_e > 0 and ce:
        ce[-1] += acc_e
        cc[-1] += acc_c
    ce, cc = np.array(ce), np.array(cc)
    chi2 = float(np.sum((cc - ce) ** 2 / ce))
    return float(stats.chi2.sf(chi2, max(len(ce) - 1, 1))), chi2, len(ce)


def bits_to_index(bits, n):
    """Samples-op rows (column col = qubit col of the last n columns,
    big-endian) to state indices."""
    bits = np.asarray(bits, np.int64)[:, -n:] if n else np.zeros((len(bits), 0), np.int64)
    idx = np.zeros(len(bits), dtype=np.int64)
    for col in range(n):
        idx = (idx << 1) | bits[:, col]
    return idx
