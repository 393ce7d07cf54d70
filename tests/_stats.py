"""Chi-square goodness of fit of sample counts against exact probabilities."""
import numpy as np
from scipy.stats import chisquare


def chi2_pvalue(counts: np.ndarray, probs: np.ndarray, min_expected: float = 5.0) -> float:
    counts = np.asarray(counts, dtype=np.float64)
    N = counts.sum()
    exp = np.asarray(probs, dtype=np.float64) * N
    keep = exp >= min_expected
    obs_k, exp_k = counts[keep], exp[keep]
    if (~keep).any() and exp[~keep].sum() > 0:
        obs_k = np.append(obs_k, counts[~keep].sum())
        exp_k = np.append(exp_k, exp[~keep].sum())
    exp_k = exp_k * (obs_k.sum() / exp_k.sum())
    return float(chisquare(obs_k, exp_k).pvalue)
