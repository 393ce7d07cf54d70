"""The oracle's Gurvits estimator (CPU): each draw is the Glynn term of its sign vector,
the mean over all 2^n sign vectors is the permanent exactly, and the estimate stays
within the Hoeffding 99% bound B sqrt(4 ln 400 / N), B = ||A||_2^n, of the exact value."""
import math

import numpy as np
import pytest

from perceval_gb300.utils.matrix import random_unitary


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7])
def test_mean_over_all_signs_is_the_permanent(oracle, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    total = sum(oracle.glynn_term(a, b) for b in range(2 ** n))
    ref = oracle.perm_brute(a)
    assert abs(total / 2 ** n - ref) <= 1e-12 * max(1.0, abs(ref))


def test_draws_bounded_by_spectral_norm(oracle):
    U = random_unitary(30, seed=2)
    a = U[:8, 3:11] * 3.0
    B = np.linalg.norm(a, 2) ** 8
    rng = np.random.default_rng(0)
    for b in rng.integers(0, 2 ** 8, 200):
        assert abs(oracle.glynn_term(a, int(b))) <= B * (1 + 1e-12)


def test_estimates_within_bound(oracle):
    U = random_unitary(64, seed=1)
    rng = np.random.default_rng(3)
    N = 4000
    outside = 0
    for t in range(40):
        n = int(rng.integers(3, 9))
        a = U[np.ix_(rng.choice(64, n, False), rng.choice(64, n, False))]
        est = oracle.gurvits(a, N, seed=11, first=t * N)
        err = np.linalg.norm(a, 2) ** n * math.sqrt(4 * math.log(400) / N)
        outside += abs(est - oracle.perm(a)) > err
    assert outside <= 1
