"""Exact one- and two-mode marginal distributions (generating-function permanents)
against brute-force sums over every output probability of the CPU oracle, at n <= 6."""
import numpy as np
import pytest

from perceval_gb300.marginals import one_mode_marginal, two_mode_marginal
from perceval_gb300.utils.matrix import random_unitary
from perceval_gb300.utils.states import fock_space_array


@pytest.mark.parametrize("m,n,seed", [(4, 2, 1), (6, 4, 2), (8, 6, 3), (9, 5, 4)])
def test_marginals_equal_brute_force(oracle, m, n, seed):
    U = random_unitary(m, seed=seed)
    rng = np.random.default_rng(seed)
    inp = np.zeros(m, dtype=int)
    inp[rng.choice(m, n, replace=False)] = 1
    p, _ = oracle.slos(U, list(inp))
    states = fock_space_array(m, n)
    assert abs(p.sum() - 1) < 1e-12
    for i in range(m):
        ref = np.bincount(states[:, i], weights=p, minlength=n + 1)
        got = one_mode_marginal(U, inp, i)
        assert np.abs(got - ref).max() < 1e-12, (i, got, ref)
    for i, j in [(0, 1), (m - 1, 0), (1, m - 2)]:
        ref = np.zeros((n + 1, n + 1))
        np.add.at(ref, (states[:, i], states[:, j]), p)
        got = two_mode_marginal(U, inp, i, j)
        assert np.abs(got - ref).max() < 1e-12, (i, j)
        assert np.abs(got.sum(axis=1) - one_mode_marginal(U, inp, i)).max() < 1e-12


def test_exact_rational_path_agrees():
    U = random_unitary(7, seed=9)
    inp = [1, 1, 1, 0, 1, 0, 0]
    for i in (0, 3, 6):
        assert np.abs(one_mode_marginal(U, inp, i, exact=True) - one_mode_marginal(U, inp, i)).max() < 1e-13
    a = two_mode_marginal(U, inp, 1, 5, exact=True)
    b = two_mode_marginal(U, inp, 1, 5)
    assert np.abs(a - b).max() < 1e-13


def test_large_instance_is_a_distribution():
    """n = 30 photons on m = 900 modes (the learned-sampler configuration): the marginals
    are non-negative distributions whose first moments match the closed form E[n_i]."""
    from perceval_gb300.learned import exact_moments
    U = random_unitary(900, seed=0)
    inp = [1] * 30 + [0] * 870
    A, E2 = exact_moments(U, inp)
    for i in (0, 29, 450, 899):
        p = one_mode_marginal(U, inp, i)
        assert p.min() > -1e-15 and abs(p.sum() - 1) < 1e-12
        assert abs(p @ np.arange(31) - A[i]) < 1e-12
    P2 = two_mode_marginal(U, inp, 3, 700)
    assert P2.min() > -1e-15 and abs(P2.sum() - 1) < 1e-12
    k = np.arange(31)
    assert abs(k @ P2 @ k - E2[3, 700]) < 1e-12
