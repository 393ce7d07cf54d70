"""GPU Clifford & Clifford sampler: sample-by-sample agreement with the CPU oracle
(same Philox stream and draw procedure) and chi-square agreement with the exact
SLOS distribution (p > 0.01)."""
import numpy as np
import pytest
import torch

from _stats import chi2_pvalue
from perceval_gb300.utils import fock_rank
from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,inp,precision", [
    (5, (1, 1, 1, 0, 0), 0), (6, (2, 0, 1, 0, 1, 0), 0), (8, (1, 1, 1, 1, 1, 1, 0, 0), 0),
    (10, (1,) * 10, 0), (12, (2, 2, 0, 0, 1, 1, 1, 1, 0, 0, 0, 1), 0), (20, (1,) * 14 + (0,) * 6, 0),
    (6, (2, 0, 1, 0, 1, 0), 1), (8, (1, 1, 1, 1, 1, 1, 0, 0), 2), (20, (1,) * 14 + (0,) * 6, 2),
    (12, (2, 2, 0, 0, 1, 1, 1, 1, 0, 0, 0, 1), 2)])
def test_samples_equal_oracle(native, oracle, m, inp, precision):
    U = random_unitary(m, seed=m)
    N = 300
    got = native.cc2017_sample(torch.from_numpy(U).cuda(), inp, N, seed=42, first_sample=7,
                               precision=precision).cpu().numpy()
    ref = oracle.cc2017(U, inp, N, seed=42, first=7)
    assert got.shape == ref.shape
    agree = np.all(got == ref, axis=1).mean()
    # a different draw needs u within ~1e-13 (float-float, FP64) / ~1e-5 (FP32) of a CDF boundary
    assert agree >= (0.98 if precision == 1 else 1.0), agree
    assert np.all(got.sum(axis=1) == sum(inp))


@pytest.mark.parametrize("inp", [(1, 1, 1, 0, 0, 0), (2, 1, 0, 0, 0, 1)])
def test_chi_square_vs_exact(native, oracle, inp):
    m = len(inp)
    U = random_unitary(m, seed=21)
    probs, _ = oracle.slos(U, inp)
    N = 200000
    got = native.cc2017_sample(torch.from_numpy(U).cuda(), inp, N, seed=9).cpu().numpy()
    idx = np.array([fock_rank(r) for r in got])
    counts = np.bincount(idx, minlength=len(probs))
    assert chi2_pvalue(counts, probs) > 0.01


def test_reproducible_and_streams_disjoint(native):
    U = torch.from_numpy(random_unitary(16, seed=3)).cuda()
    inp = (1,) * 8 + (0,) * 8
    a = native.cc2017_sample(U, inp, 64, seed=5).cpu().numpy()
    b = native.cc2017_sample(U, inp, 64, seed=5).cpu().numpy()
    c = native.cc2017_sample(U, inp, 32, seed=5, first_sample=32).cpu().numpy()
    assert np.array_equal(a, b) and np.array_equal(a[32:], c)
    d = native.cc2017_sample(U, inp, 64, seed=6).cpu().numpy()
    assert not np.array_equal(a, d)


def test_larger_n_marginals(native):
    # n = 20 on m = 400 (the sampling workload's size): one-mode marginals match the
    # exact mean occupations E[n_i] = sum_j |U_ij|^2 over occupied inputs
    m, n = 400, 20
    U = random_unitary(m, seed=0)
    inp = (1,) * n + (0,) * (m - n)
    N = 4000
    got = native.cc2017_sample(torch.from_numpy(U).cuda(), inp, N, seed=1).cpu().numpy()
    assert np.all(got.sum(axis=1) == n)
    mean = got.mean(axis=0)
    exact = (np.abs(U[:, :n]) ** 2).sum(axis=1)
    z = (mean - exact) / np.sqrt(exact / N + 1e-12)
    assert np.abs(z).max() < 6
    assert abs(mean.sum() - n) < 1e-9


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_n26_marginals_and_precision_agreement(native, precision):
    # n = 26 on m = 676: Glynn sums of 2^24 column-sum products reach 1e21 with only a
    # global scaling of U, and their squares leave the FP32 range; the per-column and
    # per-step power-of-two normalisation keeps every weight finite.  One-mode marginals
    # must match E[n_i] = sum_k |U_ik|^2 (6 sigma, Var n_i <= A_i (1 + A_i)).
    m, n = 676, 26
    U = random_unitary(m, seed=26)
    inp = (1,) * n + (0,) * (m - n)
    N = 304
    Ud = torch.from_numpy(U).cuda()
    got = native.cc2017_sample(Ud, inp, N, seed=3, precision=precision).cpu().numpy()
    assert np.all(got.sum(axis=1) == n)
    A = (np.abs(U[:, :n]) ** 2).sum(axis=1)
    z = (got.mean(axis=0) - A) / np.sqrt(A * (1 + A) / N)
    assert np.abs(z).max() < 6, np.abs(z).max()
    if precision in (1, 2):
        # same Philox stream: FP32 and float-float pick the same rows unless a draw lands
        # within the FP32 error of a CDF boundary; FP64 (fixed-point column sums,
        # block-floating products) and float-float within ~1e-13 of one
        ref = native.cc2017_sample(Ud, inp, N, seed=3, precision=0).cpu().numpy()
        agree = np.all(got == ref, axis=1).mean()
        assert agree >= (0.8 if precision == 1 else 0.99), agree


def test_n29_fp64_agrees_with_float_float(native):
    """n = 29 photons (32 padded columns, the widest sub-permanent kernel) on m = 841: the
    FP64 mode draws the float-float mode's samples (same Philox stream)."""
    m, n = 841, 29
    U = torch.from_numpy(random_unitary(m, seed=29)).cuda()
    inp = (1,) * n + (0,) * (m - n)
    a = native.cc2017_sample(U, inp, 64, seed=4, precision=2).cpu().numpy()
    b = native.cc2017_sample(U, inp, 64, seed=4, precision=0).cpu().numpy()
    assert np.all(a.sum(axis=1) == n)
    assert np.all(a == b, axis=1).mean() >= 0.97


def test_many_input_states_in_one_wavefront(native):
    """pcvl_cc2017_sample_multi: the samples of several input states of one photon count
    (including a state with no samples) equal the single-state calls with the same Philox
    counters, row for row; the backend's samples_many keeps request order across photon
    counts."""
    from perceval_gb300.backends import Clifford2017Backend
    from perceval_gb300.utils import FockState, random_seed
    m = 9
    U = random_unitary(m, seed=21)
    Ud = torch.from_numpy(U).cuda()
    states = np.array([[1, 1, 0, 0, 1, 0, 0, 0, 0], [0, 2, 0, 0, 0, 0, 1, 0, 0], [0, 0, 0, 1, 1, 1, 0, 0, 0],
                       [3, 0, 0, 0, 0, 0, 0, 0, 0]])
    counts = [700, 0, 1300, 257]
    for precision in (0, 1):
        got = native.cc2017_sample_multi(Ud, states, counts, seed=5, first_sample=11,
                                         precision=precision).cpu().numpy()
        off = 11
        row = 0
        for st, c in zip(states, counts):
            ref = native.cc2017_sample(Ud, st, c, seed=5, first_sample=off, precision=precision).cpu().numpy()
            assert np.array_equal(got[row:row + c], ref)
            off += c
            row += c
    b = Clifford2017Backend()
    b.set_circuit(U)
    reqs = [FockState([1, 1, 0, 0, 0, 0, 0, 0, 0]), FockState([0, 0, 0, 0, 0, 0, 0, 0, 1]),
            FockState([0, 0, 1, 0, 0, 0, 0, 1, 0])]
    random_seed(9)
    many = b.samples_many(reqs, [40, 30, 20])
    random_seed(9)
    b.set_input_state(reqs[0])
    first = b.samples(40)
    assert [tuple(s) for s in many[0]] == [tuple(s) for s in first]
    assert len(many[1]) == 30 and all(s.n == 1 for s in many[1])
    assert len(many[2]) == 20 and all(s.n == 2 for s in many[2])
