"""GPU Gurvits estimator and the NaiveApprox backend.

* same draws as the oracle's estimator: |gpu - oracle| <= 1e-5 B (FP32 draws, FP64 sums);
* the bound: ||A||_2^n <= B_gpu <= (||A||_2 n^(1/8192))^n, err = B sqrt(4 ln 400 / N);
* coverage: the exact permanent lies within the 99% bound;
* n = 0 and n = 1 exact; NaiveApprox wiring and confidence intervals (reference
  tests/backends/test_backends.py:91-95 and docs/source/reference/backends/naive_approx.rst)."""
import math

import numpy as np
import pytest
import torch

from perceval_gb300.utils.matrix import random_unitary
from test_permanent_gpu import haar_submatrices, pack

pytestmark = pytest.mark.gpu


def gpu_estimates(native, mats, N, seed, first=0):
    flat, offs, sizes = pack(mats)
    dev = torch.from_numpy(flat).cuda()
    out = torch.empty(len(mats), dtype=torch.complex128, device="cuda")
    err = torch.empty(len(mats), dtype=torch.float64, device="cuda")
    native.permanent_estimate_batch(dev, offs, sizes, out, err, N, seed, first)
    return out.cpu().numpy(), err.cpu().numpy()


def test_same_draws_as_oracle(native, oracle):
    mats = haar_submatrices(12, 2, 12, seed=5, big=64)
    N = 20000
    est, err = gpu_estimates(native, mats, N, seed=123, first=77)
    for i, a in enumerate(mats):
        n = a.shape[0]
        ref = oracle.gurvits(a, N, seed=123, first=77 + i * N)
        B = np.linalg.norm(a, 2) ** n
        assert abs(est[i] - ref) <= 1e-5 * B + 1e-300, (n, abs(est[i] - ref), B)


def test_bound(native):
    mats = haar_submatrices(10, 2, 30, seed=6, big=128) + [3.0 * random_unitary(40, seed=1)[:40, :40] / 7]
    N = 1000
    est, err = gpu_estimates(native, mats, N, seed=1)
    for i, a in enumerate(mats):
        n = a.shape[0]
        s = np.linalg.norm(a, 2)
        B = err[i] / math.sqrt(4 * math.log(400) / N)
        assert s ** n * (1 - 1e-9) <= B <= (s * n ** (1 / 8192)) ** n * (1 + 1e-9)


def test_coverage(native, oracle):
    mats = haar_submatrices(200, 3, 10, seed=7, big=64)
    N = 2000
    est, err = gpu_estimates(native, mats, N, seed=9)
    exact = np.array([oracle.perm(a) for a in mats])
    assert np.mean(np.abs(est - exact) > err) <= 0.01


def test_trivial_sizes(native):
    a1 = np.array([[0.3 - 0.4j]])
    est, err = gpu_estimates(native, [np.zeros((0, 0), complex), a1], 10, seed=0)
    assert est[0] == 1 and err[0] == 0
    assert est[1] == a1[0, 0] and err[1] == 0


def test_converges(native, oracle):
    a = random_unitary(32, seed=3)[:6, 10:16]
    exact = oracle.perm(a)
    est, err = gpu_estimates(native, [a], 4_000_000, seed=4)
    assert abs(est[0] - exact) <= err[0] and err[0] < 0.01 * np.linalg.norm(a, 2) ** 6


def test_backend(native):
    from perceval_gb300 import BackendFactory, BasicState, Circuit, random_seed
    from perceval_gb300.components import BS
    b = BackendFactory.get_backend("NaiveApprox")
    assert b.name == "NaiveApprox"
    b.set_circuit(Circuit(1))  # identity, one mode
    b.set_input_state(BasicState([1]))
    assert b.probability(BasicState([1])) == pytest.approx(1.0)
    random_seed(5)
    b = BackendFactory.get_backend("NaiveApprox", gurvits_iterations=200000)
    b.set_circuit(BS.H())
    b.set_input_state(BasicState([1, 1]))
    exact = {(2, 0): 0.5, (1, 1): 0.0, (0, 2): 0.5}
    for out, p in exact.items():
        lo, hi = b.probability_confidence_interval(BasicState(list(out)))
        amp, e = b.prob_amplitude_with_error(BasicState(list(out)))
        assert abs(abs(amp) ** 2 - p) < 0.02
        assert e > 0
        assert lo <= p + 1e-12 or out == (1, 1)  # the reference's lower end is (|a| - e)^2
        assert hi >= p - 1e-12
    # a fixed seed reproduces the estimates
    random_seed(8)
    a1 = b.prob_amplitude(BasicState([2, 0]))
    random_seed(8)
    assert b.prob_amplitude(BasicState([2, 0])) == a1
