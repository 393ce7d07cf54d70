"""Naive strong simulation with Gurvits estimates of the permanents
(perceval/backends/_naive_approx.py:36-69).

Same submatrices and normalisation as ``NaiveBackend``; the permanent is the mean of
``gurvits_iterations`` randomised Glynn draws (``pcvl_permanent_estimate_batch``), with
a 99% error bound.  The draws take their Philox counters from the process-wide stream
of ``perceval_gb300.utils.random_seed``, so a fixed seed reproduces every estimate.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .. import _native
from ..utils import _random
from ..utils.states import FockState
from ._naive import NaiveBackend


class NaiveApproxBackend(NaiveBackend):
    """Naive algorithm with Gurvits computations of permanents.

    :param gurvits_iterations: number of draws per permanent (default 10 000)
    """

    def __init__(self, gurvits_iterations: int = 10000):
        super().__init__()
        if int(gurvits_iterations) < 1:
            raise ValueError("gurvits_iterations must be >= 1")
        self._gurvits_iterations = int(gurvits_iterations)

    @property
    def name(self) -> str:
        return "NaiveApprox"

    def _estimates(self, flat: np.ndarray, offs: np.ndarray, sizes: np.ndarray):
        dev = torch.from_numpy(flat).to("cuda")
        out = torch.empty(len(sizes), dtype=torch.complex128, device="cuda")
        err = torch.empty(len(sizes), dtype=torch.float64, device="cuda")
        seed, first = _random.take_samples(len(sizes) * self._gurvits_iterations)
        _native.permanent_estimate_batch(dev, offs, sizes, out, err, self._gurvits_iterations, seed, first)
        return out.cpu().numpy(), err.cpu().numpy()

    def _permanents(self, flat, offs, sizes) -> np.ndarray:
        return self._estimates(flat, offs, sizes)[0]

    def prob_amplitude_with_error(self, output_state) -> tuple[complex, float]:
        """Estimated probability amplitude and its 99% error bound (_naive_approx.py:52-59)."""
        output_state = FockState(output_state)
        M = self._compute_submatrix(output_state)
        if M.size <= 1:
            return complex(M[0, 0]), 0.0
        est, err = self._estimates(np.ascontiguousarray(M).reshape(-1), np.array([0]), np.array([M.shape[0]]))
        norm = math.sqrt(output_state.prodnfact() * self._input_state.prodnfact())
        return complex(est[0]) / norm, float(err[0]) / norm

    def probability_confidence_interval(self, output_state) -> list[float]:
        """99% confidence interval of the probability, with the reference's formula
        [max((|a| - e)^2, 0), min((|a| + e)^2, 1)] (_naive_approx.py:61-66)."""
        mean, err = self.prob_amplitude_with_error(output_state)
        min_prob = max((abs(mean) - err) ** 2, 0)
        max_prob = min((abs(mean) + err) ** 2, 1)
        return [min_prob, max_prob]
