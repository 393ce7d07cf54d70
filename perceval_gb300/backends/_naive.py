"""Naive strong simulation: one permanent per output (perceval/backends/_naive.py:40-71).

``prob_amplitude`` builds the n x n submatrix exactly as ``_compute_submatrix``
(rows = output modes repeated by their counts, columns = input modes repeated,
_naive.py:51-68) and evaluates its permanent on the GPU, divided by
sqrt(prod out! * prod in!); the 1 x 1 case returns the element itself (:46-49).
``prob_amplitudes`` batches many outputs into one ``pcvl_permanent_batch`` call; the
full-space methods (``all_prob``, ``prob_distribution``, ``evolve``) use it.  The
permanents are computed in native FP64, the reference's arithmetic; ``precision=
"float-float"`` selects the faster FP32-pipe pairs (about 48 significant bits).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .. import _native
from ..utils.states import BSDistribution, FockState, StateVector
from ._abstract_backends import AStrongSimulationBackend


def _expand(state) -> np.ndarray:
    return np.repeat(np.arange(len(state)), np.asarray(state, dtype=np.int64))


class NaiveBackend(AStrongSimulationBackend):
    """Naive algorithm: no cached calculation path, every output recomputed."""

    def __init__(self, method: str = "glynn", precision: str = "fp64"):
        super().__init__()
        if method not in ("glynn", "ryser"):
            raise ValueError("method must be 'glynn' or 'ryser'")
        self._method = 0 if method == "glynn" else 1
        self._precision = _native.precision_code(precision)
        if self._precision not in (_native.PREC_FP64, _native.PREC_FLOAT_FLOAT):
            raise ValueError("precision must be 'fp64' or 'float-float'")

    @property
    def name(self) -> str:
        return "Naive"

    def _compute_submatrix(self, output_state) -> np.ndarray:
        n = self._input_state.n
        if n != output_state.n:
            return np.zeros((1, 1), dtype=complex)
        if n == 0:
            return np.ones((1, 1), dtype=complex)
        return self._umat[np.ix_(_expand(output_state), _expand(self._input_state))]

    def prob_amplitude(self, output_state) -> complex:
        return complex(self.prob_amplitudes([output_state])[0])

    def prob_amplitudes(self, output_states) -> np.ndarray:
        """Amplitudes of many outputs in one batched permanent launch.  The submatrices
        of all outputs are gathered at once: output s contributes the rows of its modes
        repeated by their counts (the same row selection as _compute_submatrix)."""
        outs = [FockState(s) for s in output_states]
        res = np.zeros(len(outs), dtype=np.complex128)
        if not outs:
            return res
        inp = self._input_state
        n, m = inp.n, inp.m
        counts = np.array([list(s) for s in outs], dtype=np.int64)
        assert counts.shape[1] == m, "output state size mismatch"
        nout = counts.sum(axis=1)
        ok = nout == n
        res[~ok] = 0.0
        if n == 0:
            res[ok] = 1.0
            return res
        idx = np.nonzero(ok)[0]
        if n == 1:  # 1 x 1 submatrix: the element itself (_naive.py:46-49)
            col = int(np.nonzero(np.asarray(list(inp)))[0][0])
            res[idx] = self._umat[np.argmax(counts[idx] > 0, axis=1), col]
            return res
        # row modes of every output (sorted, repeated by count) and the input's columns
        rows = np.repeat(np.tile(np.arange(m), len(idx)), counts[idx].reshape(-1)).reshape(len(idx), n)
        cols = _expand(inp)
        mats = np.ascontiguousarray(self._umat[rows[:, :, None], cols[None, None, :]])  # N x n x n
        lfact = np.array([math.lgamma(v + 1) for v in range(n + 1)])
        log_pout = lfact[counts[idx]].sum(axis=1)
        norms = np.exp(0.5 * (log_pout + math.log(inp.prodnfact())))
        offs = np.arange(len(idx), dtype=np.int64) * n * n
        perms = self._permanents(mats.reshape(-1), offs, np.full(len(idx), n, dtype=np.int32))
        res[idx] = perms / norms
        return res

    def _compute_permanent(self, M: np.ndarray) -> complex:
        """Permanent of one square matrix (_naive.py:70-71), through the batched call."""
        M = np.ascontiguousarray(M, dtype=np.complex128)
        n = M.shape[0]
        return complex(self._permanents(M.reshape(-1), np.zeros(1, dtype=np.int64), np.array([n], np.int32))[0])

    def _permanents(self, flat: np.ndarray, offs: np.ndarray, sizes: np.ndarray) -> np.ndarray:
        """Permanents of packed matrices, one batched launch (_naive.py:70-71)."""
        dev = torch.from_numpy(flat).to("cuda")
        out = torch.empty(len(sizes), dtype=torch.complex128, device="cuda")
        _native.permanent_batch(dev, offs, sizes, out, self._method, precision=self._precision)
        return out.cpu().numpy()

    def all_prob(self, input_state=None):
        if input_state is not None:
            self.set_input_state(input_state)
        amps = self.prob_amplitudes(self._get_iterator(self._input_state))
        return (np.abs(amps) ** 2).tolist()

    def prob_distribution(self) -> BSDistribution:
        bsd = BSDistribution()
        for s, p in zip(self._get_iterator(self._input_state), self.all_prob()):
            bsd.add(s, p)
        return bsd

    def evolve(self) -> StateVector:
        states = self._get_iterator(self._input_state)
        amps = self.prob_amplitudes(states)
        res = StateVector()
        for s, a in zip(states, amps):
            res[s] = complex(a)
        return res
