"""SLAP strong simulation on the GPU (restating perceval/backends/_slap.py:38-80).

Every output amplitude of the input state comes from one depth-first walk over the
outputs (``pcvl_slap_amplitudes`` / ``pcvl_slap_probabilities``): no intermediate
Fock layers, 2^n photon-subset values per walker, any number of modes up to 4096 (SLOS
plans stop at 32).  Results equal SLOS's and Naive's: the amplitude of output s is
Perm(U_{s,t}) / sqrt(prod s! prod t!) in descending-lexicographic order.

Under a mask, the outputs are the states ``xq.FSArray(m, n, mask)`` keeps
(_slap.py:30-36), selected on the device (``pcvl_fock_mask_ranks``).  Feed-forward
(_slap.py:82-194) belongs to the processor front-end and is not part of this package:
``can_simulate_feed_forward`` answers False so callers take their default path.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _native
from ..utils.states import BSDistribution, FockState, StateVector, fock_rank, fock_unrank_array
from ._abstract_backends import AStrongSimulationBackend, IFFBackend

_LIST_LIMIT = 1 << 22


class SLAPBackend(AStrongSimulationBackend, IFFBackend):
    def __init__(self, mask=None):
        super().__init__()
        self._u_dev: torch.Tensor | None = None
        self._cache: dict = {}
        if mask is not None:
            self.set_mask(mask)

    @property
    def name(self) -> str:
        return "SLAP"

    def set_circuit(self, circuit):
        super().set_circuit(circuit)
        self._u_dev = None
        self._cache = {}

    def clear_mask(self):
        super().clear_mask()
        self._cache = {}

    # ------------------------------------------------------------ device results
    def _unitary_device(self) -> torch.Tensor:
        if self._u_dev is None:
            _native.load()
            self._u_dev = torch.from_numpy(np.ascontiguousarray(self._umat)).to("cuda")
        return self._u_dev

    def _selection(self, st: FockState):
        """Device ranks of the outputs the mask keeps (None without a mask)."""
        if self._mask is None:
            return None
        key = ("sel", st.n)
        if key not in self._cache:
            self._cache[key] = _native.fock_mask_ranks(st.m, st.n, self._mask)
        return self._cache[key]

    def _all(self, st: FockState, amplitudes: bool) -> torch.Tensor:
        key = ("amp" if amplitudes else "prob", st)
        if key not in self._cache:
            full = _native.slap_all(self._unitary_device(), list(st), amplitudes=amplitudes)
            sel = self._selection(st)
            self._cache[key] = full if sel is None else full[sel]
        return self._cache[key]

    def all_prob_tensor(self, input_state=None) -> torch.Tensor:
        """Probabilities of every output (the accepted ones under a mask), float64 CUDA
        tensor in descending-lexicographic order."""
        if input_state is not None:
            self.set_input_state(input_state)
        return self._all(self._input_state, amplitudes=False)

    def amplitudes_tensor(self) -> torch.Tensor:
        return self._all(self._input_state, amplitudes=True)

    def _get_iterator(self, input_state):
        if self._mask is not None and isinstance(input_state, FockState) and input_state.n not in self._cache_iterator:
            ranks = self._selection(input_state).cpu().numpy()
            arr = fock_unrank_array(input_state.m, input_state.n, ranks)
            self._cache_iterator[input_state.n] = tuple(FockState(row) for row in arr)
        return super()._get_iterator(input_state)

    # ------------------------------------------------------------ reference API
    def prob_amplitude(self, output_state) -> complex:
        output_state = FockState(output_state)
        istate = self._input_state
        if istate.n != output_state.n:
            return complex(0)
        assert output_state.m == istate.m, "output state size mismatch"
        r = fock_rank(output_state)
        sel = self._selection(istate)
        if sel is not None:  # index in FSArray(m, n, mask) (_slap.py:45-50)
            ranks = sel.cpu().numpy()
            pos = int(np.searchsorted(ranks, r))
            assert pos < len(ranks) and int(ranks[pos]) == r, "output state is not accepted by the mask"
            r = pos
        return complex(self.amplitudes_tensor()[r].item())

    def all_prob(self, input_state=None):
        probs = self.all_prob_tensor(input_state).cpu().numpy()
        return probs.tolist() if probs.size <= _LIST_LIMIT else probs

    def prob_distribution(self) -> BSDistribution:
        bsd = BSDistribution()
        for s, p in zip(self._get_iterator(self._input_state), self.all_prob()):
            bsd.add(s, p)
        return bsd

    def evolve(self) -> StateVector:
        amps = self.amplitudes_tensor().cpu().numpy()
        res = StateVector()
        for s, a in zip(self._get_iterator(self._input_state), amps):
            res[s] = complex(a)
        return res

    # ------------------------------------------------------------ feed-forward
    @staticmethod
    def can_simulate_feed_forward(components, input_state, detectors=None) -> bool:
        return False

    def set_feed_forward(self, components, m: int) -> None:
        raise NotImplementedError("feed-forward configurators are not part of the GPU backends")
