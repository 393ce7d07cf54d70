"""SLOS strong simulation on the GPU (restating perceval/backends/_slos.py:105-223).

Each distinct input state gets a device plan (``pcvl_slos_plan``): the layer chain in
the photon order of ``_Path._decompose`` (_slos.py:61-86) runs as one gather kernel
per photon over on-the-fly Fock ranks, in native FP64 (complex128 coefficients, as the
reference's layers, _slos.py:44,99) unless the backend is made with
``precision="float-float"`` (FP32-pipe pairs, ~48 significant bits, faster).  As in the
reference, changing the circuit to another one of the same size keeps the plans and
recomputes their coefficients (_slos.py:130-141); a different size resets them.

Outputs come back in descending-lexicographic order (the reference's
``allstate_iterator`` order).  With a mask (``set_mask``) the plans are masked plans:
every layer holds only the states the mask can still accept (xq.FSArray(m, k, mask),
_slos.py:161-164), and the outputs are the accepted states in the same order.
``all_prob`` returns a list up to 2^22 outputs and a numpy array above;
``all_prob_tensor`` leaves the probabilities on the device.  Circuits wider than the
32 modes of SLOS plans take the SLAP walk (``pcvl_slap_*``, float-float arithmetic),
which computes the same amplitudes, with the mask's outputs selected on the device.

``all_probs_many`` / ``prob_distributions`` evaluate many input states of the circuit
at once (the per-input loop of Simulator._probs_svd_fast, simulator.py:454-468): states
with the same photon count share every layer's Fock space, so each such group runs as
one batched plan whose entries add their own input modes, one launch per photon layer
for the whole group.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .. import _native
from ..utils.states import BSDistribution, FSMask, FockState, StateVector, fock_rank, fock_unrank_array
from ._abstract_backends import AStrongSimulationBackend, _as_circuit

_LIST_LIMIT = 1 << 22
_PLAN_MAX_M = 32  # SLOS plans address modes with 32-bit masks; wider circuits take the SLAP walk


class _Entry:
    """Plan and cached results of one input state (plan None: more than 32 modes, the
    outputs come from the SLAP walk, which gives the same amplitudes)."""

    def __init__(self, plan: _native.SlosPlan | None):
        self.plan = plan
        self.fresh = False           # cached results belong to the current unitary
        self.layer_ok = False        # the plan's last layer holds this unitary's coefficients
        self.probs = None            # device tensor
        self.amps = None             # device tensor
        self.amps_host = None        # numpy copy (small spaces)
        self.ranks = None            # masked plan: full-space ranks of the accepted outputs


class SLOSBackend(AStrongSimulationBackend):
    def __init__(self, mask=None, use_symbolic: bool = False, precision: str = "fp64"):
        super().__init__()
        if use_symbolic:
            raise NotImplementedError("symbolic SLOS stays on the CPU reference; this backend is numeric only")
        self._precision = _native.precision_code(precision)
        if self._precision not in (_native.PREC_FP64, _native.PREC_FLOAT_FLOAT):
            raise ValueError("precision must be 'fp64' or 'float-float'")
        self._entries: dict[FockState, _Entry] = {}
        self._u_dev: torch.Tensor | None = None
        if mask is not None:
            self.set_mask(mask)

    @property
    def name(self) -> str:
        return "SLOS"

    def _reset(self):
        for e in self._entries.values():
            if e.plan is not None:
                e.plan.close()
        self._entries = {}
        self.clear_iterator_cache()

    def set_circuit(self, circuit):
        circuit = _as_circuit(circuit)
        previous = self._circuit
        super().set_circuit(circuit)
        self._u_dev = None
        if self._entries and previous is not None and previous.m == circuit.m:
            for e in self._entries.values():
                e.fresh = False
        else:
            self._reset()

    def clear_mask(self):
        super().clear_mask()
        self._reset()  # plans are built for a mask (_slos.py:147-149)

    def _unitary_device(self) -> torch.Tensor:
        if self._u_dev is None:
            _native.load()
            self._u_dev = torch.from_numpy(self._umat).to("cuda")
        return self._u_dev

    def set_input_state(self, input_state):
        super().set_input_state(input_state)
        self._entry()

    def preprocess(self, input_list) -> bool:
        """Plans for the input states of ``input_list`` that have none yet (_slos.py:171-185);
        True when at least one was new.  Their coefficients are computed on first use."""
        found_new = False
        for st in input_list:
            st = FockState(st)
            if st not in self._entries:
                if st.m > _PLAN_MAX_M:
                    e = _Entry(None)
                    if self._mask is not None:
                        e.ranks = _native.fock_mask_ranks(st.m, st.n, self._mask).cpu().numpy().astype(np.uint64)
                else:
                    e = _Entry(_native.SlosPlan(st.m, list(st), batch=1, keep_layers=False, mask=self._mask,
                                                precision=self._precision))
                    if self._mask is not None:
                        e.ranks = e.plan.output_ranks()
                self._entries[st] = e
                found_new = True
        return found_new

    def _entry(self) -> _Entry:
        st = self._input_state
        self.preprocess([st])
        e = self._entries[st]
        if not e.fresh:
            e.probs = e.amps = e.amps_host = None
            e.layer_ok = False
            e.fresh = True
        return e

    # -------------------------------------------------------------- results
    def all_prob_tensor(self, input_state=None) -> torch.Tensor:
        """Probabilities of every output (the accepted ones under a mask) as a float64
        CUDA tensor, in descending-lexicographic order."""
        if input_state is not None:
            self.set_input_state(input_state)
        e = self._entry()
        if e.probs is None:
            if e.plan is None:
                e.probs = self._slap(e, amplitudes=False)
            else:
                # probabilities alone: the last layer writes them directly (not stored)
                e.probs = e.plan.probabilities() if e.layer_ok else e.plan.forward_probabilities(self._unitary_device())
        return e.probs

    def amplitudes_tensor(self) -> torch.Tensor:
        """Amplitudes of every output (the accepted ones under a mask) as a complex128
        CUDA tensor, in descending-lexicographic order."""
        e = self._entry()
        if e.amps is None:
            if e.plan is None:
                e.amps = self._slap(e, amplitudes=True)
            else:
                if not e.layer_ok:
                    e.plan.forward(self._unitary_device())
                    e.layer_ok = True
                e.amps = e.plan.amplitudes()
        return e.amps

    def _slap(self, e: _Entry, amplitudes: bool) -> torch.Tensor:
        """Outputs of a circuit wider than SLOS plans, by the SLAP walk (mask applied)."""
        full = _native.slap_all(self._unitary_device(), list(self._input_state), amplitudes=amplitudes)
        if e.ranks is None:
            return full
        return full[torch.from_numpy(e.ranks.astype(np.int64)).to(full.device)]

    def _get_iterator(self, input_state):
        # under a mask, the accepted outputs are the plan's own (no full-space enumeration)
        if self._mask is not None and isinstance(input_state, FockState) and input_state.n not in self._cache_iterator:
            e = self._entries.get(input_state)
            if e is not None and e.ranks is not None:
                arr = fock_unrank_array(input_state.m, input_state.n, e.ranks)
                self._cache_iterator[input_state.n] = tuple(FockState(row) for row in arr)
        return super()._get_iterator(input_state)

    def _group_mask(self, m: int, n: int) -> FSMask | None:
        """The mask of an input state of n photons (_abstract_backends.py:126-137)."""
        if self._masks_str is None:
            return None
        return FSMask(m, self._mask_n or n, self._masks_str, self._no_limit_modes)

    def all_probs_many(self, input_states, max_device_bytes: int = 1 << 31) -> list[np.ndarray]:
        """Probabilities of every output (descending-lexicographic order, mask applied)
        for each of ``input_states``, evaluated as batched plans grouped by photon count."""
        assert self._circuit is not None, "set_circuit first"
        states = [FockState(s) for s in input_states]
        m = self._circuit.m
        groups: dict[int, list[int]] = {}
        for i, s in enumerate(states):
            assert s.m == m, "input state size mismatch"
            groups.setdefault(s.n, []).append(i)
        U = self._unitary_device()
        res: list = [None] * len(states)
        if m > _PLAN_MAX_M:  # wider than SLOS plans: the SLAP walk per input state
            for n, idxs in groups.items():
                mask = self._group_mask(m, n)
                sel = None if mask is None else _native.fock_mask_ranks(m, n, mask)
                for i in idxs:
                    p = _native.slap_all(U, list(states[i]))
                    res[i] = (p if sel is None else p[sel]).cpu().numpy()
            return res
        for n, idxs in sorted(groups.items()):
            count = math.comb(m + n - 1, n)
            # two layers of 16-byte coefficients per entry dominate a plan's memory
            per_entry = 2 * 16 * max(count, 1)
            step = max(1, min(len(idxs), max_device_bytes // per_entry))
            mask = self._group_mask(m, n)
            for c0 in range(0, len(idxs), step):
                chunk = idxs[c0:c0 + step]
                arr = np.array([list(states[i]) for i in chunk], dtype=np.int32)
                plan = _native.SlosPlan(m, arr, keep_layers=False, mask=mask, precision=self._precision)
                try:
                    plan.forward(U)
                    host = plan.probabilities().view(plan.count, len(chunk)).cpu().numpy()
                finally:
                    plan.close()
                for col, i in enumerate(chunk):
                    res[i] = np.ascontiguousarray(host[:, col])
        return res

    def prob_distributions(self, input_states) -> list[BSDistribution]:
        """``prob_distribution`` of each input state, computed by ``all_probs_many``."""
        states = [FockState(s) for s in input_states]
        out = []
        for s, probs in zip(states, self.all_probs_many(states)):
            bsd = BSDistribution()
            for o, p in zip(self._get_iterator(s), probs):
                bsd.add(o, p)
            out.append(bsd)
        return out

    def all_prob(self, input_state=None):
        if input_state is not None:
            self.set_input_state(input_state)
        probs = self.all_prob_tensor().cpu().numpy()
        return probs.tolist() if probs.size <= _LIST_LIMIT else probs

    def prob_distribution(self) -> BSDistribution:
        probs = self.all_prob()
        bsd = BSDistribution()
        for s, p in zip(self._get_iterator(self._input_state), probs):
            bsd.add(s, p)
        return bsd

    def prob_amplitude(self, output_state) -> complex:
        output_state = FockState(output_state)
        if self._input_state.n != output_state.n:
            return complex(0)
        assert output_state.m == self._input_state.m, "output state size mismatch"
        e = self._entry()
        r = fock_rank(output_state)
        if e.ranks is not None:  # index among the accepted outputs (_slos.py:190-191)
            pos = int(np.searchsorted(e.ranks, np.uint64(r)))
            assert pos < len(e.ranks) and int(e.ranks[pos]) == r, "output state is not accepted by the mask"
            r = pos
        count = e.plan.count if e.plan is not None else (
            len(e.ranks) if e.ranks is not None else _native.slap_output_count(output_state.m, list(self._input_state)))
        if count <= _LIST_LIMIT:
            if e.amps_host is None:
                e.amps_host = self.amplitudes_tensor().cpu().numpy()
            return complex(e.amps_host[r])
        return complex(self.amplitudes_tensor()[r].item())

    def evolve(self) -> StateVector:
        amps = self.amplitudes_tensor().cpu().numpy()
        res = StateVector()
        states = self._get_iterator(self._input_state)
        for s, a in zip(states, amps):
            res[s] = complex(a)
        return res
