"""Backend interfaces, restating perceval/backends/_abstract_backends.py:39-208.

Same method names, argument meaning and error behaviour as the reference:
``set_circuit`` raises RuntimeError for polarized circuits and clears the input state;
``set_input_state`` asserts that a circuit is set and that the sizes match;
``prob_amplitude`` / ``probability`` / ``all_prob`` / ``prob_distribution`` /
``prob_iterator`` / ``evolve`` / ``set_mask`` / ``clear_mask`` behave as there.
``set_circuit`` also accepts a raw m x m unitary (wrapped like ``Unitary(U)``).
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Iterable

import numpy as np

from ..components import ACircuit, Unitary
from ..utils.states import (BSDistribution, BSSamples, FockState, FSMask, StateVector, allstate_iterator)
from ..utils.globals import global_params


def _as_circuit(circuit) -> ACircuit:
    if isinstance(circuit, ACircuit):
        return circuit
    return Unitary(np.asarray(circuit, dtype=complex))


class ABackend(ABC):
    def __init__(self):
        self._circuit = None
        self._umat = None
        self._input_state = None

    def set_circuit(self, circuit):
        """Sets the circuit to simulate (no polarized components); clears the input state."""
        circuit = _as_circuit(circuit)
        if circuit.requires_polarization:
            raise RuntimeError("Circuit must not contain polarized components")
        self._input_state = None
        self._circuit = circuit
        self._umat = np.ascontiguousarray(circuit.compute_unitary(), dtype=np.complex128)

    def set_input_state(self, input_state):
        """Sets a Fock input state (no annotations)."""
        input_state = FockState(input_state)
        self._check_state(input_state)
        self._input_state = input_state

    def _check_state(self, state: FockState):
        assert self._circuit is not None, 'Circuit must be set before the input state'
        assert self._circuit.m == state.m, f'Circuit({self._circuit.m}) and state({state.m}) size mismatch'

    @property
    @abstractmethod
    def name(self) -> str:
        """Back-end name"""


class ASamplingBackend(ABackend):
    @abstractmethod
    def sample(self) -> FockState:
        """One sample of the output for the current circuit and input state"""

    @abstractmethod
    def samples(self, count: int) -> BSSamples:
        """``count`` samples of the output for the current circuit and input state"""


class _StateProbIterator:
    def __init__(self, states, probs):
        self.states = states
        self.probs = probs

    def __iter__(self):
        return zip(self.states, self.probs)


class AStrongSimulationBackend(ABackend):
    def __init__(self):
        super().__init__()
        self._mask_n = None
        self._cache_iterator: dict = {}
        self._masks_str: list[str] | None = None
        self._mask: FSMask | None = None
        self._no_limit_modes: list[int] | None = None

    def set_mask(self, masks: str | list[str], n=None, at_least_modes=None):
        """Restrict strong simulation to output states matching one of ``masks``
        (digits fix a mode's photon count, space or ``*`` accept any count)."""
        self.clear_mask()
        if isinstance(masks, str):
            masks = [masks]
        mask_length = len(masks[0])
        for m in masks:
            m = m.replace("*", " ")
            assert len(m) == mask_length, "Inconsistent mask lengths"
        self._masks_str = masks
        self._mask_n = n
        self._no_limit_modes = at_least_modes
        self._init_mask()

    def _init_mask(self):
        if self._masks_str is not None and self._input_state is not None:
            instate = self._input_state
            assert len(self._masks_str[0]) == instate.m, "Mask and input state lengths have to be the same"
            self._mask = FSMask(instate.m, self._mask_n or instate.n, self._masks_str, self._no_limit_modes)

    def clear_mask(self):
        """Removes any mask."""
        self._masks_str = None
        self._mask = None
        self._mask_n = None
        self.clear_iterator_cache()

    def set_input_state(self, input_state):
        super().set_input_state(input_state)
        self._init_mask()

    def _get_iterator(self, input_state: FockState):
        n = input_state.n
        if n not in self._cache_iterator:
            self._cache_iterator[n] = tuple(allstate_iterator(input_state, self._mask))
        return self._cache_iterator[n]

    def clear_iterator_cache(self):
        self._cache_iterator = {}

    def set_circuit(self, circuit):
        circuit = _as_circuit(circuit)
        if self._circuit is not None and circuit.m != self._circuit.m:
            self.clear_iterator_cache()
        super().set_circuit(circuit)

    @abstractmethod
    def prob_amplitude(self, output_state) -> complex:
        """Amplitude of ``output_state`` (circuit and input state must be set)."""

    def probability(self, output_state) -> float:
        return abs(self.prob_amplitude(output_state)) ** 2

    def all_prob(self, input_state=None) -> list[float]:
        """Probabilities of all output states (mask respected), in ``allstate_iterator`` order."""
        if input_state is not None:
            self.set_input_state(input_state)
        return [self.probability(s) for s in self._get_iterator(self._input_state)]

    def prob_distribution(self) -> BSDistribution:
        bsd = BSDistribution()
        for s, p in zip(self._get_iterator(self._input_state), self.all_prob()):
            bsd.add(s, p)
        return bsd

    def prob_iterator(self, min_p: float = global_params["min_p"]) -> Iterable[tuple[FockState, float]]:
        probs = self.all_prob(self._input_state)
        states = [s for i, s in enumerate(self._get_iterator(self._input_state)) if probs[i] > min_p]
        return _StateProbIterator(states, [p for p in probs if p > min_p])

    def evolve(self) -> StateVector:
        res = StateVector()
        for s in self._get_iterator(self._input_state):
            res[s] = complex(self.prob_amplitude(s))
        return res


class IFFBackend(ABC):
    """Backends that can simulate feed-forward configurators themselves
    (perceval/backends/_abstract_backends.py:211-236); the feed-forward simulator asks
    ``can_simulate_feed_forward`` before handing them the components."""

    @staticmethod
    @abstractmethod
    def can_simulate_feed_forward(components, input_state, detectors=None) -> bool:
        """True when the backend's output for these components and input is correct."""

    @abstractmethod
    def set_feed_forward(self, components, m: int) -> None:
        """Sets the components (with at least one configurator) in place of a circuit."""
