"""Fock-state containers used at the backend boundary.

The reference aliases these to closed native types (perceval/utils/states.py:42-49:
``FockState``, ``BasicState``, ``BSDistribution``, ``BSSamples``, ``BSCount``,
``StateVector``).  They are restated here as small pure-Python containers with the
same observable behaviour that the backend API relies on:

* ``FockState`` is an immutable, hashable occupation vector with ``m``, ``n``,
  ``prodnfact()``, indexing (a slice is a ``FockState``), iteration, the ``|a,b,c>``
  text form, ``merge`` (mode-wise sum of two states' photons, what the simulators'
  recombination of distinguishable parts calls, perceval/simulators/
  _simulator_utils.py:77,164) and ``set_slice`` (perceval/simulators/stepper.py:94).
* ``StateVector`` maps ``FockState`` to complex amplitudes, supports ``+``, ``-``
  and scalar ``*`` and ``normalize()``; iterating it yields (state, amplitude) pairs,
  as the reference's does (perceval/simulators/stepper.py:92,
  _simulator_utils.py:132), and so does ``unnormalized_iterator()``; ``keys()`` gives
  the states.
* ``BSDistribution`` maps ``FockState`` to probabilities (``add`` accumulates).
* ``BSSamples`` is a list of ``FockState``; ``BSCount`` counts them.

Enumeration order follows the reference: descending lexicographic order of the
occupation vector within a fixed photon number
(tests/utils/test_statevector.py:430-438, perceval/utils/states.py:268-298).
"""
from __future__ import annotations

import functools
import math
import re
from typing import Iterable, Iterator, Sequence

import numpy as np

from .globals import global_params

_MIN_P = global_params["min_p"]

class FockState(tuple):
    """Occupation numbers of m optical modes (photon counts per mode)."""

    __slots__ = ()

    def __new__(cls, state: "Sequence[int] | str | int" = ()):
        if isinstance(state, FockState):
            return state
        if isinstance(state, str):
            state = _parse_state(state)
        elif isinstance(state, (int, np.integer)):
            state = [0] * int(state)
        vals = tuple(int(v) for v in state)
        if any(v < 0 for v in vals):
            raise ValueError("photon counts must be non-negative")
        return super().__new__(cls, vals)

    @classmethod
    def _trusted(cls, counts: tuple) -> "FockState":
        """A state from a tuple of non-negative Python ints, without checks."""
        return tuple.__new__(cls, counts)

    @property
    def m(self) -> int:
        return len(self)

    @property
    def n(self) -> int:
        return sum(self)

    def prodnfact(self) -> int:
        """Product of the factorials of the per-mode photon counts."""
        p = 1
        for v in self:
            p *= math.factorial(v)
        return p

    def photon2mode(self, k: int) -> int:
        """Mode index of the k-th photon (photons ordered by mode)."""
        acc = 0
        for i, v in enumerate(self):
            acc += v
            if k < acc:
                return i
        raise IndexError(k)

    def __str__(self) -> str:
        return "|" + ",".join(str(v) for v in self) + ">"

    def __repr__(self) -> str:
        return str(self)

    def __mul__(self, other):
        if isinstance(other, FockState):
            # tensor product of two Fock states
            return FockState(tuple(self) + tuple(other))
        if isinstance(other, (int, float, complex, np.number)):
            return StateVector({self: complex(other)})
        return NotImplemented

    def __rmul__(self, other):
        if isinstance(other, (int, float, complex, np.number)):
            return StateVector({self: complex(other)})
        return NotImplemented

    def __add__(self, other):
        return StateVector(self) + other

    def __getitem__(self, item):
        res = tuple.__getitem__(self, item)
        if isinstance(item, slice):
            return FockState(res)
        return res

    def merge(self, other: "FockState") -> "FockState":
        """The state holding both states' photons: counts added mode by mode (the two
        states have the same number of modes)."""
        other = FockState(other)
        if len(other) != len(self):
            raise ValueError(f"cannot merge states of {len(self)} and {len(other)} modes")
        return FockState._trusted(tuple(a + b for a, b in zip(self, other)))

    def set_slice(self, sl: slice, state: "FockState") -> "FockState":
        """A copy whose modes ``sl`` are replaced by the occupations of ``state``."""
        vals = list(self)
        idx = range(*sl.indices(len(vals)))
        state = FockState(state)
        if len(idx) != len(state):
            raise ValueError("the replacement state does not have the slice's number of modes")
        for i, v in zip(idx, state):
            vals[i] = v
        return FockState._trusted(tuple(vals))


BasicState = FockState


def _parse_state(s: str) -> list[int]:
    s = s.strip()
    m = re.fullmatch(r"\|([0-9,\s]*)>", s)
    if not m:
        raise ValueError(f"cannot parse Fock state {s!r}")
    body = m.group(1).strip()
    if not body:
        return []
    return [int(x) for x in body.split(",")]


class StateVector(dict):
    """Superposition of Fock states: ``FockState -> complex`` amplitude."""

    def __init__(self, init=None):
        super().__init__()
        if init is None:
            return
        if isinstance(init, dict):
            for k, v in init.items():
                self[FockState(k)] = complex(v)
        else:
            self[FockState(init)] = 1.0 + 0j

    @property
    def m(self) -> int:
        return next(iter(self.keys())).m if self else 0

    def __iter__(self):
        """(state, amplitude) pairs, as the reference's StateVector iterates."""
        return iter(self.items())

    def unnormalized_iterator(self):
        """(state, amplitude) pairs without normalisation."""
        return iter(self.items())

    def __add__(self, other):
        res = StateVector(dict(self))
        if isinstance(other, FockState):
            other = StateVector(other)
        for k, v in other.items():
            res[k] = res.get(k, 0j) + v
        return res

    __iadd__ = __add__

    def __sub__(self, other):
        return self + (-1) * (StateVector(other) if isinstance(other, FockState) else other)

    def __mul__(self, scalar):
        if not isinstance(scalar, (int, float, complex, np.number)):
            return NotImplemented
        return StateVector({k: v * scalar for k, v in self.items()})

    __rmul__ = __mul__

    def __neg__(self):
        return self * -1

    def normalize(self):
        """Drop numerically-zero amplitudes (|a|^2 < min_p) and rescale to unit norm."""
        for k in [k for k, v in self.items() if abs(v) ** 2 < _MIN_P]:
            del self[k]
        norm = math.sqrt(sum(abs(v) ** 2 for v in self.values()))
        if norm > 0:
            for k in list(self.keys()):
                self[k] /= norm
        return self


class BSDistribution(dict):
    """Probability distribution over Fock states.

    ``add`` ignores probabilities below ``global_params["min_p"]`` (1e-16): the
    reference's distributions leave numerically-zero outputs out (a masked CNOT
    distribution has exactly its two non-zero outputs,
    tests/backends/test_backends.py:203-218).
    """

    def __missing__(self, key):
        # a state absent from the distribution has probability 0, so ``d[s] += p``
        # accumulates (perceval/simulators/simulator.py:497)
        return 0.0

    def add(self, state: FockState, p: float):
        p = float(p)
        if p < _MIN_P:
            return
        state = FockState(state)
        self[state] = self.get(state, 0.0) + p

    def normalize(self):
        tot = sum(self.values())
        if tot > 0:
            for k in self:
                self[k] /= tot
        return self


class BSCount(dict):
    """Occurrence counts of Fock states (missing keys count 0)."""

    def __missing__(self, key):
        return 0

    def __getitem__(self, key):
        return dict.get(self, FockState(key), 0)

    def __setitem__(self, key, value):
        dict.__setitem__(self, FockState(key), value)


class BSSamples(list):
    """List of sampled Fock states."""


# ----------------------------------------------------------------------------------
# Fock-space enumeration (the FSArray equivalent), descending lexicographic order.
# ----------------------------------------------------------------------------------

def fock_space_size(m: int, n: int) -> int:
    """Number of n-photon states on m modes: C(m+n-1, n)."""
    if m <= 0:
        return 1 if n == 0 else 0
    return math.comb(m + n - 1, n)


def fock_space_array(m: int, n: int) -> np.ndarray:
    """All n-photon occupation vectors on m modes, descending-lex order, as an int array.

    Row r is the state of rank r (the index used by ``all_prob``).  Built by the
    block recursion of descending-lex order: states with first-mode count a form a
    contiguous block, blocks ordered from a = n down to 0.
    """
    if m == 0:
        return np.zeros((1 if n == 0 else 0, 0), dtype=np.int32)
    if m == 1:
        return np.array([[n]], dtype=np.int32)
    blocks = []
    for a in range(n, -1, -1):
        tail = fock_space_array(m - 1, n - a)
        blk = np.empty((tail.shape[0], m), dtype=np.int32)
        blk[:, 0] = a
        blk[:, 1:] = tail
        blocks.append(blk)
    return np.concatenate(blocks, axis=0)


def fock_rank(state: Sequence[int]) -> int:
    """Rank of a state in descending-lex order of its (m, n) Fock space.

    rank(s) = sum_i count(m - i, r_{i+1} - 1) where r_{i+1} is the number of photons
    in modes after i: every state with a larger count in mode i (and equal counts
    before) precedes s, and those form count(m - i, r_{i+1} - 1) states.
    """
    m = len(state)
    rest = sum(state)
    rank = 0
    for i, v in enumerate(state):
        rest -= v
        if rest > 0:
            rank += fock_space_size(m - i, rest - 1)
    return rank


@functools.lru_cache(maxsize=64)
def _rank_sizes(m: int, n: int) -> np.ndarray:
    """size[M, x] = count(M, x - 1), the states of x - 1 photons on M modes (0 for x = 0)."""
    size = np.zeros((m + 1, n + 1), dtype=np.int64)
    for M in range(1, m + 1):
        for x in range(1, n + 1):
            size[M, x] = fock_space_size(M, x - 1)
    size.setflags(write=False)
    return size


def fock_rank_array(arr) -> np.ndarray:
    """Ranks (int64) of the occupation vectors in the rows of ``arr``, all of one photon
    count; vectorised ``fock_rank``."""
    arr = np.asarray(arr, dtype=np.int64)
    if arr.ndim != 2 or arr.shape[0] == 0:
        return np.zeros(arr.shape[0] if arr.ndim == 2 else 0, dtype=np.int64)
    k, m = arr.shape
    n = int(arr[0].sum())
    size = _rank_sizes(m, n)
    rest = n - np.cumsum(arr, axis=1)  # photons after each mode
    return size[np.arange(m, 0, -1)[None, :], rest].sum(axis=1)


def fock_unrank(m: int, n: int, rank: int) -> FockState:
    """Inverse of ``fock_rank``."""
    out = []
    rest = n
    for i in range(m - 1):
        # choose the count v in mode i: blocks for v = rest, rest-1, ..., 0
        v = rest
        while True:
            blk = fock_space_size(m - i - 1, rest - v)
            if rank < blk:
                break
            rank -= blk
            v -= 1
        out.append(v)
        rest -= v
    out.append(rest)
    return FockState(out)


def fock_unrank_array(m: int, n: int, ranks) -> np.ndarray:
    """Occupation vectors (rows) of the states with the given ranks in the n-photon
    space on m modes; vectorised ``fock_unrank``."""
    r = np.asarray(ranks, dtype=np.int64).copy()
    out = np.zeros((len(r), m), dtype=np.int32)
    rest = np.full(len(r), n, dtype=np.int64)
    for i in range(m - 1):
        # photons after mode i: smallest x with rank < count(m - i, x); offset count(m - i, x - 1)
        after = np.zeros(len(r), dtype=np.int64)
        for x in range(n + 1):
            cum = fock_space_size(m - i, x)
            after += (r >= cum) & (after == x) & (x < rest)
        prev = np.array([fock_space_size(m - i, int(x) - 1) if x > 0 else 0 for x in range(n + 1)],
                        dtype=np.int64)
        r = r - prev[after]
        out[:, i] = rest - after
        rest = after
    out[:, m - 1] = rest
    return out


def allstate_iterator(input_state, mask=None) -> Iterator[FockState]:
    """Iterate all output states with the input's photon number(s), respecting a mask.

    Follows perceval/utils/states.py:268-290 (order of ``FSArray`` iteration).
    """
    m = input_state.m
    if isinstance(input_state, StateVector):
        ns = sorted({s.n for s in input_state.keys()})
    else:
        ns = [input_state.n]
    for n in ns:
        arr = fock_space_array(m, n)
        if mask is not None:
            arr = arr[mask.accepts_space(arr)]
        for row in arr:
            yield FockState(row)


def max_photon_state_iterator(m: int, n_max: int) -> Iterator[FockState]:
    """All states on m modes with 0..n_max photons (perceval/utils/states.py:292-298)."""
    for n in range(n_max + 1):
        for row in fock_space_array(m, n):
            yield FockState(row)


class FSMask:
    """Restriction of a Fock space by per-mode conditions.

    Restates the mask semantics used by ``AStrongSimulationBackend.set_mask``
    (perceval/backends/_abstract_backends.py:103-137; tests/utils/test_mask.py:32-45):
    each mask string has one character per mode; a digit fixes the photon count of
    that mode, a space or ``*`` accepts any count.  A state is accepted when it
    matches at least one mask string.  Modes listed in ``at_least_modes`` accept any
    count greater than or equal to their digit.  ``match(state, partial=True)``
    accepts states with fewer photons that can still be completed to a match with
    the ``n`` photons the mask was built for.
    """

    def __init__(self, m: int, n: int, masks: Iterable[str], at_least_modes=None):
        self.m = m
        self.n = n
        self._conds = []
        at_least = set(at_least_modes or [])
        self._at_least = at_least
        for s in masks:
            s = s.replace("*", " ")
            assert len(s) == m, "Mask and state lengths have to be the same"
            cond = []
            for i, ch in enumerate(s):
                if ch == " ":
                    continue
                cond.append((i, int(ch), i in at_least))
            self._conds.append(cond)

    def match(self, state, partial: bool = False) -> bool:
        state = FockState(state)
        for cond in self._conds:
            if self._match_one(cond, state, partial):
                return True
        return False

    def _match_one(self, cond, state, partial) -> bool:
        missing = 0
        for i, d, at_least in cond:
            v = state[i]
            if at_least:
                if v < d:
                    if not partial:
                        return False
                    missing += d - v
            elif partial:
                if v > d:
                    return False
                missing += d - v
            elif v != d:
                return False
        if partial:
            return missing <= self.n - state.n
        return True

    def match_array(self, arr: np.ndarray, partial: bool = False) -> np.ndarray:
        """Vectorised ``match`` over rows of an occupation array."""
        ok = np.zeros(arr.shape[0], dtype=bool)
        spare = self.n - arr.sum(axis=1)
        for cond in self._conds:
            cur = np.ones(arr.shape[0], dtype=bool)
            missing = np.zeros(arr.shape[0], dtype=np.int64)
            for i, d, at_least in cond:
                v = arr[:, i]
                if not partial:
                    cur &= (v >= d) if at_least else (v == d)
                elif at_least:
                    missing += np.maximum(d - v, 0)
                else:
                    cur &= v <= d
                    missing += d - v
            if partial:
                cur &= missing <= spare
            ok |= cur
        return ok

    def accepts_space(self, arr: np.ndarray) -> np.ndarray:
        """The states of one layer that ``xq.FSArray(m, k, mask)`` keeps: those that can
        still be completed to a match with ``n`` photons (a full match when they hold
        ``n`` photons)."""
        return self.match_array(arr, partial=True)

    @property
    def at_least_modes(self) -> list[int]:
        return sorted(self._at_least)

    def device_spec(self):
        """(digits, at_least bits, n) for ``pcvl_slos_plan_create_masked``: digits is an
        int8 (masks x m) array with -1 where a mask accepts any count."""
        digits = np.full((len(self._conds), self.m), -1, dtype=np.int8)
        for q, cond in enumerate(self._conds):
            for i, d, _ in cond:
                digits[q, i] = d
        bits = 0
        for i in self._at_least:
            if 0 <= i < self.m:
                bits |= 1 << i
        return np.ascontiguousarray(digits), bits, self.n
