"""Callers of the backends that simulate many input states at once.

Perceval's simulators reach the backends through per-input loops; this module restates the
two that matter for throughput so that every distinct input state of a request goes to the
device in one batched call per photon count:

* ``Simulator.probs_svd`` follows Simulator.probs_svd / _preprocess_svd / _probs_svd_fast
  (perceval/simulators/simulator.py:524-567, 412-514, 576-648) for a mixture of input states,
  each given by its separated, mutually distinguishable parts (the result of
  ``NoisyFockState.separate_state``, or a plain Fock state): inputs below the
  detected-photon filter count against the physical performance, inputs at or below the
  probability threshold max(min_p, max_p x precision) are dropped, every distinct part is
  simulated once (``SLOSBackend.all_probs_many``: one batched plan per photon count, in place
  of one ``set_input_state`` + ``prob_iterator`` per state), the parts of an input are merged
  like _list_merge (perceval/simulators/_simulator_utils.py:148-171: photon counts add mode by
  mode, probabilities multiply, a branch is cut as soon as its product falls below
  threshold / (10 prob)), and the merged distributions are weighted by the inputs'
  probabilities, summed and normalised.
* ``SamplesProvider`` follows perceval/simulators/noisy_sampling_simulator.py:44-131: pools
  of output samples per input state.  ``prepare`` draws the first pools of every input with
  one sampler wavefront per photon count (``Clifford2017Backend.samples_many``); the samples
  equal the reference's loop of ``set_input_state`` + ``samples(count)`` in the same order,
  since every input keeps the sample counters it would have in that loop.

Heralds, detectors, post-selection and superposed (non-separable) inputs belong to the
processor front-end and are not part of this module.
"""
from __future__ import annotations

import math
from typing import Callable

import numpy as np

from .utils.globals import global_params
from .utils.states import BSCount, BSDistribution, BSSamples, FockState, fock_rank_array, fock_unrank_array

__all__ = ["Simulator", "SamplesProvider"]

# outputs whose m per-mode counts fit in this many bits are merged as packed integer keys
_PACKED_BITS = 64


def _parts(key) -> tuple[FockState, ...]:
    """Separated parts of an input key: a Fock state, or a sequence of Fock states."""
    if isinstance(key, (FockState, str)):
        return (FockState(key),)
    key = tuple(key)
    if key and not isinstance(key[0], (int, np.integer)):
        return tuple(FockState(p) for p in key)
    return (FockState(key),)


def _input_items(input_dist) -> list[tuple[tuple[FockState, ...], float]]:
    """(parts, probability) of every input of a mapping (one entry per key, like an
    SVDistribution) or of an iterable of (key, probability) pairs, kept entry by entry as
    _probs_svd_fast takes its (states, prob) list (simulator.py:430-431)."""
    items = input_dist.items() if hasattr(input_dist, "items") else input_dist
    return [(_parts(key), float(p)) for key, p in items]


class Simulator:
    """Probability distributions of mixtures of separable input states through one circuit.

    ``backend`` is a strong-simulation backend; SLOS evaluates all distinct input parts of a
    request in batched plans, other backends take them one at a time.
    """

    def __init__(self, backend):
        self._backend = backend
        self._rel_precision = 1e-6  # relative to the most probable input (simulator.py:67)
        self._min_detected_photons_filter = 0
        self._logical_perf = 1.0
        self.DEBUG_merge_count = 0

    @property
    def precision(self) -> float:
        return self._rel_precision

    @precision.setter
    def precision(self, value: float):
        self._rel_precision = float(value)

    def set_precision(self, precision: float):
        self.precision = precision

    def set_min_detected_photons_filter(self, value: int):
        self._min_detected_photons_filter = int(value)

    @property
    def min_detected_photons_filter(self) -> int:
        return self._min_detected_photons_filter

    def set_circuit(self, circuit):
        self._backend.set_circuit(circuit)

    def _get_prob_threshold(self, max_p: float) -> float:
        return max(global_params["min_p"], max_p * self._rel_precision)

    # ------------------------------------------------------------ strong simulation
    def _strong(self, thresholds: dict[FockState, float]) -> dict[FockState, tuple[np.ndarray, np.ndarray]]:
        """(output ranks, probabilities) of every distinct input part, outputs above the
        part's threshold in the order of ``prob_iterator``: one batched call per photon count
        where the backend offers it, else one evaluation per state."""
        res = {}
        work = []
        for s in thresholds:
            if s.n == 0:  # a unitary circuit keeps the vacuum
                res[s] = (np.zeros(1, dtype=np.int64), np.ones(1))
            else:
                work.append(s)
        if not work:
            return res
        if hasattr(self._backend, "all_probs_many"):
            for s, probs in zip(work, self._backend.all_probs_many(work)):
                probs = np.asarray(probs, dtype=np.float64)
                idx = np.nonzero(probs > thresholds[s])[0]
                res[s] = (idx.astype(np.int64), probs[idx])
        else:
            for s in work:
                self._backend.set_input_state(s)
                states_p = list(self._backend.prob_iterator(thresholds[s]))
                rows = np.array([list(o) for o, _ in states_p], dtype=np.int64).reshape(len(states_p), s.m)
                res[s] = (fock_rank_array(rows), np.array([p for _, p in states_p], dtype=np.float64))
        return res

    @staticmethod
    def _merge(parts, cache, rows_cache: dict, threshold: float):
        """_list_merge over the parts' outputs: every combination whose running product stays
        at or above ``threshold``, photon counts summed mode by mode; products are formed left
        to right and the combinations come in the order of the reference's recursion.
        Returns (occupation rows of the merged outputs, probabilities)."""

        def rows(s):
            if s not in rows_cache:
                rows_cache[s] = fock_unrank_array(s.m, s.n, cache[s][0]).astype(np.int64)
            return rows_cache[s]

        p = cache[parts[0]][1]
        keep = p >= threshold
        cur, p = rows(parts[0])[keep], p[keep]
        for s in parts[1:]:
            prod = p[:, None] * cache[s][1][None, :]
            i, j = np.nonzero(prod >= threshold)
            cur = cur[i] + rows(s)[j]
            p = prod[i, j]
        return cur, p

    @staticmethod
    def _merge_keys(parts, cache, keys_cache: dict, shifts: np.ndarray, threshold: float):
        """``_merge`` on packed outputs: a state is one uint64 key (per-mode counts in digits
        of fixed width, mode 0 highest), so merged photon counts are sums of keys.  Returns
        (keys of the merged outputs, probabilities)."""

        def keys(s):
            if s not in keys_cache:
                rows = fock_unrank_array(s.m, s.n, cache[s][0]).astype(np.uint64)
                keys_cache[s] = (rows << shifts).sum(axis=1, dtype=np.uint64)
            return keys_cache[s]

        p = cache[parts[0]][1]
        keep = p >= threshold
        k, p = keys(parts[0])[keep], p[keep]
        for s in parts[1:]:
            prod = p[:, None] * cache[s][1][None, :]
            i, j = np.nonzero(prod >= threshold)
            k = k[i] + keys(s)[j]
            p = prod[i, j]
        return k, p

    def _recombine_packed(self, decomposed, cache, p_threshold: float, m: int, bits: int) -> BSDistribution:
        """Recombination on packed keys: each input's merged outputs summed per state in the
        recursion's order, then every input's weighted sums added per state in input order
        (one ``bincount`` over all of them), as the reference's dict accumulates them."""
        shifts = (bits * np.arange(m - 1, -1, -1)).astype(np.uint64)
        keys_cache: dict = {}
        all_k, all_w = [], []
        for prob0, parts, _ in decomposed:
            k, p = self._merge_keys(parts, cache, keys_cache, shifts, p_threshold / (10 * prob0))
            self.DEBUG_merge_count += len(parts) - 1
            if len(parts) == 1:  # distinct outputs already
                out, within = k, p
            else:
                out, inv = np.unique(k, return_inverse=True)
                within = np.bincount(inv, weights=p, minlength=len(out))
            self._logical_perf += float(within.sum()) * prob0
            all_k.append(out)
            all_w.append(within * prob0)
        res = BSDistribution()
        K = np.concatenate(all_k) if all_k else np.zeros(0, dtype=np.uint64)
        if len(K):
            uk, inv = np.unique(K, return_inverse=True)
            acc = np.bincount(inv, weights=np.concatenate(all_w), minlength=len(uk))
            rows = (uk[:, None] >> shifts) & np.uint64((1 << bits) - 1)
            order = np.lexsort((~uk, rows.sum(axis=1)))  # by photon count, then descending-lex
            for row, v in zip(rows[order].astype(np.int64).tolist(), acc[order].tolist()):
                dict.__setitem__(res, FockState._trusted(tuple(row)), v)
        return res

    def probs_svd(self, input_dist, progress_callback: Callable | None = None) -> dict:
        """Output distribution of a mixture of inputs and its performances.

        ``input_dist`` maps each input (a Fock state, or the tuple of its separated parts) to
        its probability, or is an iterable of such (input, probability) pairs.  Returns
        ``{"results": BSDistribution, "physical_perf", "logical_perf", "global_perf"}``.
        """
        items = _input_items(input_dist)
        # trimming (_preprocess_svd, simulator.py:524-567)
        max_p, physical_perf, kept = 0.0, 1.0, []
        for parts, p in items:
            if sum(s.n for s in parts) >= self._min_detected_photons_filter:
                max_p = max(p, max_p)
                kept.append((parts, p))
            else:
                physical_perf -= p
        p_threshold = self._get_prob_threshold(max_p)
        decomposed = [(p, parts, sum(s.n for s in parts)) for parts, p in kept if p > p_threshold]

        self._logical_perf = 0.0
        res = self._probs_svd_fast(decomposed, p_threshold, progress_callback)
        if self._logical_perf > 0 and physical_perf > 0:
            self._logical_perf /= physical_perf
        logical = self._logical_perf if len(res) else 0.0
        return {"results": res, "physical_perf": physical_perf, "logical_perf": logical,
                "global_perf": physical_perf * logical}

    def _use_mask(self):
        """Without heralds the simulator runs on the whole Fock space: a mask left on the
        backend is cleared (Simulator.use_mask, simulator.py:668-672)."""
        if getattr(self._backend, "_masks_str", None) is not None:
            self._backend.clear_mask()

    def _probs_svd_fast(self, decomposed, p_threshold: float, progress_callback=None) -> BSDistribution:
        if not decomposed:
            return BSDistribution()
        self._use_mask()
        if len(decomposed) == 1 and len(decomposed[0][1]) == 1:  # one input, one part (simulator.py:434-444)
            prob0, (state,), _ = decomposed[0]
            self._backend.set_input_state(state)
            res = self._backend.prob_distribution()
            self._logical_perf += sum(res.values()) * prob0
            if len(res):
                res.normalize()
            return res

        # the most probable input that holds each distinct part sets its threshold
        top: dict[FockState, float] = {}
        for prob0, parts, _ in decomposed:
            for s in parts:
                if prob0 > top.get(s, 0.0):
                    top[s] = prob0
        cache = self._strong({s: p_threshold / (10 * p0) for s, p0 in top.items()})
        if progress_callback is not None:
            progress_callback(0.5, "compute probability distributions")

        m = decomposed[0][1][0].m
        bits = max(1, max(n for _, _, n in decomposed).bit_length())
        if m * bits <= _PACKED_BITS:
            res = self._recombine_packed(decomposed, cache, p_threshold, m, bits)
            if progress_callback is not None:
                progress_callback(1.0, "recombine distributions")
            if len(res):
                res.normalize()
            return res

        # wider states: the same recombination on occupation rows
        rows_cache: dict = {}
        all_r, all_w = [], []
        for prob0, parts, _ in decomposed:
            r, p = self._merge(parts, cache, rows_cache, p_threshold / (10 * prob0))
            self.DEBUG_merge_count += len(parts) - 1
            if len(parts) == 1:  # distinct outputs already
                out, within = r, p
            else:  # sums of one input per output, added in recursion order
                out, inv = np.unique(r, axis=0, return_inverse=True)
                within = np.bincount(inv.ravel(), weights=p, minlength=len(out))
            self._logical_perf += float(within.sum()) * prob0
            all_r.append(out)
            all_w.append(within * prob0)
        if progress_callback is not None:
            progress_callback(1.0, "recombine distributions")
        res = BSDistribution()
        R = np.concatenate(all_r) if all_r else np.zeros((0, m), dtype=np.int64)
        if len(R):
            ur, inv = np.unique(R, axis=0, return_inverse=True)
            acc = np.bincount(inv.ravel(), weights=np.concatenate(all_w), minlength=len(ur))
            # by photon count, then descending-lex
            order = np.lexsort(tuple(-ur[:, i] for i in range(m - 1, -1, -1)) + (ur.sum(axis=1),))
            for row, v in zip(ur[order].tolist(), acc[order].tolist()):
                dict.__setitem__(res, FockState._trusted(tuple(row)), v)
        if len(res):
            res.normalize()
        return res

    def probs(self, input_state) -> BSDistribution:
        """Output distribution of one input (a Fock state or its separated parts)."""
        return self.probs_svd({_parts(input_state): 1.0})["results"]


class SamplesProvider:
    """Pools of output samples per input state (noisy_sampling_simulator.py:44-131)."""

    def __init__(self, sampling_backend):
        self._backend = sampling_backend
        self._pools: dict[FockState, list] = {}
        self._weights = BSCount()
        self._sample_coeff = 1.1
        self._min_samples = 100  # sampled at once
        self._max_samples = 2000  # sampled at once; at least 10 x _min_samples
        self.sleep_between_batches = 0.2

    def _pool(self, state: FockState) -> list:
        return self._pools.setdefault(FockState(state), BSSamples())

    def prepare(self, progress_callback: Callable | None = None):
        """First pool of every input whose weight has been estimated: one sampler wavefront
        per photon count for all of them."""
        items = [(FockState(s), min(int(c), self._max_samples)) for s, c in self._weights.items()]
        draw = [(s, c) for s, c in items if s.n > 0]
        if draw and hasattr(self._backend, "samples_many"):
            pools = self._backend.samples_many([s for s, _ in draw], [c for _, c in draw])
        else:
            pools = []
            for s, c in draw:
                self._backend.set_input_state(s)
                pools.append(self._backend.samples(c))
        drawn = dict(zip([s for s, _ in draw], pools))
        for s, c in items:
            self._pools[s] = BSSamples([s] * c) if s.n == 0 else BSSamples(drawn[s])
            self._weights[s] = math.ceil(0.1 * self._weights[s])
        if progress_callback is not None:
            progress_callback(0, "prepare sampling")

    def estimate_weights_from_distribution(self, noisy_input, n_samples: int):
        """Samples to draw per input state when its pool runs empty, from the probability of
        each (separable) input: ``noisy_input`` maps inputs (Fock states or tuples of their
        separated parts) to probabilities."""
        if not n_samples:
            return
        for parts, prob in _input_items(noisy_input):
            ns = min(math.ceil(prob * n_samples), self._max_samples)
            for bs in parts:
                if self._weights[bs] + ns < self._max_samples:
                    self._weights[bs] = self._weights[bs] + ns
                else:
                    self._weights[bs] = self._max_samples

    def estimate_weights_from_source(self, sample_generator: Callable[[int], list], n_samples: int) -> list:
        """Weights from a batch of input samples (each a list of separated Fock states);
        returns that batch."""
        input_samples = sample_generator(n_samples)
        for sample in input_samples:
            for state in sample:
                if self._weights[state] < self._max_samples:
                    self._weights[state] = self._weights[state] + 1
        return input_samples

    def _compute_samples(self, fock_state: FockState):
        if fock_state not in self._weights:
            self._weights[fock_state] = self._min_samples
        n_samples = min(self._weights[fock_state], self._max_samples)
        self._backend.set_input_state(fock_state)
        self._pool(fock_state).extend(self._backend.samples(n_samples))
        self._weights[fock_state] = min(max(int(self._weights[fock_state] * self._sample_coeff), 16),
                                        self._max_samples)

    def sample_from(self, input_state) -> FockState:
        """Pops an output of ``input_state`` from its pool, drawing a new batch when empty."""
        input_state = FockState(input_state)
        if not len(self._pool(input_state)):
            self._compute_samples(input_state)
        return self._pool(input_state).pop()
