"""Simulator.probs_svd and SamplesProvider (the callers that batch many input states).

Host logic on the CPU with fake backends whose distributions come from the oracle's SLOS:
the batched recombination equals a loop-and-dict restatement of the reference's
_probs_svd_fast / _list_merge (perceval/simulators/simulator.py:412-514,
perceval/simulators/_simulator_utils.py:148-171), and the provider's batched pools equal its
per-input loop.  On the GPU the same checks run through SLOS, Naive and CC2017."""
import math
from collections import defaultdict

import numpy as np
import pytest

from perceval_gb300.simulators import SamplesProvider, Simulator
from perceval_gb300.utils import BSDistribution, FockState, random_unitary
from perceval_gb300.utils.states import fock_space_array

MIN_P = 1e-16


# ------------------------------------------------------------------ loop-and-dict restatement
def ref_probs_svd(dist, input_dist, precision=1e-6, min_photons=0):
    """dist(state, min_p) -> [(FockState, p)] in iteration order; input_dist: list of
    (parts, prob).  Returns (distribution dict, physical_perf, logical_perf)."""
    max_p, phys, kept = 0.0, 1.0, []
    for parts, p in input_dist:
        if sum(s.n for s in parts) >= min_photons:
            max_p = max(p, max_p)
            kept.append((parts, p))
        else:
            phys -= p
    thr = max(MIN_P, max_p * precision)
    dec = [(p, parts) for parts, p in kept if p > thr]
    logical = 0.0
    if len(dec) == 1 and len(dec[0][1]) == 1:
        res = {s: p for s, p in dist(dec[0][1][0], MIN_P)}
        logical += sum(res.values()) * dec[0][0]
    else:
        top = {}
        for p, parts in dec:
            for s in parts:
                top[s] = max(top.get(s, 0.0), p)
        cache = {s: dist(s, thr / (10 * p0)) for s, p0 in top.items()}
        res = defaultdict(float)
        for p0, parts in dec:
            t = thr / (10 * p0)
            merged = defaultdict(float)

            def inner(rest, cur, cp):
                if not rest:
                    merged[cur] += cp
                    return
                for bs, q in rest[0]:
                    pr = cp * q
                    if pr < t:
                        continue
                    inner(rest[1:], FockState(a + b for a, b in zip(cur, bs)), pr)

            for bs, q in cache[parts[0]]:
                if q < t:
                    continue
                inner([cache[s] for s in parts[1:]], bs, q)
            logical += sum(merged.values()) * p0
            for bs, q in merged.items():
                res[bs] += q * p0
    tot = sum(res.values())
    res = {k: v / tot for k, v in res.items()} if tot > 0 else {}
    if logical > 0 and phys > 0:
        logical /= phys
    return res, phys, logical


def oracle_dist(oracle, U):
    cache = {}

    def dist(state, min_p):
        if state not in cache:
            cache[state] = oracle.slos(U, list(state))[0] if state.n else np.ones(1)
        probs = cache[state]
        rows = fock_space_array(state.m, state.n)
        return [(FockState(r), float(p)) for r, p in zip(rows, probs) if p > min_p]
    return dist


class FakeStrong:
    """Strong-simulation backend on the oracle's SLOS (CPU), with or without the batched
    entry point."""

    def __init__(self, oracle, U, batched):
        self._U, self._oracle = U, oracle
        self._masks_str = None
        self._input_state = None
        self.batched_calls = 0
        if batched:
            self.all_probs_many = self._all_probs_many

    def _probs(self, s):
        return self._oracle.slos(self._U, list(s))[0]

    def _all_probs_many(self, states):
        self.batched_calls += 1
        return [self._probs(s) for s in states]

    def set_input_state(self, s):
        self._input_state = FockState(s)

    def prob_iterator(self, min_p):
        rows = fock_space_array(self._input_state.m, self._input_state.n)
        return [(FockState(r), float(p)) for r, p in zip(rows, self._probs(self._input_state)) if p > min_p]

    def prob_distribution(self):
        bsd = BSDistribution()
        for s, p in self.prob_iterator(0.0):
            bsd.add(s, p)
        return bsd


def mixture(m, seed, n_inputs, max_parts=3, max_n=2):
    rng = np.random.default_rng(seed)
    items = []
    for _ in range(n_inputs):
        parts = []
        for _ in range(int(rng.integers(1, max_parts + 1))):
            st = [0] * m
            for _ in range(int(rng.integers(0 if parts else 1, max_n + 1))):
                st[int(rng.integers(0, m))] += 1
            parts.append(FockState(st))
        items.append((tuple(parts), float(rng.random() ** 3)))
    return items


def same_dist(got, ref, rtol):
    assert set(got) == set(ref)
    top = max(ref.values())
    assert all(abs(got[k] - ref[k]) <= rtol * top for k in ref)


@pytest.mark.parametrize("packed", [True, False])
@pytest.mark.parametrize("batched", [True, False])
@pytest.mark.parametrize("seed", range(4))
def test_probs_svd_host_logic(oracle, monkeypatch, packed, batched, seed):
    """Both recombinations: packed integer keys, and output ranks (states too wide to pack)."""
    import perceval_gb300.simulators as S
    if not packed:
        monkeypatch.setattr(S, "_PACKED_BITS", 0)
    m = 8
    U = random_unitary(m, seed=seed)
    items = mixture(m, 100 + seed, 40)  # holds repeated inputs, kept entry by entry
    assert len({k for k, _ in items}) < len(items)
    be = FakeStrong(oracle, U, batched)
    sim = Simulator(be)
    sim.set_min_detected_photons_filter(2 if seed % 2 else 0)
    sim.precision = 1e-2 if seed >= 2 else 1e-6  # 1e-2: the merge cuts many branches
    out = sim.probs_svd(items)
    ref, phys, logical = ref_probs_svd(oracle_dist(oracle, U), items, precision=sim.precision,
                                       min_photons=sim.min_detected_photons_filter)
    same_dist(out["results"], ref, 1e-13)
    assert math.isclose(out["physical_perf"], phys, rel_tol=1e-13, abs_tol=1e-15)
    assert math.isclose(out["logical_perf"], logical, rel_tol=1e-12)
    assert math.isclose(sum(out["results"].values()), 1.0, rel_tol=1e-12)
    if batched:
        assert be.batched_calls == 1


def test_probs_svd_wide_states(oracle):
    """m = 40 with up to 3 photons: 40 modes x 2 bits do not pack into 64 bits, so the
    recombination runs on occupation rows; memory follows the outputs, not the Fock space."""
    m = 40
    U = random_unitary(m, seed=5)
    items = mixture(m, 7, 10, max_parts=3, max_n=1)
    sim = Simulator(FakeStrong(oracle, U, True))
    out = sim.probs_svd(items)
    ref, phys, logical = ref_probs_svd(oracle_dist(oracle, U), items)
    same_dist(out["results"], ref, 1e-13)
    assert math.isclose(out["logical_perf"], logical, rel_tol=1e-12)


def test_probs_svd_shortcut_and_thresholds(oracle):
    m = 5
    U = random_unitary(m, seed=9)
    sim = Simulator(FakeStrong(oracle, U, True))
    single = sim.probs(FockState([1, 1, 0, 0, 0]))
    ref = {FockState(r): p for r, p in zip(fock_space_array(m, 2), oracle.slos(U, [1, 1, 0, 0, 0])[0]) if p >= MIN_P}
    same_dist(single, {k: v / sum(ref.values()) for k, v in ref.items()}, 1e-14)
    # an input at or below max_p x precision is dropped before simulation
    items = [((FockState([1, 0, 0, 0, 0]),), 1.0), ((FockState([0, 0, 0, 0, 2]),), 1e-7)]
    out = sim.probs_svd(items)["results"]
    assert all(k.n == 1 for k in out)
    sim.precision = 1e-8
    assert any(k.n == 2 for k in sim.probs_svd(items)["results"])


class FakeSampler:
    """Sampling backend whose samples encode (input state, sample counter): the batched and
    the looped pools must match sample for sample."""

    def __init__(self, batched):
        self.counter = 0
        self._input_state = None
        if batched:
            self.samples_many = self._samples_many

    def _draw(self, st, count, first):
        return [FockState([first + i] + list(st)) for i in range(count)]

    def set_input_state(self, s):
        self._input_state = FockState(s)

    def samples(self, count):
        out = self._draw(self._input_state, count, self.counter)
        self.counter += count
        return out

    def _samples_many(self, states, counts):
        out, off = [], self.counter
        for st, c in zip(states, counts):
            out.append(self._draw(FockState(st), c, off))
            off += c
        self.counter = off
        return out


def test_samples_provider_batched_equals_loop():
    noisy = {(FockState([1, 0, 1]), FockState([0, 1, 0])): 0.6, FockState([1, 1, 0]): 0.3,
             FockState([0, 0, 0]): 0.1, (FockState([2, 0, 0]),): 0.05}
    pools = []
    for batched in (True, False):
        sp = SamplesProvider(FakeSampler(batched))
        sp.estimate_weights_from_distribution(noisy, 5000)
        sp.prepare()
        pools.append({k: list(v) for k, v in sp._pools.items()})
        assert sp._weights[FockState([1, 1, 0])] == math.ceil(0.1 * 1500)
        # a pool that runs empty draws min(weight, max) more through one backend call
        s = FockState([0, 1, 0])
        drawn = [sp.sample_from(s) for _ in range(len(sp._pools[s]) + 1)]
        assert drawn[0][1:] == s
    assert pools[0] == pools[1]
    assert pools[0][FockState([0, 0, 0])] == [FockState([0, 0, 0])] * 500
    assert len(pools[0][FockState([2, 0, 0])]) == 250


def test_samples_provider_weights_from_source():
    sp = SamplesProvider(FakeSampler(True))
    batch = [[FockState([1, 0]), FockState([0, 1])], [FockState([1, 0])]]
    assert sp.estimate_weights_from_source(lambda n: batch[:n], 2) == batch
    assert sp._weights[FockState([1, 0])] == 2 and sp._weights[FockState([0, 1])] == 1


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(3))
def test_probs_svd_slos_gpu(native, oracle, seed):
    from perceval_gb300 import NaiveBackend, SLOSBackend
    m = 8
    U = random_unitary(m, seed=20 + seed)
    items = mixture(m, 100 + seed, 40, max_parts=3, max_n=2)
    ref, phys, logical = ref_probs_svd(oracle_dist(oracle, U), items)
    for backend in (SLOSBackend(), NaiveBackend()):
        sim = Simulator(backend)
        sim.set_circuit(U)
        out = sim.probs_svd(items)
        same_dist(out["results"], ref, 1e-10)
        assert math.isclose(out["logical_perf"], logical, rel_tol=1e-10)


@pytest.mark.gpu
def test_probs_svd_clears_backend_mask(native, oracle):
    from perceval_gb300 import SLOSBackend
    m = 6
    U = random_unitary(m, seed=3)
    be = SLOSBackend()
    be.set_circuit(U)
    be.set_mask(["    00"])
    items = [((FockState([1, 0, 0, 1, 0, 0]), FockState([0, 1, 0, 0, 0, 0])), 0.7),
             ((FockState([0, 0, 1, 0, 0, 0]),), 0.3)]
    out = Simulator(be).probs_svd(items)["results"]
    ref, _, _ = ref_probs_svd(oracle_dist(oracle, U), items)
    same_dist(out, ref, 1e-10)


@pytest.mark.gpu
def test_samples_provider_cc2017_gpu(native):
    from perceval_gb300 import Clifford2017Backend
    from perceval_gb300.utils import random_seed
    m = 10
    U = random_unitary(m, seed=4)
    rng = np.random.default_rng(5)
    noisy = {}
    for _ in range(30):
        st = [0] * m
        for _ in range(int(rng.integers(1, 5))):
            st[int(rng.integers(0, m))] += 1
        noisy[FockState(st)] = float(rng.random())
    pools = []
    for batched in (True, False):
        random_seed(11)
        be = Clifford2017Backend()
        be.set_circuit(U)
        sp = SamplesProvider(be if batched else _LoopOnly(be))
        sp.estimate_weights_from_distribution(noisy, 3000)
        sp.prepare()
        pools.append({k: [tuple(x) for x in v] for k, v in sp._pools.items()})
    assert pools[0] == pools[1]
    assert all(sum(o) == k.n for k, v in pools[0].items() for o in v)


class _LoopOnly:
    """The sampler without its batched entry point (the reference's per-input loop)."""

    def __init__(self, be):
        self._be = be

    def set_input_state(self, s):
        self._be.set_input_state(s)

    def samples(self, count):
        return self._be.samples(count)
