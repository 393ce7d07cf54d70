"""The GPU backends under the reference's own caller sequences.

The reference's simulators cannot run here (its native library is absent), so these
tests replay, step for step, what two of its callers do with a backend and with the
states the backend returns, on this package's backends and state types:

* ``Simulator._probs_svd_fast`` (perceval/simulators/simulator.py:412-514): reset the
  backend's input, ``use_mask`` (``set_mask`` of a herald string, or ``clear_mask``,
  simulator.py:640-672), ``set_input_state`` and ``prob_iterator(threshold)`` once per
  distinct part, then the ``_list_merge`` recombination
  (perceval/simulators/_simulator_utils.py:148-171), which iterates each cached iterator
  several times and merges output states with ``FockState.merge``, and accumulation into
  a ``BSDistribution`` with ``res[bs] += p``;
* ``Stepper.apply`` (perceval/simulators/stepper.py:62-96): slices of the input states,
  ``set_circuit`` / ``set_input_state`` / ``prob_amplitude`` over ``allstate_iterator``,
  then ``state.set_slice(...) * amplitude`` accumulated into a ``StateVector`` iterated
  as (state, amplitude) pairs.

Each replay is compared with an independent computation from the CPU oracle.
"""
import math
from collections import defaultdict

import numpy as np
import pytest

from perceval_gb300 import BackendFactory
from perceval_gb300.utils import BSDistribution, FockState, StateVector
from perceval_gb300.utils.matrix import random_unitary
from perceval_gb300.utils.states import allstate_iterator, fock_space_array

pytestmark = pytest.mark.gpu


def list_merge(distributions, prob_threshold=0.0):
    """The recombination of perceval/simulators/_simulator_utils.py:148-171, step for step."""
    if len(distributions) == 0:
        return dict()
    res = defaultdict(float)

    def inner(dist, current_state, current_prob):
        if len(dist) == 0:
            res[current_state] += current_prob
            return
        for bs, p in dist[0]:
            prob = current_prob * p
            if prob < prob_threshold:
                continue
            inner(dist[1:], current_state.merge(bs), prob)

    for bs, p in distributions[0]:
        if p < prob_threshold:
            continue
        inner(distributions[1:], bs, p)
    return res


def replay_probs_svd_fast(backend, input_list, p_threshold, herald_mask=None):
    """Simulator._probs_svd_fast's calls on the backend for a list of
    (probability, [parts], photon count) inputs (simulator.py:431-513)."""
    decomposed_input = [(prob, states, sum(s.n for s in states)) for states, prob in input_list]
    cache = {}
    input_dict = defaultdict(float)
    for prob, states, n in decomposed_input:
        for state in states:
            key = (state, n)
            if prob > input_dict[key]:
                input_dict[key] = prob
    previous_n = None
    for (state, n), prob0 in sorted(input_dict.items(), key=lambda x: x[0][1]):
        if n != previous_n and n != 0:
            previous_n = n
            backend._input_state = None
            if herald_mask is not None:
                backend.set_mask(herald_mask, n)
            elif backend._masks_str is not None:
                backend.clear_mask()
        backend.set_input_state(state)
        cache[(state, n)] = backend.prob_iterator(p_threshold / (10 * prob0))
    res = BSDistribution()
    logical = 0.0
    for prob0, bs_data, n in decomposed_input:
        probs_in_s = list_merge([cache[(state, n)] for state in bs_data], prob_threshold=p_threshold / (10 * prob0))
        logical += sum(probs_in_s.values()) * prob0
        for bs, p in probs_in_s.items():
            res[bs] += p * prob0
    if len(res):
        res.normalize()
    return res, logical


def oracle_distribution(oracle, U, part):
    p, _ = oracle.slos(U, list(part))
    return {FockState(row): float(v) for row, v in zip(fock_space_array(U.shape[0], part.n), p)}


@pytest.mark.parametrize("backend_name", ["SLOS", "Naive"])
def test_probs_svd_fast_sequence(native, oracle, backend_name):
    """A mixture of separable inputs on m = 6: every output probability of the replayed
    recombination equals the oracle's convolution of the parts' distributions."""
    m = 6
    U = random_unitary(m, seed=21)
    a = FockState([1, 1, 0, 0, 0, 0])
    b = FockState([0, 0, 1, 0, 0, 0])
    c = FockState([0, 0, 0, 1, 0, 1])
    inputs = [([a.merge(b)], 0.5), ([a, b], 0.3), ([c, b], 0.2)]
    backend = BackendFactory.get_backend(backend_name)
    backend.set_circuit(U)
    got, logical = replay_probs_svd_fast(backend, inputs, p_threshold=1e-16)
    want = defaultdict(float)
    for parts, prob in inputs:
        dists = [oracle_distribution(oracle, U, s) for s in parts]
        acc = {FockState([0] * m): 1.0}
        for d in dists:
            nxt = defaultdict(float)
            for s1, p1 in acc.items():
                for s2, p2 in d.items():
                    nxt[s1.merge(s2)] += p1 * p2
            acc = nxt
        for s, p in acc.items():
            want[s] += prob * p
    tot = sum(want.values())
    assert abs(logical - 1.0) < 1e-12
    keys = {k for k, v in want.items() if v / tot > 1e-15}
    assert keys <= set(got.keys())
    assert max(abs(got.get(k, 0.0) - want[k] / tot) for k in want) < 1e-12


def test_probs_svd_fast_sequence_with_heralds(native, oracle):
    """The same replay with the simulator's herald mask (mode 5 detected empty,
    simulator.py:640-662): only the accepted outputs come back; the logical
    performance is their total probability."""
    m = 6
    U = random_unitary(m, seed=22)
    a, b = FockState([1, 0, 1, 0, 0, 0]), FockState([0, 1, 0, 0, 0, 0])
    backend = BackendFactory.get_backend("SLOS")
    backend.set_circuit(U)
    got, logical = replay_probs_svd_fast(backend, [([a, b], 1.0)], p_threshold=1e-16, herald_mask="     0")
    da, db = oracle_distribution(oracle, U, a), oracle_distribution(oracle, U, b)
    want = defaultdict(float)
    for s1, p1 in da.items():
        if s1[5]:
            continue
        for s2, p2 in db.items():
            if not s2[5]:
                want[s1.merge(s2)] += p1 * p2
    assert abs(logical - sum(want.values())) < 1e-12
    for k, v in want.items():
        assert abs(got[k] - v / logical) < 1e-12
    assert all(k[5] == 0 for k in got)


def replay_stepper_apply(backend, sv, r, U_c):
    """Stepper.apply (stepper.py:62-96) for one component on modes r, without the
    result cache's reuse across calls."""
    min_r, max_r = r[0], r[-1] + 1
    sub_input_state = {state[min_r:max_r] for state in sv.keys()}
    backend.set_circuit(U_c)
    mapping = {}
    for input_state in sub_input_state:
        backend.set_input_state(input_state)
        mapping[input_state] = {out: backend.prob_amplitude(out) for out in allstate_iterator(input_state)}
    nsv = StateVector()
    for state, sv_pa in sv:
        for output_state, prob_ampli in mapping[state[min_r:max_r]].items():
            nsv += state.set_slice(slice(min_r, max_r), output_state) * (prob_ampli * sv_pa)
    return nsv


@pytest.mark.parametrize("backend_name", ["SLOS", "Naive"])
def test_stepper_apply_sequence(native, oracle, backend_name):
    """A superposition of three 3-photon states on m = 5 through a 3-mode component on
    modes 1..3: the replayed StateVector equals the oracle's amplitudes through the
    embedded 5-mode unitary."""
    m = 5
    Uc = random_unitary(3, seed=23)
    U = np.eye(m, dtype=complex)
    U[1:4, 1:4] = Uc
    sv = (0.6 * StateVector([1, 1, 0, 1, 0]) + 0.48j * StateVector([0, 1, 1, 0, 1])
          + 0.64 * StateVector([1, 0, 2, 0, 0]))
    backend = BackendFactory.get_backend(backend_name)
    got = replay_stepper_apply(backend, sv, [1, 2, 3], Uc)
    want = defaultdict(complex)
    for state, amp in sv:
        _, amps = oracle.slos(U, list(state))
        for row, a in zip(fock_space_array(m, state.n), amps):
            want[FockState(row)] += amp * a
    for k, v in want.items():
        if abs(v) > 1e-14:
            assert abs(got.get(k, 0j) - v) < 1e-12, (k, got.get(k, 0j), v)
    assert abs(sum(abs(v) ** 2 for _, v in got) - 1.0) < 1e-12
