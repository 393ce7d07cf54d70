"""SLOS plans over many input states (one batched plan, one launch per photon layer
for every input of one photon count): probabilities, amplitudes and adjoint gradients of
every entry against the oracle at 1e-10 relative, with a shared unitary and with one
unitary per entry; the backend's many-input calls against its one-input calls."""
import math

import numpy as np
import pytest
import torch

from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu
RTOL = 1e-10

STATES_8_4 = [(1, 1, 1, 1, 0, 0, 0, 0), (0, 0, 0, 0, 1, 1, 1, 1), (2, 0, 1, 0, 0, 1, 0, 0), (0, 4, 0, 0, 0, 0, 0, 0),
              (1, 0, 0, 2, 0, 0, 0, 1), (0, 0, 0, 0, 0, 0, 2, 2)]


def close(a, b):
    return np.abs(a - b).max() <= RTOL * np.abs(b).max()


@pytest.mark.parametrize("shared", [True, False])
def test_multi_plan_against_oracle(native, oracle, shared):
    m = 8
    B = len(STATES_8_4)
    Us = np.stack([random_unitary(m, seed=3 if shared else 30 + b) for b in range(B)])
    plan = native.SlosPlan(m, np.array(STATES_8_4))
    assert plan.batch == B
    u = torch.from_numpy(Us[0] if shared else Us).cuda()
    plan.forward(u)
    p = plan.probabilities().cpu().numpy().reshape(-1, B)
    a = plan.amplitudes().cpu().numpy().reshape(-1, B)
    for b, s in enumerate(STATES_8_4):
        rp, ra = oracle.slos(Us[b], s)
        assert close(p[:, b], rp) and close(a[:, b], ra), s
        assert abs(p[:, b].sum() - 1) < 1e-12


def test_multi_plan_batches_beyond_one_warp(native, oracle):
    m, n = 6, 3
    rng = np.random.default_rng(0)
    states = []
    for _ in range(70):
        s = np.zeros(m, int)
        for mode in rng.integers(0, m, n):
            s[mode] += 1
        states.append(tuple(s))
    U = random_unitary(m, seed=9)
    plan = native.SlosPlan(m, np.array(states))
    plan.forward(torch.from_numpy(U).cuda())
    p = plan.probabilities().cpu().numpy().reshape(-1, len(states))
    for b in (0, 31, 32, 69):
        assert close(p[:, b], oracle.slos(U, states[b])[0])


def test_multi_plan_gradients(native, oracle):
    m = 8
    B = len(STATES_8_4)
    Us = np.stack([random_unitary(m, seed=60 + b) for b in range(B)])
    count = math.comb(m + 3, 4)
    w = np.random.default_rng(2).normal(size=(count, B))
    plan = native.SlosPlan(m, np.array(STATES_8_4), keep_layers=True)
    plan.forward(torch.from_numpy(Us).cuda())
    plan.probabilities()
    g = plan.backward(torch.from_numpy(np.ascontiguousarray(w.reshape(-1))).cuda()).cpu().numpy()
    g = g.reshape(B, m, m)
    for b, s in enumerate(STATES_8_4):
        ref = oracle.slos_grad(Us[b], s, w[:, b])
        assert np.abs(g[b] - ref).max() <= RTOL * np.abs(ref).max(), s


def test_mixed_photon_counts_are_refused(native):
    with pytest.raises(RuntimeError, match="photon count"):
        native.SlosPlan(4, np.array([(1, 1, 0, 0), (1, 0, 0, 0)]))


def test_backend_many_inputs(native):
    from perceval_gb300 import BackendFactory, BasicState
    U = random_unitary(8, seed=5)
    states = [BasicState(list(s)) for s in STATES_8_4] + [BasicState([1, 0, 1, 0, 0, 0, 0, 0]),
                                                          BasicState([0, 0, 0, 1, 0, 0, 0, 0])]
    b = BackendFactory.get_backend("SLOS")
    b.set_circuit(U)
    many = b.all_probs_many(states)
    dists = b.prob_distributions(states[:2])
    for s, p in zip(states, many):
        b.set_input_state(s)
        one = np.asarray(b.all_prob())
        assert p.shape == one.shape and np.abs(p - one).max() <= 1e-13
    b.set_input_state(states[0])
    ref = b.prob_distribution()
    assert set(dists[0].keys()) == set(ref.keys())
    assert max(abs(dists[0][k] - ref[k]) for k in ref.keys()) <= 1e-13
    # a mask applies to every input's outputs
    b.set_mask("1       ")
    masked = b.all_probs_many(states[:3])
    for s, p in zip(states[:3], masked):
        b.set_input_state(s)
        assert np.abs(p - np.asarray(b.all_prob())).max() <= 1e-13
