"""Masked SLOS plans (every layer restricted to the states a mask can still accept):
the kept outputs are exactly the states ``FSMask.accepts_space`` selects from the full
space, and their probabilities, amplitudes and adjoint gradients equal the full-space
oracle's at 1e-10 relative, for one circuit, for batches of circuits, for several input
states per plan, with several masks, at-least modes, a mask built for more photons than
the input holds, masks that accept nothing and the vacuum.  Backend calls under
``set_mask`` use the masked plans."""
import numpy as np
import pytest
import torch

from perceval_gb300.utils import FSMask, FockState
from perceval_gb300.utils.matrix import random_unitary
from perceval_gb300.utils.states import fock_space_array

pytestmark = pytest.mark.gpu
RTOL = 1e-10

# (m, input state, mask strings, at-least modes, mask photon count or None)
CASES = [
    (8, (1, 1, 1, 1, 0, 0, 0, 0), ["******00"], None, None),
    (8, (1, 0, 1, 0, 1, 0, 1, 0), ["1 1     ", "0 2     "], None, None),
    (8, (2, 0, 1, 0, 0, 1, 0, 0), ["1*******"], [0], None),
    (9, (1, 1, 1, 0, 0, 0, 0, 0, 0), ["*****1***", "*****0**1"], [8], 4),
    (10, (1, 1, 1, 1, 1, 0, 0, 0, 0, 0), ["    10  01"], None, None),
    (12, (1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0), ["**********00", "0000********"], None, None),
    (6, (3, 0, 0, 0, 0, 0), ["   111"], None, None),
]


def kept_ranks(m, n, mask):
    return np.nonzero(mask.accepts_space(fock_space_array(m, n)))[0]


def close(a, b):
    scale = np.abs(b).max() if b.size else 1.0
    return a.shape == b.shape and (a.size == 0 or np.abs(a - b).max() <= RTOL * scale)


@pytest.mark.parametrize("prec", ["fp64", "float-float"])
@pytest.mark.parametrize("case", CASES, ids=[str(i) for i in range(len(CASES))])
def test_masked_plan_against_oracle(native, oracle, case, prec):
    m, inp, masks, at_least, mask_n = case
    n = sum(inp)
    mask = FSMask(m, mask_n or n, masks, at_least)
    U = random_unitary(m, seed=m + n)
    plan = native.SlosPlan(m, inp, mask=mask, precision=prec)
    sel = kept_ranks(m, n, mask)
    assert plan.count == len(sel)
    assert np.array_equal(plan.output_ranks().astype(np.int64), sel)
    plan.forward(torch.from_numpy(U).cuda())
    rp, ra = oracle.slos(U, inp)
    assert close(plan.probabilities().cpu().numpy(), rp[sel])
    assert close(plan.amplitudes().cpu().numpy(), ra[sel])


def test_masked_plan_is_smaller():
    """Six empty heralded modes of 16: 24,310 of 490,314 outputs kept; the masked plan
    (layers plus its parent tables) holds under a third of the full plan's memory."""
    from perceval_gb300 import _native
    m, inp = 16, (1,) * 8 + (0,) * 8
    mask = FSMask(m, 8, ["**********000000"])
    plan = _native.SlosPlan(m, inp, mask=mask)
    full = _native.SlosPlan(m, inp)
    assert plan.count == len(kept_ranks(m, 8, mask)) == 24310
    assert plan.device_bytes * 3 < full.device_bytes


@pytest.mark.parametrize("B", [3, 40])
def test_masked_batch_of_circuits(native, oracle, B):
    m, inp = 8, (1, 1, 0, 1, 0, 1, 0, 0)
    mask = FSMask(m, 4, ["****1**0", "****0**1"])
    Us = np.stack([random_unitary(m, seed=100 + b) for b in range(B)])
    plan = native.SlosPlan(m, inp, batch=B, mask=mask)
    plan.forward(torch.from_numpy(Us).cuda())
    p = plan.probabilities().cpu().numpy().reshape(-1, B)
    sel = kept_ranks(m, 4, mask)
    for b in (0, B // 2, B - 1):
        assert close(p[:, b], oracle.slos(Us[b], inp)[0][sel])


def test_masked_many_inputs(native, oracle):
    m = 8
    states = np.array([(1, 1, 1, 0, 0, 0, 0, 0), (0, 0, 0, 0, 0, 1, 1, 1), (2, 0, 0, 0, 1, 0, 0, 0)])
    mask = FSMask(m, 3, ["0*******", "1******0"])
    U = random_unitary(m, seed=5)
    plan = native.SlosPlan(m, states, mask=mask)
    plan.forward(torch.from_numpy(U).cuda())
    p = plan.probabilities().cpu().numpy().reshape(-1, len(states))
    sel = kept_ranks(m, 3, mask)
    for b, s in enumerate(states):
        assert close(p[:, b], oracle.slos(U, s)[0][sel])


@pytest.mark.parametrize("B", [1, 33])
def test_masked_adjoint(native, oracle, B):
    """dL/dU of L = sum over kept outputs of w p equals the full-space adjoint with the
    weights of every other output set to zero."""
    m, inp = 8, (1, 0, 1, 1, 0, 0, 1, 0)
    mask = FSMask(m, 4, ["*****00*", "******11"])
    sel = kept_ranks(m, 4, mask)
    Us = np.stack([random_unitary(m, seed=200 + b) for b in range(B)])
    plan = native.SlosPlan(m, inp, batch=B, keep_layers=True, mask=mask)
    plan.forward(torch.from_numpy(Us).cuda())
    w = np.random.default_rng(1).normal(size=(len(sel), B))
    g = plan.backward(torch.from_numpy(w.reshape(-1).copy()).cuda()).cpu().numpy().reshape(B, m, m)
    wf = np.zeros(len(fock_space_array(m, 4)))
    for b in (0, B - 1):
        wf[:] = 0
        wf[sel] = w[:, b]
        ref = oracle.slos_grad(Us[b], inp, wf)
        assert close(g[b], ref)


def test_mask_accepting_nothing_and_vacuum(native):
    plan = native.SlosPlan(6, (1, 1, 0, 0, 0, 0), mask=FSMask(6, 2, ["33****"]))
    assert plan.count == 0
    plan.forward(torch.from_numpy(random_unitary(6, seed=1)).cuda())
    assert plan.probabilities().numel() == 0
    vac = native.SlosPlan(4, (0, 0, 0, 0), mask=FSMask(4, 0, ["0***"]))
    assert vac.count == 1
    vac.forward(torch.from_numpy(random_unitary(4, seed=1)).cuda())
    assert vac.probabilities().cpu().numpy().tolist() == [1.0]
    assert native.SlosPlan(4, (0, 0, 0, 0), mask=FSMask(4, 0, ["1***"])).count == 0


def test_backend_uses_masked_plans(native, oracle):
    from perceval_gb300.backends import SLOSBackend
    m, inp = 10, FockState([1, 1, 1, 0, 1, 0, 0, 0, 0, 0])
    U = random_unitary(m, seed=11)
    b = SLOSBackend()
    b.set_circuit(U)
    b.set_mask(["********00", "*******1*0"])
    b.set_input_state(inp)
    entry = b._entries[inp]
    assert entry.plan.masked
    probs = np.array(b.all_prob())
    states = list(b.prob_distribution().keys())
    mask = FSMask(m, 4, ["********00", "*******1*0"])
    sel = kept_ranks(m, 4, mask)
    rp, ra = oracle.slos(U, list(inp))
    assert close(probs, rp[sel])
    assert [tuple(s) for s in states] == [tuple(r) for r in fock_space_array(m, 4)[sel]]
    s0 = states[len(states) // 2]
    assert abs(b.prob_amplitude(s0) - ra[sel][len(states) // 2]) <= RTOL
    with pytest.raises(AssertionError):
        b.prob_amplitude(FockState([0, 0, 0, 0, 0, 0, 1, 1, 1, 1]))
    sv = b.evolve()
    assert len(sv) == len(sel)
    b.clear_mask()
    assert len(b.all_prob()) == len(rp)


def _random_case(rng):
    m = int(rng.integers(3, 11))
    n = int(rng.integers(1, 6))
    inp = np.zeros(m, dtype=int)
    for _ in range(n):
        inp[rng.integers(0, m)] += 1
    nmask = int(rng.integers(1, 4))
    masks = ["".join(rng.choice(list("**  00112"), size=m)) for _ in range(nmask)]
    at_least = [int(i) for i in np.nonzero(rng.random(m) < 0.2)[0]]
    mask_n = n + int(rng.integers(0, 2))
    return m, tuple(int(v) for v in inp), masks, at_least, mask_n


@pytest.mark.parametrize("seed", range(24))
def test_random_masks_against_oracle(native, oracle, seed):
    """Seeded random masks (digits 0..2, '*' and spaces, several strings, at-least modes,
    a mask photon count of n or n + 1) on random inputs with collisions: the kept outputs
    and their probabilities equal the oracle's full distribution restricted by
    ``FSMask.accepts_space``."""
    rng = np.random.default_rng(1000 + seed)
    m, inp, masks, at_least, mask_n = _random_case(rng)
    n = sum(inp)
    mask = FSMask(m, mask_n, masks, at_least)
    sel = kept_ranks(m, n, mask)
    plan = native.SlosPlan(m, inp, mask=mask)
    assert plan.count == len(sel)
    if plan.count == 0:
        return
    assert np.array_equal(plan.output_ranks().astype(np.int64), sel)
    U = random_unitary(m, seed=seed)
    plan.forward(torch.from_numpy(U).cuda())
    rp, ra = oracle.slos(U, list(inp))
    assert close(plan.probabilities().cpu().numpy(), rp[sel])
    assert close(plan.amplitudes().cpu().numpy(), ra[sel])
