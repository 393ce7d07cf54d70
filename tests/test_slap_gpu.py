"""SLAP (depth-first walk over the outputs with 2^n photon-subset tables): every
probability and amplitude equals the oracle's SLOS at 1e-10 relative, from one photon to
twelve, with collision inputs, beyond the 32 modes of SLOS plans, and against oracle
permanents at m = 300; the device mask selection equals ``FSMask.accepts_space``; the
backend under ``BackendFactory.get_backend("SLAP")`` follows the reference API."""
import math

import numpy as np
import pytest
import torch

from perceval_gb300.utils import FSMask, FockState
from perceval_gb300.utils.matrix import random_unitary
from perceval_gb300.utils.states import fock_space_array, fock_unrank_array

pytestmark = pytest.mark.gpu
RTOL = 1e-10

CASES = [
    (4, (1, 0, 0, 0)),
    (5, (1, 1, 0, 0, 0)),
    (6, (2, 0, 1, 0, 0, 1)),
    (8, (1, 1, 1, 1, 0, 0, 0, 0)),
    (12, (1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0)),
    (7, (0, 3, 0, 2, 0, 0, 0)),
    (3, (4, 4, 4)),                     # 12 photons: one warp per CTA, 64 KB of subset table
    (40, (1, 1, 0, 1, 1) + (0,) * 35),  # beyond SLOS plans
    (33, (0,) * 32 + (2,)),
    # prefixes shorter than n - 1: the walk descends through interior levels
    (48, tuple(1 if i % 10 == 0 else 0 for i in range(48))),
    (16, (2, 0) + (1,) * 8 + (0,) * 6),
]


def close(a, b):
    return np.abs(a - b).max() <= RTOL * np.abs(b).max()


@pytest.mark.parametrize("m,inp", CASES, ids=[f"m{c[0]}_n{sum(c[1])}" for c in CASES])
def test_slap_against_oracle(native, oracle, m, inp):
    U = random_unitary(m, seed=m + 7)
    Ud = torch.from_numpy(U).cuda()
    rp, ra = oracle.slos(U, list(inp))
    assert native.slap_output_count(m, inp) == len(rp)
    p = native.slap_all(Ud, inp).cpu().numpy()
    a = native.slap_all(Ud, inp, amplitudes=True).cpu().numpy()
    assert close(p, rp) and close(a, ra)


def test_slap_equals_slos_plan(native):
    m, inp = 20, [1] * 6 + [0] * 14
    Ud = torch.from_numpy(random_unitary(m, seed=3)).cuda()
    plan = native.SlosPlan(m, inp)
    plan.forward(Ud)
    ref = plan.amplitudes().cpu().numpy()
    got = native.slap_all(Ud, inp, amplitudes=True).cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    assert abs(native.slap_all(Ud, inp).sum().item() - 1) < 1e-12


def test_slap_large_m_against_permanents(native, oracle):
    """m = 300, n = 3: 4,545,100 outputs; 64 of them against oracle permanents, and the
    unitarity sum rule over all of them."""
    m, n = 300, 3
    inp = np.zeros(m, dtype=np.int32)
    inp[[5, 77, 200]] = 1
    U = random_unitary(m, seed=1)
    a = native.slap_all(torch.from_numpy(U).cuda(), inp, amplitudes=True)
    assert a.numel() == math.comb(m + n - 1, n)
    assert abs(float((a.abs() ** 2).sum()) - 1) < 1e-12
    ranks = np.random.default_rng(0).choice(a.numel(), 64, replace=False)
    outs = fock_unrank_array(m, n, ranks)
    cols = np.repeat(np.arange(m), inp)
    mats = [U[np.ix_(np.repeat(np.arange(m), o), cols)] for o in outs]
    flat = np.concatenate([x.reshape(-1) for x in mats])
    perms = oracle.perm_batch(flat, np.arange(64) * n * n, np.full(64, n))
    norms = np.sqrt([math.prod(math.factorial(v) for v in o) for o in outs])
    ref = perms / norms
    got = a.cpu().numpy()[ranks]
    assert np.abs(got - ref).max() <= RTOL * np.abs(ref).max()


def test_slap_vacuum(native):
    p = native.slap_all(torch.from_numpy(random_unitary(3, seed=0)).cuda(), [0, 0, 0])
    assert p.cpu().numpy().tolist() == [1.0]


@pytest.mark.parametrize("m,n,masks,at_least,mask_n", [
    (6, 2, ["    00"], None, 2),
    (9, 4, ["*****1***", "*****0**1"], [8], 5),
    (40, 3, ["1" + "*" * 39, "*" * 38 + "00"], None, 3),
])
def test_fock_mask_ranks(native, m, n, masks, at_least, mask_n):
    mask = FSMask(m, mask_n, masks, at_least)
    got = native.fock_mask_ranks(m, n, mask).cpu().numpy()
    ref = np.nonzero(mask.accepts_space(fock_space_array(m, n)))[0]
    assert np.array_equal(got, ref)


def test_slap_backend_api(native, oracle):
    from perceval_gb300 import BackendFactory
    m = 6
    U = random_unitary(m, seed=4)
    b = BackendFactory.get_backend("SLAP")
    assert b.name == "SLAP"
    b.set_circuit(U)
    inp = FockState([1, 0, 1, 0, 1, 0])
    b.set_input_state(inp)
    rp, ra = oracle.slos(U, list(inp))
    assert close(np.array(b.all_prob()), rp)
    s = FockState([0, 1, 0, 1, 0, 1])
    idx = [tuple(r) for r in fock_space_array(m, 3)].index(tuple(s))
    assert abs(b.prob_amplitude(s) - ra[idx]) <= RTOL
    assert len(b.evolve()) == len(rp)
    b.set_mask(["    00"])
    sel = np.nonzero(FSMask(m, 3, ["    00"]).accepts_space(fock_space_array(m, 3)))[0]
    bsd = b.prob_distribution()
    assert [tuple(k) for k in bsd.keys()] == [tuple(r) for r in fock_space_array(m, 3)[sel]]
    assert close(np.array(list(bsd.values())), rp[sel])
    with pytest.raises(AssertionError):
        b.prob_amplitude(FockState([0, 0, 0, 1, 1, 1]))
    assert not b.can_simulate_feed_forward([], inp)


@pytest.mark.parametrize("seed", range(16))
def test_slap_random_against_oracle(native, oracle, seed):
    """Seeded random sizes (both walk endings: m >= 16 n and below) and inputs with
    collisions: probabilities and amplitudes equal the oracle's SLOS at 1e-10."""
    rng = np.random.default_rng(2000 + seed)
    if seed % 2:  # few modes: the sibling-batch ending
        n = int(rng.integers(1, 7))
        m = int(rng.integers(2, 20))
    else:  # many modes per photon: the one-node ending
        n = int(rng.integers(1, 4))
        m = int(rng.integers(16 * n, 16 * n + 20))
    inp = np.zeros(m, dtype=np.int32)
    for _ in range(n):
        inp[rng.integers(0, m)] += 1
    U = random_unitary(m, seed=seed)
    Ud = torch.from_numpy(U).cuda()
    rp, ra = oracle.slos(U, [int(v) for v in inp])
    assert close(native.slap_all(Ud, inp).cpu().numpy(), rp)
    assert close(native.slap_all(Ud, inp, amplitudes=True).cpu().numpy(), ra)
