"""The reference's backend tests (tests/backends/test_backends.py) as known-answer
data, run through BackendFactory on the GPU backends."""
import math

import numpy as np
import pytest

from _circuits import build
from perceval_gb300 import BackendFactory, BasicState, BSCount, Circuit
from perceval_gb300.components import BS, catalog
from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu
STRONG = ["SLOS", "SLAP", "Naive"]


def check_output_distribution(backend, input_state, expected):
    # mirrors tests/backends/test_backends.py:70-81
    backend.set_input_state(input_state)
    probs = []
    for out, p in backend.prob_distribution().items():
        assert p == pytest.approx(expected.get(str(out), 0.0), abs=1e-12), str(out)
        probs.append(p)
    assert sum(probs) == pytest.approx(1)


@pytest.mark.parametrize("name", STRONG)
def test_kat_distributions(native, kats, name):
    for case in kats["distributions"]:
        b = BackendFactory.get_backend(name)
        b.set_circuit(build(case["m"], case["ops"]))
        check_output_distribution(b, BasicState(case["input"]), case["expected"])


@pytest.mark.parametrize("name", STRONG)
def test_kat_cnot(native, kats, name):
    for group in kats["probabilities"]:
        b = BackendFactory.get_backend(name)
        b.set_circuit(build(group["m"], group["ops"]))
        for inp, out, p in group["cases"]:
            b.set_input_state(BasicState(inp))
            assert b.probability(BasicState(out)) == pytest.approx(p, abs=1e-12)
    case = kats["heralded_mass"][0]
    b = BackendFactory.get_backend(name)
    b.set_circuit(build(case["m"], case["ops"]))
    b.set_input_state(BasicState(case["input"]))
    mass = sum(p for s, p in b.prob_distribution().items() if any(s[k] for k in case["modes"]))
    assert mass == pytest.approx(case["expected"])


@pytest.mark.parametrize("name", STRONG)
def test_kat_masks(native, kats, name):
    case = kats["masked"][0]
    b = BackendFactory.get_backend(name)
    b.set_mask(case["mask"])
    b.set_circuit(build(case["m"], case["ops"]))
    b.set_input_state(BasicState(case["input"]))
    bsd = b.prob_distribution()
    assert len(bsd) == 2
    for s, p in case["expected"].items():
        assert bsd[BasicState(s)] == pytest.approx(p)
    case = kats["masked"][1]
    b = BackendFactory.get_backend(name)
    b.set_mask([case["mask"]])
    b.set_circuit(build(case["m"], case["ops"]))
    b.set_input_state(BasicState(case["input"]))
    mass = sum(p for s, p in b.prob_distribution().items() if any(s[k] for k in case["heralded_modes"]))
    assert mass == pytest.approx(case["heralded_expected"])


@pytest.mark.parametrize("name", STRONG)
def test_kat_amplitudes_and_evolve(native, kats, name):
    for case in kats["amplitudes"]:
        b = BackendFactory.get_backend(name)
        b.set_circuit(build(case["m"], case["ops"]))
        b.set_input_state(BasicState(case["input"]))
        assert b.prob_amplitude(BasicState(case["output"])) == pytest.approx(complex(*case["expected"]))
    for case in kats["evolve"]:
        b = BackendFactory.get_backend(name)
        b.set_circuit(build(case["m"], case["ops"]))
        b.set_input_state(BasicState(case["input"]))
        sv = b.evolve()
        sv.normalize()
        assert {str(k) for k in sv.keys()} == set(case["expected"])
        for s, v in case["expected"].items():
            assert sv[BasicState(s)] == pytest.approx(complex(*v))


def test_slos_refresh_coefs(native):
    # tests/backends/test_backends.py:252-277
    slos = BackendFactory.get_backend("SLOS")
    slos.set_circuit(BS())
    slos.set_input_state(BasicState("|1,1>"))
    slos.set_input_state(BasicState("|8,5>"))
    check_output_distribution(slos, BasicState("|1,1>"), {"|0,2>": 0.5, "|2,0>": 0.5})
    slos.set_circuit(Circuit(2))
    check_output_distribution(slos, BasicState("|1,1>"), {"|1,1>": 1.0})


def test_slos_equals_naive_on_random_circuit(native):
    U = random_unitary(7, seed=11)
    inp = BasicState([1, 0, 2, 0, 1, 0, 1])
    s, n = BackendFactory.get_backend("SLOS"), BackendFactory.get_backend("Naive")
    for b in (s, n):
        b.set_circuit(U)
        b.set_input_state(inp)
    ps, pn = np.array(s.all_prob()), np.array(n.all_prob())
    assert np.abs(ps - pn).max() <= 1e-10 * ps.max()
    out = BasicState([0, 2, 0, 1, 1, 1, 0])
    assert abs(s.prob_amplitude(out) - n.prob_amplitude(out)) <= 1e-10 * abs(n.prob_amplitude(out))
    assert s.prob_amplitude(BasicState([1] * 7)) == 0


@pytest.mark.parametrize("prec", ["fp64", "float-float"])
def test_naive_batched_collision_free_outputs(native, oracle, prec):
    # the small configuration's second half: Naive amplitudes of its 1000 random
    # collision-free outputs (6 of 12 modes, default_rng(0)), every one against the oracle
    U = random_unitary(12, seed=0)
    inp = BasicState([1] * 6 + [0] * 6)
    rng = np.random.default_rng(0)
    outs = []
    for _ in range(1000):
        o = np.zeros(12, dtype=int)
        o[rng.choice(12, 6, replace=False)] = 1
        outs.append(BasicState(o))
    b = BackendFactory.get_backend("Naive", precision=prec)
    b.set_circuit(U)
    b.set_input_state(inp)
    got = b.prob_amplitudes(outs)
    assert len(got) == 1000
    _, ref = oracle.slos(U, list(inp))
    from perceval_gb300.utils import fock_rank
    want = np.array([ref[fock_rank(o)] for o in outs])
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()


def test_clifford_bs_kat(native, kats):
    case = kats["sampling"][0]
    b = BackendFactory.get_backend("CliffordClifford2017")
    b.set_circuit(build(case["m"], case["ops"]))
    b.set_input_state(BasicState(case["input"]))
    counts = BSCount()
    for s in b.samples(case["samples"]):
        counts[s] += 1
    for o in case["outcomes"]:
        assert case["band"][0] * case["samples"] < counts[BasicState(o)] < case["band"][1] * case["samples"]
    assert isinstance(b.sample(), BasicState)


def test_api_surface_helpers(native, oracle):
    """preprocess (plans ahead, True when new), _compute_permanent (one matrix, through the
    batch call; NaiveApprox's is the estimate), IFFBackend on SLAP."""
    from perceval_gb300.backends import IFFBackend, NaiveApproxBackend, NaiveBackend, SLAPBackend, SLOSBackend
    from perceval_gb300.utils.matrix import random_unitary
    U = random_unitary(5, seed=3)
    b = SLOSBackend()
    b.set_circuit(U)
    assert b.preprocess([BasicState([1, 1, 0, 0, 0]), BasicState([0, 1, 0, 1, 0])]) is True
    assert b.preprocess([BasicState([1, 1, 0, 0, 0])]) is False
    b.set_input_state(BasicState([0, 1, 0, 1, 0]))
    rp, _ = oracle.slos(U, [0, 1, 0, 1, 0])
    assert np.allclose(b.all_prob(), rp, atol=1e-12)
    M = random_unitary(8, seed=1)[:6, :6]
    ref = oracle.perm_batch(M.reshape(-1).copy(), np.array([0]), np.array([6]))[0]
    assert abs(NaiveBackend()._compute_permanent(M) - ref) <= 1e-10 * abs(ref)
    est = NaiveApproxBackend(gurvits_iterations=200000)._compute_permanent(M)
    assert abs(est - ref) <= 0.05 * np.linalg.norm(M, 2) ** 6
    assert isinstance(SLAPBackend(), IFFBackend) and not isinstance(SLOSBackend(), IFFBackend)


def test_slos_backend_beyond_32_modes(native, oracle):
    """A 40-mode circuit on the SLOS backend (wider than SLOS plans): probabilities,
    amplitudes, a masked distribution and many inputs come from the SLAP walk and equal
    the oracle's SLOS."""
    from perceval_gb300.backends import SLOSBackend
    from perceval_gb300.utils import FSMask
    from perceval_gb300.utils.matrix import random_unitary
    from perceval_gb300.utils.states import fock_space_array
    m = 40
    U = random_unitary(m, seed=12)
    inp = BasicState([1, 0, 1, 0, 1] + [0] * 35)
    rp, ra = oracle.slos(U, list(inp))
    b = SLOSBackend()
    b.set_circuit(U)
    b.set_input_state(inp)
    assert np.abs(np.array(b.all_prob()) - rp).max() <= 1e-10 * rp.max()
    out = BasicState([0] * 37 + [1, 1, 1])
    idx = [tuple(r) for r in fock_space_array(m, 3)].index(tuple(out))
    assert abs(b.prob_amplitude(out) - ra[idx]) <= 1e-10 * np.abs(ra).max()
    many = b.all_probs_many([inp, BasicState([0, 2, 0, 0, 1] + [0] * 35)])
    assert np.abs(many[0] - rp).max() <= 1e-10 * rp.max()
    b.set_mask(["*" * 38 + "00"])
    sel = np.nonzero(FSMask(m, 3, ["*" * 38 + "00"]).accepts_space(fock_space_array(m, 3)))[0]
    assert np.abs(np.array(b.all_prob()) - rp[sel]).max() <= 1e-10 * rp.max()
    assert len(b.prob_distribution()) == len(sel)
