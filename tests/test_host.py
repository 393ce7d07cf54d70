"""Host-side logic: states, enumeration, masks, circuits, factory and error
behaviour of the backend API (no GPU)."""
import math

import numpy as np
import pytest
import torch

from _circuits import build
from perceval_gb300 import BackendFactory, BasicState, Circuit, StateVector
from perceval_gb300.backends import ABackend, AStrongSimulationBackend
from perceval_gb300.components import BS, PERM, PS, GenericInterferometer, Unitary, catalog
from perceval_gb300.components.mesh import clements_mesh_unitary, clements_mesh_phase_count
from perceval_gb300.utils import (BSCount, BSDistribution, FSMask, allstate_iterator, max_photon_state_iterator,
                                  random_seed, random_unitary)
from perceval_gb300.utils.matrix import is_unitary


def test_fock_state_basics():
    s = BasicState("|2,0,1>")
    assert s.m == 3 and s.n == 3 and s.prodnfact() == 2 and str(s) == "|2,0,1>"
    assert s == BasicState([2, 0, 1]) and hash(s) == hash(BasicState((2, 0, 1)))
    assert s[0] == 2 and list(s) == [2, 0, 1]
    sv = math.sqrt(2) / 2 * StateVector([1, 0]) + math.sqrt(2) / 2 * StateVector([0, 1])
    assert len(sv) == 2 and sv[BasicState([1, 0])] == pytest.approx(math.sqrt(2) / 2)
    with pytest.raises(ValueError):
        BasicState([1, -1])


def test_enumeration_order_reference():
    # tests/utils/test_statevector.py:430-438
    expected = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1],
                [2, 0, 0], [1, 1, 0], [1, 0, 1], [0, 2, 0], [0, 1, 1], [0, 0, 2]]
    assert [list(s) for s in max_photon_state_iterator(3, 2)] == expected
    # tests/utils/test_statevector.py:441-452
    it = list(allstate_iterator(BasicState([1, 0, 0, 0])))
    assert len(it) == 4 and set(it) == {BasicState(v) for v in ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1])}
    sv = StateVector([0] * 6) + StateVector([1] + [0] * 5) + StateVector([2] + [0] * 5)
    assert len(list(allstate_iterator(sv))) == 28


def test_mask_reference():
    # tests/utils/test_mask.py:32-45
    mask = FSMask(6, 4, ["    11"])
    assert mask.match(BasicState("|0,0,1,1,1,1>"))
    assert not mask.match(BasicState("|0,0,1,1,1,0>"), False)
    assert mask.match(BasicState("|0,0,1,1,1,0>"), True)
    mask = FSMask(6, 4, ["   011", "   110"])
    assert mask.match(BasicState("|0,0,1,0,1,1>"))
    assert mask.match(BasicState("|0,0,1,1,1,0>"))
    assert not mask.match(BasicState("|0,0,1,1,1,1>"))


def test_mask_layers_and_device_spec():
    """The vectorised partial / full matches agree with ``match`` on every layer; the
    kept layers are closed under removing a photon (what a masked SLOS plan relies on);
    the device encoding carries the digits, the at-least modes and the photon count."""
    from perceval_gb300.utils.states import fock_rank, fock_space_array, fock_unrank_array
    mask = FSMask(7, 4, ["   01 1", " 2   0 "], at_least_modes=[6])
    for k in range(6):
        arr = fock_space_array(7, k)
        part = mask.match_array(arr, partial=True)
        assert np.array_equal(part, [mask.match(BasicState(list(s)), True) for s in arr])
        assert np.array_equal(mask.match_array(arr), [mask.match(BasicState(list(s))) for s in arr])
        for s in arr[part]:
            for j in np.nonzero(s)[0]:
                p = s.copy()
                p[j] -= 1
                assert mask.match(BasicState(list(p)), True)
    assert np.array_equal(mask.accepts_space(fock_space_array(7, 4)), mask.match_array(fock_space_array(7, 4)))
    digits, bits, n = mask.device_spec()
    assert digits.tolist() == [[-1, -1, -1, 0, 1, -1, 1], [-1, 2, -1, -1, -1, 0, -1]]
    assert bits == 1 << 6 and n == 4
    ranks = np.array([0, 5, 17, 83, 209])
    arr = fock_unrank_array(7, 4, ranks)
    assert [fock_rank(list(s)) for s in arr] == ranks.tolist()
    assert np.array_equal(fock_unrank_array(7, 4, np.arange(210)), fock_space_array(7, 4))
    from perceval_gb300.utils.states import fock_rank_array
    for m, n in [(1, 0), (1, 3), (4, 0), (7, 4), (12, 6)]:
        assert np.array_equal(fock_rank_array(fock_space_array(m, n)), np.arange(math.comb(m + n - 1, n)))
    assert fock_rank_array(arr).tolist() == ranks.tolist()


def test_bsdistribution_and_counts():
    d = BSDistribution()
    d.add(BasicState([1, 0]), 0.25)
    d.add(BasicState([1, 0]), 0.25)
    d.add(BasicState([0, 1]), 1e-30)
    assert d[BasicState([1, 0])] == 0.5 and len(d) == 1
    c = BSCount()
    c[BasicState([1, 0])] += 2
    assert c[BasicState([1, 0])] == 2 and c[BasicState([0, 1])] == 0


def test_bs_conventions():
    # perceval/components/unitary_components.py:142-183
    r = math.sqrt(0.5)
    assert np.allclose(BS().U, [[r, 1j * r], [1j * r, r]])
    assert np.allclose(BS.H().U, [[r, r], [r, -r]])
    assert np.allclose(BS.Ry().U, [[r, -r], [r, r]])
    th = 1.1
    u = BS(theta=th, phi_tl=0.1, phi_bl=0.2, phi_tr=0.3, phi_br=0.4).U
    assert u[0, 0] == pytest.approx(np.exp(1j * 0.4) * math.cos(th / 2))
    assert u[0, 1] == pytest.approx(1j * np.exp(1j * 0.5) * math.sin(th / 2))
    assert u[1, 0] == pytest.approx(1j * np.exp(1j * 0.5) * math.sin(th / 2))
    assert u[1, 1] == pytest.approx(np.exp(1j * 0.6) * math.cos(th / 2))
    assert np.allclose(PS(0.3).U, [[np.exp(0.3j)]])
    p = PERM([2, 0, 1]).U
    assert p[2, 0] == 1 and p[0, 1] == 1 and p[1, 2] == 1


def test_circuit_composition_order():
    c = Circuit(3) // BS.H() // (1, PS(math.pi / 4)) // (1, BS.H())
    u1 = np.eye(3, dtype=complex)
    u1[0:2, 0:2] = BS.H().U
    u2 = np.eye(3, dtype=complex)
    u2[1, 1] = np.exp(1j * math.pi / 4)
    u3 = np.eye(3, dtype=complex)
    u3[1:3, 1:3] = BS.H().U
    assert np.allclose(c.U, u3 @ u2 @ u1)
    assert is_unitary(catalog["postprocessed cnot"].build_circuit().U)


def test_identity_mesh_and_parameters():
    gi = GenericInterferometer(16, catalog["mzi phase last"].generate)
    assert len(gi.get_parameters()) == 240 == clements_mesh_phase_count(16)
    gi6 = GenericInterferometer(6, catalog["mzi phase last"].generate)
    gi6.set_identity_mode()
    assert np.allclose(np.abs(gi6.U), np.eye(6), atol=1e-12)


def test_torch_mesh_matches_circuit():
    m = 6
    gi = GenericInterferometer(m, catalog["mzi phase last"].generate)
    rng = np.random.default_rng(0)
    phases = rng.uniform(0, 2 * math.pi, clements_mesh_phase_count(m))
    for p in gi.get_parameters():
        idx = int(p.name[5:])
        p.set_value(phases[2 * idx + (0 if p.name[4] == "a" else 1)])
    U = clements_mesh_unitary(torch.tensor(phases), m).numpy()
    assert np.allclose(U, gi.U, atol=1e-13)


def test_random_unitary_matches_reference_recipe():
    np.random.seed(0)
    u = np.random.randn(4, 4) + 1j * np.random.randn(4, 4)
    q, r = np.linalg.qr(u)
    ref = q @ np.diag(np.sign(np.diagonal(np.real(r))))
    assert np.array_equal(random_unitary(4, seed=0), ref)
    assert is_unitary(random_unitary(12, seed=0))


def test_factory_and_errors():
    assert set(BackendFactory.list()) == {"SLOS", "SLAP", "Naive", "NaiveApprox", "CliffordClifford2017"}
    assert BackendFactory.get_backend("nope").name == "SLOS"
    assert BackendFactory.get_backend().name == "SLOS"
    for name in ("SLOS", "SLAP", "Naive", "NaiveApprox", "CliffordClifford2017"):
        b = BackendFactory.get_backend(name)
        assert b.name == name
        # tests/backends/test_backends.py:106-113
        with pytest.raises(AssertionError):
            b.set_circuit(Circuit(2))
            b.set_input_state(BasicState([1, 1, 1]))
        with pytest.raises(AssertionError):
            BackendFactory.get_backend(name).set_input_state(BasicState([1, 0]))


def test_unitary_circuit_wrapping():
    b = BackendFactory.get_backend("Naive")
    u = random_unitary(3, seed=1)
    b.set_circuit(u)
    assert np.allclose(b._umat, u)
    with pytest.raises(AssertionError):
        Unitary(np.zeros((2, 3)))


def test_seed_reproducible_counters():
    from perceval_gb300.utils import _random
    random_seed(5)
    a = _random.take_samples(10)
    b = _random.take_samples(3)
    random_seed(5)
    assert _random.take_samples(10) == a and a == (5, 0) and b == (5, 10)


def test_counts_to_sorted_modes():
    """Occupation rows -> photon modes in ascending order (the keys of the exact empirical
    TVD), against a repeat of each mode by its count."""
    from perceval_gb300.learned import counts_to_sorted_modes
    rng = np.random.default_rng(3)
    for m, n in ((6, 3), (64, 8), (5, 9)):
        occ = np.array([np.bincount(rng.integers(0, m, n), minlength=m) for _ in range(200)], dtype=np.int32)
        got = counts_to_sorted_modes(torch.from_numpy(occ), n).numpy()
        want = np.array([np.repeat(np.arange(m), r) for r in occ])
        assert np.array_equal(got, want)


def test_exact_empirical_tvd_without_photons():
    """No photons: the vacuum is the only output, so any samples match the law exactly."""
    from perceval_gb300.learned import exact_empirical_tvd
    got = exact_empirical_tvd(np.eye(3, dtype=complex), [0, 0, 0], np.zeros((5, 0), dtype=np.int64))
    assert got == {"samples": 5, "distinct_outputs": 1, "observed_mass": 1.0, "tvd": 0.0}
