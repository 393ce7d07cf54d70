"""The CPU oracle pinned against brute force, mpmath golden vectors and the
reference's known-answer tests (no GPU)."""
import math

import numpy as np
import pytest

from _circuits import build
from perceval_gb300.utils import FockState, fock_space_array, fock_rank, fock_unrank
from perceval_gb300.utils.matrix import random_unitary


def test_perm_vs_brute(oracle):
    rng = np.random.default_rng(1)
    for n in range(0, 8):
        a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        ref = oracle.perm_brute(a) if n else 1.0
        for method in ("glynn", "ryser"):
            assert abs(oracle.perm(a, method) - ref) <= 1e-12 * max(1.0, abs(ref))


def test_perm_golden(oracle, golden):
    for case in golden["permanents"]:
        n = case["n"]
        a = np.array([complex(*v) for v in case["matrix"]]).reshape(n, n)
        ref = complex(float(case["perm"][0]), float(case["perm"][1]))
        for method in ("glynn", "ryser"):
            assert abs(oracle.perm(a, method) - ref) <= 1e-12 * abs(ref), (n, case["kind"], method)


def test_slos_golden(oracle, golden):
    for case in golden["slos"]:
        m = case["m"]
        U = np.array([complex(*v) for v in case["unitary"]]).reshape(m, m)
        # the fixture's unitary is the seeded recipe's (to rounding: LAPACK's QR differs in
        # the last bits between builds and machines)
        assert np.allclose(U, random_unitary(m, seed=case["unitary_seed"]), atol=1e-14, rtol=0)
        ref = np.array([complex(float(a), float(b)) for a, b in case["amplitudes"]])
        _, amps = oracle.slos(U, case["input"])
        assert np.max(np.abs(amps - ref)) <= 1e-13
        assert [list(s) for s in fock_space_array(m, sum(case["input"]))] == case["states"]


def test_slos_vs_brute(oracle):
    U = random_unitary(5, seed=3)
    for inp in [(1, 1, 1, 0, 0), (2, 0, 1, 0, 0), (0, 3, 0, 0, 1), (0, 0, 0, 0, 0)]:
        p, a = oracle.slos(U, inp)
        pb, ab = oracle.slos_brute(U, inp)
        assert np.max(np.abs(a - ab)) < 1e-13
        assert abs(p.sum() - 1) < 1e-13


def test_slos_order_matches_path_decomposition(oracle):
    # _slos.py:61-86: max remaining count first, first index on ties
    assert oracle.slos_order((2, 0, 3)) == [2, 0, 2, 0, 2]
    assert oracle.slos_order((1, 1, 1, 0)) == [0, 1, 2]
    assert oracle.slos_order((0, 0)) == []


def test_ranks_roundtrip(oracle):
    for m, n in [(1, 3), (3, 2), (5, 3), (7, 4), (12, 6)]:
        arr = fock_space_array(m, n)
        assert arr.shape[0] == math.comb(m + n - 1, n)
        for r in range(0, arr.shape[0], max(1, arr.shape[0] // 97)):
            s = tuple(int(v) for v in arr[r])
            assert fock_rank(s) == r == oracle.fock_rank(s)
            assert fock_unrank(m, n, r) == FockState(s)
            assert oracle.fock_unrank(m, n, r) == s


def _dist(oracle, case):
    c = build(case["m"], case["ops"])
    probs, _ = oracle.slos(c.U, case["input"])
    states = fock_space_array(case["m"], sum(case["input"]))
    return {str(FockState(s)): p for s, p in zip(states, probs)}


def test_reference_kat_distributions(oracle, kats):
    for case in kats["distributions"]:
        d = _dist(oracle, case)
        for s, p in d.items():
            assert p == pytest.approx(case["expected"].get(s, 0.0), abs=1e-12), (case["source"], s)
        assert sum(d.values()) == pytest.approx(1.0)


def test_reference_kat_probabilities(oracle, kats):
    for group in kats["probabilities"]:
        c = build(group["m"], group["ops"])
        for inp, out, p in group["cases"]:
            _, amps = oracle.slos(c.U, inp)
            assert abs(amps[fock_rank(out)]) ** 2 == pytest.approx(p, abs=1e-12), group["source"]


def test_reference_kat_heralded_and_masked(oracle, kats):
    for case in kats["heralded_mass"]:
        d = _dist(oracle, case)
        mass = sum(p for s, p in d.items() if any(FockState(s)[k] for k in case["modes"]))
        assert mass == pytest.approx(case["expected"])
    case = kats["masked"][0]
    d = _dist(oracle, case)
    kept = {s: p for s, p in d.items() if FockState(s)[4] == 0 and FockState(s)[5] == 0 and p > 1e-16}
    assert kept == pytest.approx(case["expected"])


def test_reference_kat_amplitude_and_evolve(oracle, kats):
    for case in kats["amplitudes"]:
        c = build(case["m"], case["ops"])
        _, amps = oracle.slos(c.U, case["input"])
        assert amps[fock_rank(case["output"])] == pytest.approx(complex(*case["expected"]))
        assert oracle.amplitude_brute(c.U, case["input"], case["output"]) == pytest.approx(complex(*case["expected"]))
    for case in kats["evolve"]:
        c = build(case["m"], case["ops"])
        _, amps = oracle.slos(c.U, case["input"])
        states = fock_space_array(case["m"], sum(case["input"]))
        got = {str(FockState(s)): a for s, a in zip(states, amps) if abs(a) > 1e-12}
        assert got.keys() == case["expected"].keys()
        for s, v in case["expected"].items():
            assert got[s] == pytest.approx(complex(*v))


def test_cc2017_oracle_statistics(oracle, kats):
    case = kats["sampling"][0]
    c = build(case["m"], case["ops"])
    out = oracle.cc2017(c.U, case["input"], case["samples"], seed=123)
    for o in case["outcomes"]:
        cnt = int(np.sum(np.all(out == np.array(FockState(o)), axis=1)))
        assert case["band"][0] * case["samples"] < cnt < case["band"][1] * case["samples"]


def test_cc2017_oracle_chi_square(oracle):
    from _stats import chi2_pvalue
    U = random_unitary(5, seed=5)
    inp = (1, 1, 1, 0, 0)
    probs, _ = oracle.slos(U, inp)
    N = 20000
    out = oracle.cc2017(U, inp, N, seed=7)
    idx = np.array([fock_rank(r) for r in out])
    counts = np.bincount(idx, minlength=len(probs))
    assert chi2_pvalue(counts, probs) > 0.01


def test_slos_grad_oracle_vs_finite_differences(oracle):
    U = random_unitary(4, seed=9)
    inp = (1, 1, 0, 1)
    rng = np.random.default_rng(3)
    w = rng.normal(size=math.comb(4 + 3 - 1, 3))
    g = oracle.slos_grad(U, inp, w)
    h = 1e-6
    for (i, j) in [(0, 0), (2, 3), (3, 1)]:
        for part, unit in ((0, 1.0), (1, 1j)):
            Up, Um = U.copy(), U.copy()
            Up[i, j] += h * unit
            Um[i, j] -= h * unit
            fd = (w @ oracle.slos(Up, inp)[0] - w @ oracle.slos(Um, inp)[0]) / (2 * h)
            got = g[i, j].real if part == 0 else g[i, j].imag
            assert got == pytest.approx(fd, rel=1e-6, abs=1e-9)


def test_philox_known_answer(oracle):
    # Known-answer vectors published with Random123 (Salmon et al. 2011) for
    # philox4x32-10: counter 0 / key 0, and counter all-ones / key all-ones.
    assert oracle.philox((0, 0, 0, 0), (0, 0)) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert oracle.philox((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)


def test_mlp_reference_gradient_finite_differences():
    # the float64 restatement of the proposal network, checked by central differences
    # (bf16 rounding switched off so the function is smooth)
    from oracle import mlp_ref
    rng = np.random.default_rng(0)
    m, n, D, H = 7, 3, 5, 6
    params = {"mode_emb": rng.normal(size=(m, D)), "pos_emb": rng.normal(size=(n, D)),
              "W": [rng.normal(size=(H, D)) / 2, rng.normal(size=(H, H)) / 2, rng.normal(size=(H, H)) / 2],
              "b": [rng.normal(size=H) * 0.1 for _ in range(3)], "Wo": rng.normal(size=(m, H)) / 2,
              "bo": rng.normal(size=m) * 0.1}
    seq = rng.integers(0, m, size=(4, n))
    saved = mlp_ref.bf16
    mlp_ref.bf16 = lambda x: np.asarray(x, dtype=np.float64)
    try:
        _, g = mlp_ref.forward_backward(params, seq)
        h = 1e-6
        for key, idx in (("Wo", (2, 3)), ("bo", (4,)), ("mode_emb", (1, 2)), ("pos_emb", (2, 1))):
            p = params[key]
            old = p[idx]
            p[idx] = old + h
            lp, _ = mlp_ref.forward_backward(params, seq)
            p[idx] = old - h
            lm, _ = mlp_ref.forward_backward(params, seq)
            p[idx] = old
            assert (lp - lm) / (2 * h) == pytest.approx(g[key][idx], rel=1e-5, abs=1e-8)
        for i in range(3):
            W = params["W"][i]
            old = W[1, 2]
            W[1, 2] = old + h
            lp, _ = mlp_ref.forward_backward(params, seq)
            W[1, 2] = old - h
            lm, _ = mlp_ref.forward_backward(params, seq)
            W[1, 2] = old
            assert (lp - lm) / (2 * h) == pytest.approx(g["W"][i][1, 2], rel=1e-5, abs=1e-8)
    finally:
        mlp_ref.bf16 = saved


def test_host_tuned_paths_equal_the_restatements(oracle):
    """The CPU baseline's batched Glynn, parallel sampler, SLOS and Gurvits estimates compute
    what the plain restatements compute: permanents to 1e-12 relative, samples one for one,
    SLOS outputs bit for bit and its gradient to 1e-12, estimates to 1e-13."""
    from perceval_gb300.utils.matrix import random_unitary
    U = random_unitary(64, seed=3)
    rng = np.random.default_rng(3)
    mats = [np.zeros((0, 0), complex)] + [np.ascontiguousarray(U[np.ix_(rng.choice(64, n, False),
                                                                          rng.choice(64, n, False))])
                                          for n in (1, 2, 3, 7, 12, 14)]
    sizes = np.array([a.shape[0] for a in mats], dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum([a.size for a in mats])[:-1]]).astype(np.int64)
    flat = np.concatenate([a.reshape(-1) for a in mats] + [np.zeros(1, complex)])
    ref = oracle.perm_batch(flat, offs, sizes)
    got = oracle.perm_batch_fast(flat, offs, sizes)
    assert got[0] == 1
    assert np.max(np.abs(got[1:] - ref[1:]) / np.abs(ref[1:])) < 1e-12
    V = random_unitary(12, seed=4)
    inp = [1, 0, 1, 1, 0, 0, 1, 0, 1, 0, 0, 0]
    assert np.array_equal(oracle.cc2017_fast(V, inp, 300, seed=5, first=7), oracle.cc2017(V, inp, 300, seed=5, first=7))
    # ten photons: steps k >= 6 take the vector-lane sub-permanents (two to sixteen blocks)
    V = random_unitary(24, seed=6)
    inp = [1] * 10 + [0] * 14
    assert np.array_equal(oracle.cc2017_fast(V, inp, 120, seed=8), oracle.cc2017(V, inp, 120, seed=8))
    # SLOS: the same sums per state (bit for bit), the gradient up to the order in which the
    # threads' shares of a column are added; ranges of 8192 states split the larger layers
    for m, inp in ((7, [0, 3, 0, 0, 1, 0, 2]), (12, [1] * 6 + [0] * 6), (16, [2, 1, 1, 0, 1, 1] + [0] * 10)):
        V = random_unitary(m, seed=m)
        p, a = oracle.slos(V, inp)
        pf, af = oracle.slos_fast(V, inp)
        assert np.array_equal(p, pf) and np.array_equal(a, af)
        w = np.random.default_rng(m).normal(size=len(p))
        g, gf = oracle.slos_grad(V, inp, w), oracle.slos_grad_fast(V, inp, w)
        assert np.max(np.abs(gf - g)) <= 1e-12 * np.max(np.abs(g))
    # Gurvits: the same draws, added in another order (both compensated)
    gm = [np.ascontiguousarray(U[np.ix_(rng.choice(64, n, False), rng.choice(64, n, False))]) for n in (1, 5, 20, 33)]
    firsts = [0, 7, 1000, 5]
    got = oracle.gurvits_batch_fast(gm, 1000, 9, firsts)
    ref = np.array([oracle.gurvits(a, 1000, seed=9, first=f) for a, f in zip(gm, firsts)])
    assert np.max(np.abs(got - ref)) <= 1e-13
