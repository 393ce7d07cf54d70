"""GPU permanents against the FP64 oracle, the mpmath golden vectors and exact
identities, in every arithmetic (FP64 with exact row sums, the default; FP64 with FP64
row sums; float-float).
Tolerance: 1e-10 relative (|gpu - ref| <= 1e-10 |ref|) wherever the problem's own
conditioning allows it; the all-ones and equal-row cases state their rounding bound."""
import json
import math
from pathlib import Path

import numpy as np
import pytest
import torch

from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu
RTOL = 1e-10
PRECS = ["fp64", "fp64-dadd", "float-float"]
UNIT = {"fp64": 2.0 ** -53, "fp64-dadd": 2.0 ** -53, "float-float": 2.0 ** -47}  # unit roundoff


def pack(mats):
    sizes = np.array([m.shape[0] for m in mats], dtype=np.int32)
    offs = np.zeros(len(mats), dtype=np.int64)
    if len(mats) > 1:
        offs[1:] = np.cumsum([m.size for m in mats])[:-1]
    flat = np.concatenate([m.reshape(-1) for m in mats]) if mats else np.zeros(1, complex)
    return flat, offs, sizes


def gpu_perms(native, mats, method=0, prec="fp64"):
    flat, offs, sizes = pack(mats)
    dev = torch.from_numpy(flat).cuda()
    out = torch.empty(len(mats), dtype=torch.complex128, device="cuda")
    native.permanent_batch(dev, offs, sizes, out, method, precision=prec)
    return out.cpu().numpy()


def haar_submatrices(count, nmin, nmax, seed, big=1024):
    U = random_unitary(big, seed=0)
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        r = rng.choice(big, n, replace=False)
        c = rng.choice(big, n, replace=False)
        mats.append(np.ascontiguousarray(U[np.ix_(r, c)]))
    return mats


@pytest.mark.parametrize("prec", PRECS)
def test_golden_vectors(native, golden, prec):
    mats, refs = [], []
    for case in golden["permanents"]:
        n = case["n"]
        mats.append(np.array([complex(*v) for v in case["matrix"]]).reshape(n, n))
        refs.append(complex(float(case["perm"][0]), float(case["perm"][1])))
    for method in (0, 1):
        got = gpu_perms(native, mats, method, prec)
        for g, r in zip(got, refs):
            assert abs(g - r) <= RTOL * abs(r), (method, abs(g - r) / abs(r))
    if prec != "float-float":
        # FP64 precision: Glynn within 3e-14 of the 40-digit values (n <= 10), where the
        # oracle's own FP64 Glynn sum comes within 1e-14
        got = gpu_perms(native, mats, 0, prec)
        rel = max(abs(g - r) / abs(r) for g, r in zip(got, refs))
        assert rel <= 3e-14, rel


@pytest.mark.parametrize("prec", PRECS)
def test_edge_cases(native, prec):
    mats = [np.zeros((0, 0), complex), np.array([[2 - 1j]]), np.eye(5, dtype=complex), np.zeros((6, 6), complex),
            np.ones((7, 7), dtype=complex)]
    for method in (0, 1):
        got = gpu_perms(native, mats, method, prec)
        assert got[0] == 1 and got[1] == 2 - 1j
        assert abs(got[2] - 1) < 1e-14 and got[3] == 0
        assert abs(got[4] - math.factorial(7)) <= RTOL * math.factorial(7)
    assert len(gpu_perms(native, [], 0)) == 0


@pytest.mark.parametrize("prec", PRECS)
def test_batched_haar_vs_oracle(native, oracle, prec):
    mats = haar_submatrices(300, 1, 16, seed=1)
    flat, offs, sizes = pack(mats)
    ref = oracle.perm_batch(flat, offs, sizes)
    got = gpu_perms(native, mats, 0, prec)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel.max() <= RTOL, (rel.max(), sizes[rel.argmax()])
    # Ryser's alternating subset sum cancels more than Glynn's: float-float Ryser is
    # held to 1e-10 up to n = 12 and used as a looser cross-check above
    got = gpu_perms(native, mats, 1, prec)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel[sizes <= 12].max() <= RTOL
    assert rel.max() <= (1e-8 if prec == "float-float" else 1e-10)


@pytest.mark.parametrize("prec", PRECS)
def test_config_sizes_vs_oracle(native, oracle, prec):
    # the batched workload's size range, n uniform in 8..24 (subset checked on the CPU)
    mats = haar_submatrices(40, 8, 24, seed=2)
    flat, offs, sizes = pack(mats)
    ref = oracle.perm_batch(flat, offs, sizes)
    got = gpu_perms(native, mats, 0, prec)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel.max() <= RTOL, (rel.max(), sizes[rel.argmax()])


@pytest.mark.parametrize("prec", PRECS)
def test_scale_up_sizes_vs_oracle(native, oracle, prec):
    """n = 25..30, one seeded Haar submatrix each (the scale-up sizes of the plain
    permanent target), against the oracle's FP64 Glynn sum at 1e-10 (about 15 s of
    oracle time on 16 cores)."""
    mats = [haar_submatrices(1, n, n, seed=100 + n)[0] for n in range(25, 31)]
    flat, offs, sizes = pack(mats)
    ref = oracle.perm_batch(flat, offs, sizes)
    got = gpu_perms(native, mats, 0, prec)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel.max() <= RTOL, (rel, sizes)


@pytest.mark.parametrize("prec", PRECS)
def test_n32_against_committed_oracle_value(native, prec):
    """n = 32 against the oracle's Glynn sum committed by tests/golden/make_perm_fixtures.py
    (the oracle takes minutes there); Glynn at 1e-10, the GPU's Ryser within the
    Glynn-Ryser spread the oracle itself shows."""
    doc = json.loads((Path(__file__).parent / "golden" / "perm_large.json").read_text())
    for case in doc["cases"]:
        n = case["n"]
        a = np.array([complex(*v) for v in case["matrix"]]).reshape(n, n)
        ref = complex(*case["perm_glynn"])
        g = gpu_perms(native, [a], 0, prec)[0]
        assert abs(g - ref) <= RTOL * abs(ref), abs(g - ref) / abs(ref)
        if prec != "float-float":
            r = gpu_perms(native, [a], 1, prec)[0]
            assert abs(r - ref) <= 1e-6 * abs(ref)


@pytest.mark.parametrize("prec", PRECS)
def test_glynn_ryser_agree_large(native, prec):
    mats = haar_submatrices(4, 25, 28, seed=3)
    g = gpu_perms(native, mats, 0, prec)
    r = gpu_perms(native, mats, 1, prec)
    assert np.max(np.abs(g - r) / np.abs(g)) <= 1e-6


@pytest.mark.parametrize("prec", PRECS)
def test_rows_summing_to_one(native, oracle, prec):
    """Doubly stochastic matrices |U_ij|^2 of Haar unitaries: non-negative real rows whose
    l1 norm is 1 up to rounding, the case where the fixed-point scaling needs its margin
    below 2^62 (every Glynn row sum with all signs + equals the row's l1)."""
    rng = np.random.default_rng(13)
    mats = []
    for n in range(8, 21):
        U = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))[0]
        mats.append(np.ascontiguousarray(np.abs(U) ** 2).astype(complex))
    flat, offs, sizes = pack(mats)
    ref = oracle.perm_batch(flat, offs, sizes)
    got = gpu_perms(native, mats, 0, prec)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel.max() <= RTOL, (rel.max(), sizes[rel.argmax()])
    # Ryser's alternating subset sums of a positive matrix cancel from O(1) terms down to a
    # permanent near n!/n^n: sum |terms| / |perm| is 2.1e3 at n = 8, 2.3e5 at n = 12 and
    # 3.6e7 at n = 16 for these matrices, so Ryser is held to bounds with a tenfold margin
    # over the errors measured (FP64 9e-9, float-float 1.3e-6 at n = 20)
    got = gpu_perms(native, mats, 1, prec)
    rel = np.abs(got - ref) / np.abs(ref)
    ff = prec == "float-float"
    assert rel[sizes <= 12].max() <= (1e-7 if ff else 1e-9), rel[sizes <= 12].max()
    assert rel.max() <= (1e-5 if ff else 1e-7), (rel.max(), sizes[rel.argmax()])


def test_every_large_size_fp64_vs_float_float(native):
    """Sizes 31, 33, 34, 35, whose FP64 kernels (each size its own split of the product
    between the FP64 and integer pipes) no other test runs on Haar data: FP64 against the
    independent float-float kernel on one seeded submatrix each, at the float-float
    accuracy (about 20 s)."""
    for n in (31, 33, 34, 35):
        a = haar_submatrices(1, n, n, seed=200 + n)[0]
        f = gpu_perms(native, [a], 0, "fp64")[0]
        ff = gpu_perms(native, [a], 0, "float-float")[0]
        assert abs(f - ff) <= 1e-8 * abs(f), (n, f, ff)


def _abs_term_sum(r, ryser):
    """Exact sum of |term| over Glynn's sign vectors (delta_0 = +1) or Ryser's subsets for
    a matrix whose rows all equal the positive integer vector r (dynamic programme over
    the values of the row sum)."""
    counts = {r[0]: 1} if not ryser else {0: 1, r[0]: 1}
    for x in r[1:]:
        nxt = {}
        for s, c in counts.items():
            for v in ((s + x, s - x) if not ryser else (s, s + x)):
                nxt[v] = nxt.get(v, 0) + c
        counts = nxt
    n = len(r)
    return sum(c * abs(s) ** n for s, c in counts.items())


# (n, method, arithmetics): Ryser is conditioned like n^n / n! on these matrices, so it is
# checked only where its rounding bound stays small; FP64 n = 40 would take ~5 minutes
EQUAL_ROW_CASES = [(n, 0, p) for n in (20, 24, 28, 32) for p in PRECS] + \
                  [(36, 0, "fp64"), (36, 0, "float-float"), (40, 0, "float-float")] + \
                  [(n, 1, p) for n in (20, 24) for p in PRECS]


@pytest.mark.parametrize("n,method,prec", EQUAL_ROW_CASES)
def test_all_ones_and_equal_rows(native, n, method, prec):
    """Matrices whose rows are all equal to r * (3 + 4i), r a positive integer vector
    (all ones: the all-ones matrix J_n): perm = n! prod(r) (3 + 4i)^n exactly.  Their
    term magnitudes span the widest exponent range the row scaling must keep inside
    FP32 (float-float) and FP64.  The check is the rounding bound of the sum:
    |gpu - perm| <= max(1e-10, 16 n u cond) |perm|, with cond = sum |terms| / |sum|
    computed exactly (u: the arithmetic's unit roundoff; a term is a product of n row
    sums, each rounded, and float-float's lazy pairs lose about one more bit per
    operation than u).  At n = 40 in float-float the bound is 7e-6 relative."""
    rng = np.random.default_rng(1000 + n)
    for r in (np.ones(n, dtype=np.int64), rng.integers(1, 4, n)):
        a = np.tile(r.astype(float), (n, 1)) * (3 + 4j)
        exact_int = math.factorial(n) * math.prod(int(v) for v in r)
        gr, gi = 1, 0  # (3 + 4i)^n as a Gaussian integer
        for _ in range(n):
            gr, gi = 3 * gr - 4 * gi, 4 * gr + 3 * gi
        ref = complex(exact_int * gr, exact_int * gi)
        terms = _abs_term_sum([int(v) for v in r], method == 1)
        denom = exact_int * (2 ** (n - 1) if method == 0 else 1)
        cond = terms / denom
        tol = max(RTOL, 16 * n * UNIT[prec] * cond)
        got = gpu_perms(native, [np.ascontiguousarray(a)], method, prec)[0]
        assert np.isfinite(got.real) and np.isfinite(got.imag)
        assert abs(got - ref) <= tol * abs(ref), (abs(got - ref) / abs(ref), tol, cond)


@pytest.mark.parametrize("prec", PRECS)
def test_scaling_identities(native, prec):
    rng = np.random.default_rng(4)
    a = rng.normal(size=(12, 12)) + 1j * rng.normal(size=(12, 12))
    p = np.random.default_rng(5).permutation(12)
    d = np.exp(1j * rng.uniform(0, 6, 12)) * rng.uniform(0.5, 2, 12)
    got = gpu_perms(native, [a, a[p][:, ::-1].copy(), (a * d[:, None]).copy(), a.T.copy(), 1e-5 * a, 1e5 * a],
                    0, prec)
    assert abs(got[1] - got[0]) <= RTOL * abs(got[0])       # invariant under row/column permutations
    assert abs(got[2] - got[0] * np.prod(d)) <= RTOL * abs(got[2])  # multilinear in rows
    assert abs(got[3] - got[0]) <= RTOL * abs(got[0])       # transpose
    assert abs(got[4] - got[0] * 1e-60) <= RTOL * abs(got[4])
    assert abs(got[5] - got[0] * 1e60) <= RTOL * abs(got[5])


def test_bad_arguments_raise(native):
    dev = torch.zeros(4, dtype=torch.complex128, device="cuda")
    out = torch.empty(1, dtype=torch.complex128, device="cuda")
    with pytest.raises(RuntimeError, match="outside"):
        native.permanent_batch(torch.zeros(41 * 41, dtype=torch.complex128, device="cuda"), np.array([0]),
                               np.array([41]), out)
    with pytest.raises(ValueError):
        native.permanent_batch(dev, np.array([0]), np.array([3]), out)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("method", [0, 1])
def test_permuted_diagonal_identity(native, method, prec):
    """perm(P D) = prod of the nonzeros: every Glynn / Ryser term has the same magnitude,
    so the identity is checked at full precision up to n = 28."""
    rng = np.random.default_rng(7 + method)
    mats, refs = [], []
    for n in (5, 13, 20, 24, 28):
        d = np.exp(1j * rng.uniform(0, 2 * np.pi, n)) * rng.uniform(0.5, 1.5, n)
        perm = rng.permutation(n)
        a = np.zeros((n, n), complex)
        a[np.arange(n), perm] = d
        mats.append(a)
        refs.append(np.prod(d))
    got = gpu_perms(native, mats, method, prec)
    for g, r in zip(got, refs):
        assert abs(g - r) <= RTOL * abs(r)


@pytest.mark.parametrize("prec", PRECS)
def test_block_diagonal_identity(native, oracle, prec):
    """perm of a block-diagonal matrix = product of the blocks' permanents (n = 21 from
    Haar blocks of 6, 7 and 8, and n = 16 from two blocks of 8, with the rows and columns
    shuffled)."""
    rng = np.random.default_rng(3)
    mats, refs = [], []
    for sizes in ((6, 7, 8), (8, 8)):
        blocks = [haar_submatrices(1, s, s, seed=10 * s + i)[0] for i, s in enumerate(sizes)]
        n = sum(sizes)
        a = np.zeros((n, n), complex)
        o = 0
        for b in blocks:
            a[o:o + b.shape[0], o:o + b.shape[0]] = b
            o += b.shape[0]
        a = a[rng.permutation(n)][:, rng.permutation(n)]
        mats.append(np.ascontiguousarray(a))
        flat, offs, sz = pack(blocks)
        refs.append(np.prod(oracle.perm_batch(flat, offs, sz)))
    got = gpu_perms(native, mats, 0, prec)
    for g, r in zip(got, refs):
        assert abs(g - r) <= RTOL * abs(r)


def test_fixed_point_conversion_rounding(native):
    """The FP64 default converts each exact integer row sum to FP64 with integer operations:
    matrices whose row sums are exactly representable at every sign vector (dyadic
    entries) give exactly the same permanent in both FP64 kernels, and products of
    diagonal entries near the rounding boundary are rounded to nearest."""
    rng = np.random.default_rng(77)
    for n in (3, 9, 17):
        a = (rng.integers(-64, 65, (n, n)) + 1j * rng.integers(-64, 65, (n, n))) / 64.0
        fx = gpu_perms(native, [a], 0, "fp64")[0]
        dd = gpu_perms(native, [a], 0, "fp64-dadd")[0]
        assert abs(fx - dd) <= 1e-13 * abs(dd)
    d = 1.0 + np.array([2.0 ** -52, 3 * 2.0 ** -53, 2.0 ** -30, -2.0 ** -40])
    got = gpu_perms(native, [np.diag(d).astype(complex)], 0, "fp64")[0]
    assert abs(got - np.prod(d)) <= 4 * 2.0 ** -53
