"""GPU permanents against the FP64 oracle, the mpmath golden vectors and exact
identities.  Tolerance: 1e-10 relative (|gpu - ref| <= 1e-10 |ref|)."""
import math

import numpy as np
import pytest
import torch

from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def pack(mats):
    sizes = np.array([m.shape[0] for m in mats], dtype=np.int32)
    offs = np.zeros(len(mats), dtype=np.int64)
    if len(mats) > 1:
        offs[1:] = np.cumsum([m.size for m in mats])[:-1]
    flat = np.concatenate([m.reshape(-1) for m in mats]) if mats else np.zeros(1, complex)
    return flat, offs, sizes


def gpu_perms(native, mats, method=0):
    flat, offs, sizes = pack(mats)
    dev = torch.from_numpy(flat).cuda()
    out = torch.empty(len(mats), dtype=torch.complex128, device="cuda")
    native.permanent_batch(dev, offs, sizes, out, method)
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


def test_golden_vectors(native, golden):
    mats, refs = [], []
    for case in golden["permanents"]:
        n = case["n"]
        mats.append(np.array([complex(*v) for v in case["matrix"]]).reshape(n, n))
        refs.append(complex(float(case["perm"][0]), float(case["perm"][1])))
    for method in (0, 1):
        got = gpu_perms(native, mats, method)
        for g, r in zip(got, refs):
            assert abs(g - r) <= RTOL * abs(r), (method, abs(g - r) / abs(r))


def test_edge_cases(native):
    mats = [np.zeros((0, 0), complex), np.array([[2 - 1j]]), np.eye(5, dtype=complex), np.zeros((6, 6), complex),
            np.ones((7, 7), dtype=complex)]
    for method in (0, 1):
        got = gpu_perms(native, mats, method)
        assert got[0] == 1 and got[1] == 2 - 1j
        assert abs(got[2] - 1) < 1e-14 and got[3] == 0
        assert abs(got[4] - math.factorial(7)) <= RTOL * math.factorial(7)
    assert len(gpu_perms(native, [], 0)) == 0


def test_batched_haar_vs_oracle(native, oracle):
    mats = haar_submatrices(300, 1, 16, seed=1)
    flat, offs, sizes = pack(mats)
    ref = oracle.perm_batch(flat, offs, sizes)
    got = gpu_perms(native, mats, 0)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel.max() <= RTOL, (rel.max(), sizes[rel.argmax()])
    # Ryser's alternating subset sum cancels more than Glynn's: float-float Ryser is
    # held to 1e-10 up to n = 12 and used as a looser cross-check above
    got = gpu_perms(native, mats, 1)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel[sizes <= 12].max() <= RTOL
    assert rel.max() <= 1e-8


def test_config_sizes_vs_oracle(native, oracle):
    # the batched workload's size range, n uniform in 8..24 (subset checked on the CPU)
    mats = haar_submatrices(40, 8, 24, seed=2)
    flat, offs, sizes = pack(mats)
    ref = oracle.perm_batch(flat, offs, sizes)
    got = gpu_perms(native, mats, 0)
    rel = np.abs(got - ref) / np.abs(ref)
    assert rel.max() <= RTOL, (rel.max(), sizes[rel.argmax()])


def test_glynn_ryser_agree_large(native):
    mats = haar_submatrices(4, 25, 28, seed=3)
    g = gpu_perms(native, mats, 0)
    r = gpu_perms(native, mats, 1)
    assert np.max(np.abs(g - r) / np.abs(g)) <= 1e-6


def test_scaling_identities(native):
    rng = np.random.default_rng(4)
    a = rng.normal(size=(12, 12)) + 1j * rng.normal(size=(12, 12))
    p = np.random.default_rng(5).permutation(12)
    d = np.exp(1j * rng.uniform(0, 6, 12)) * rng.uniform(0.5, 2, 12)
    got = gpu_perms(native, [a, a[p][:, ::-1].copy(), (a * d[:, None]).copy(), a.T.copy(), 1e-5 * a, 1e5 * a])
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


@pytest.mark.parametrize("method", [0, 1])
def test_permuted_diagonal_identity(native, method):
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
    got = gpu_perms(native, mats, method)
    for g, r in zip(got, refs):
        assert abs(g - r) <= RTOL * abs(r)


def test_block_diagonal_identity(native, oracle):
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
    got = gpu_perms(native, mats)
    for g, r in zip(got, refs):
        assert abs(g - r) <= RTOL * abs(r)
