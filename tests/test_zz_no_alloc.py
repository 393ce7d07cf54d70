"""The allocation-free permanent entry point, called through the C ABI.

Some callers cannot call cudaMalloc (a plugin inside a host program whose memory pool
already holds the GPU, a latency-critical loop, a process whose allocations are frozen
after start-up); pcvl_permanent_batch_noalloc serves them from a fixed scratch array.
This file sorts last so that a run stopping at the first failure has run every other
test before it; it also passes alone in a fresh process.
"""
import numpy as np
import pytest
import torch

from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def batch(seed: int, count: int, nmax: int):
    U = random_unitary(512, seed=seed)
    rng = np.random.default_rng(seed)
    mats = [np.zeros((0, 0), complex), np.array([[0.5 - 0.25j]])]
    for _ in range(count):
        n = int(rng.integers(2, nmax + 1))
        mats.append(np.ascontiguousarray(U[np.ix_(rng.choice(512, n, False), rng.choice(512, n, False))]))
    sizes = np.array([a.shape[0] for a in mats], dtype=np.int32)
    offs = np.zeros(len(mats), dtype=np.int64)
    offs[1:] = np.cumsum([a.size for a in mats])[:-1]
    flat = torch.from_numpy(np.concatenate([a.reshape(-1) for a in mats])).cuda()
    return flat, offs, sizes


@pytest.mark.parametrize("prec", ["fp64", "float-float"])
def test_noalloc_matches_allocating_entry_point_on_two_calls(native, prec):
    # two calls in a row on different batches: the second must not see the first's scratch
    for seed, count, nmax in ((1, 300, 20), (2, 120, 24)):
        flat, offs, sizes = batch(seed, count, nmax)
        ref = torch.empty(len(sizes), dtype=torch.complex128, device="cuda")
        native.permanent_batch(flat, offs, sizes, ref, precision=prec)
        got = torch.full((len(sizes),), complex("nan"), dtype=torch.complex128, device="cuda")
        native.permanent_batch_noalloc(flat, offs, sizes, got, precision=prec)
        ref, got = ref.cpu().numpy(), got.cpu().numpy()
        assert got[0] == 1 and got[1] == 0.5 - 0.25j
        assert np.all(np.abs(got - ref) <= RTOL * np.abs(ref)), np.max(np.abs(got - ref) / np.abs(ref))


def test_noalloc_refuses_requests_beyond_its_limits(native):
    out = torch.empty(16385, dtype=torch.complex128, device="cuda")
    mats = torch.zeros(16385, dtype=torch.complex128, device="cuda")
    with pytest.raises(RuntimeError, match="maximum of 16384"):
        native.permanent_batch_noalloc(mats, np.arange(16385), np.ones(16385, np.int32), out)
    big = torch.zeros(40 * 40 * 2000, dtype=torch.complex128, device="cuda")
    with pytest.raises(RuntimeError, match="elements, more than the maximum"):
        native.permanent_batch_noalloc(big, np.arange(2000) * 1600, np.full(2000, 40, np.int32), out)


def test_noalloc_refuses_too_many_partial_sums(native):
    """Launch shapes tuned to many CTAs per SM give a single large matrix thousands of
    partial sums; one such matrix in each of the 14 sizes 27..40 passes the 2^17 limit
    and is refused before any device work."""
    sizes = np.arange(27, 41, dtype=np.int32)
    offs = np.zeros(len(sizes), dtype=np.int64)
    offs[1:] = np.cumsum(sizes.astype(np.int64) ** 2)[:-1]
    mats = torch.zeros(int((sizes.astype(np.int64) ** 2).sum()), dtype=torch.complex128, device="cuda")
    out = torch.empty(len(sizes), dtype=torch.complex128, device="cuda")
    try:
        for n in sizes:
            native.set_perm_tuning(0, int(n), 7, 64)
        with pytest.raises(RuntimeError, match="partial sums, more than the maximum"):
            native.permanent_batch_noalloc(mats, offs, sizes, out)
    finally:
        for n in sizes:
            native.set_perm_tuning(0, int(n))
