"""SLOS adjoint: GPU dL/dU against the oracle's reverse sweep, central finite
differences (h = 1e-6) and float64 torch autograd through dense permanents; the chain
rule to the phases of a Clements mesh of MZIs, both by hand and through the
torch.autograd.Function; in both arithmetics (FP64, the default, and float-float)."""
import itertools
import math

import numpy as np
import pytest
import torch

from perceval_gb300.components.mesh import clements_mesh_phase_count, clements_mesh_unitary
from perceval_gb300.utils import fock_space_array
from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu


PRECS = ["fp64", "float-float"]


def gpu_grad(native, Us, inp, w, prec="fp64"):
    B, m = Us.shape[0], Us.shape[1]
    plan = native.SlosPlan(m, inp, batch=B, keep_layers=True, precision=prec)
    plan.forward(torch.from_numpy(np.ascontiguousarray(Us)).cuda())
    p = plan.probabilities().cpu().numpy().reshape(-1, B)
    g = plan.backward(torch.from_numpy(np.ascontiguousarray(w.reshape(-1))).cuda()).cpu().numpy()
    return p, g.reshape(B, m, m)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("B", [1, 3, 40])
def test_grad_vs_oracle(native, oracle, B, prec):
    m, inp = 6, (1, 0, 2, 1, 0, 0)
    Us = np.stack([random_unitary(m, seed=50 + b) for b in range(B)])
    count = math.comb(m + 4 - 1, 4)
    w = np.random.default_rng(1).normal(size=(count, B))
    p, g = gpu_grad(native, Us, inp, w, prec)
    for b in {0, B // 2, B - 1}:
        ref = oracle.slos_grad(Us[b], inp, w[:, b])
        assert np.abs(g[b] - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("prec", PRECS)
def test_grad_batched_m20_partial_chunk(native, oracle, prec):
    """m = 20 (the 24-mode kernels), 17 circuits: a full and a partial chunk of 16."""
    m, inp = 20, (1, 0, 1, 0, 0, 2) + (0,) * 14
    B = 17
    Us = np.stack([random_unitary(m, seed=80 + b) for b in range(B)])
    count = math.comb(m + 4 - 1, 4)
    w = np.random.default_rng(3).normal(size=(count, B))
    p, g = gpu_grad(native, Us, inp, w, prec)
    for b in (0, 8, 15, 16):
        ref = oracle.slos_grad(Us[b], inp, w[:, b])
        assert np.abs(g[b] - ref).max() <= 1e-10 * np.abs(ref).max()


def perm_torch(a):
    n = a.shape[0]
    tot = torch.zeros((), dtype=a.dtype)
    for S in range(1, 1 << n):
        cols = [j for j in range(n) if S >> j & 1]
        tot = tot + (-1) ** len(cols) * torch.prod(a[:, cols].sum(dim=1))
    return (-1) ** n * tot


@pytest.mark.parametrize("prec", PRECS)
def test_grad_vs_torch_dense_permanent(native, prec):
    m, inp = 4, (1, 1, 0, 1)
    U = random_unitary(m, seed=8)
    states = fock_space_array(m, 3)
    w = np.random.default_rng(2).normal(size=len(states))
    Ut = torch.tensor(U, dtype=torch.complex128, requires_grad=True)
    cols = [i for i, v in enumerate(inp) for _ in range(v)]
    L = torch.zeros((), dtype=torch.float64)
    for s, ws in zip(states, w):
        rows = [j for j, v in enumerate(s) for _ in range(v)]
        f = math.prod(math.factorial(int(v)) for v in s)
        L = L + ws * perm_torch(Ut[rows][:, cols]).abs() ** 2 / f
    L.backward()
    _, g = gpu_grad(native, U[None], inp, w[:, None], prec)
    assert np.abs(g[0] - Ut.grad.numpy()).max() <= 1e-10 * np.abs(Ut.grad.numpy()).max()
    # the same through the autograd function (one unitary, unbatched)
    from perceval_gb300.autograd import slos_probabilities
    Ug = torch.tensor(U, dtype=torch.complex128, device="cuda", requires_grad=True)
    p = slos_probabilities(Ug, inp, precision=prec)
    (p * torch.from_numpy(w).cuda()).sum().backward()
    assert np.abs(Ug.grad.cpu().numpy() - Ut.grad.numpy()).max() <= 1e-10 * np.abs(Ut.grad.numpy()).max()


@pytest.mark.parametrize("prec", PRECS)
def test_mesh_phase_gradient_vs_finite_differences(native, prec):
    m, n = 6, 3
    inp = [1] * n + [0] * (m - n)
    K = clements_mesh_phase_count(m)
    B = 2
    phases = torch.tensor(np.random.default_rng(3).uniform(0, 2 * math.pi, (B, K)), requires_grad=True)
    count = math.comb(m + n - 1, n)
    w = np.random.default_rng(4).normal(size=(count, B))
    U = clements_mesh_unitary(phases, m)
    _, g = gpu_grad(native, U.detach().numpy(), inp, w, prec)
    U.backward(torch.from_numpy(g))
    dphi = phases.grad.numpy()
    # the autograd function end to end: phases -> U (torch) -> probabilities -> L
    from perceval_gb300.autograd import slos_probabilities
    ph2 = phases.detach().clone().cuda().requires_grad_(True)
    P = slos_probabilities(clements_mesh_unitary(ph2, m).contiguous(), inp, precision=prec)
    (P * torch.from_numpy(w).cuda()).sum().backward()
    assert np.allclose(ph2.grad.cpu().numpy(), dphi, rtol=1e-10, atol=1e-12)
    plan = native.SlosPlan(m, inp, batch=B, precision=prec)
    wd = torch.from_numpy(w.reshape(-1)).cuda()

    def loss(ph):
        Ux = clements_mesh_unitary(torch.from_numpy(ph), m).contiguous()
        plan.forward(Ux.cuda())
        return (plan.probabilities() * wd).reshape(count, B).sum(dim=0).cpu().numpy()

    h = 1e-6
    base = phases.detach().numpy()
    for k in (0, 7, K - 1):
        up, dn = base.copy(), base.copy()
        up[:, k] += h
        dn[:, k] -= h
        fd = (loss(up) - loss(dn)) / (2 * h)
        assert np.allclose(dphi[:, k], fd, rtol=1e-6, atol=1e-8)


@pytest.mark.parametrize("prec", PRECS)
def test_config_clements_m16_n8_batch(native, oracle, prec):
    # the gradient workload's shape on 8 circuits: m = 16, n = 8, 490,314 outputs
    m, n, B = 16, 8, 8
    K = clements_mesh_phase_count(m)
    phases = torch.tensor(np.random.default_rng(0).uniform(0, 2 * math.pi, (B, K)))
    U = clements_mesh_unitary(phases, m).numpy()
    count = math.comb(m + n - 1, n)
    w = np.random.default_rng(0).normal(size=(count, B))
    p, g = gpu_grad(native, U, [1] * n + [0] * (m - n), w, prec)
    assert np.abs(p.sum(axis=0) - 1).max() < 1e-11
    ref = oracle.slos_grad(U[3], [1] * n + [0] * (m - n), w[:, 3])
    assert np.abs(g[3] - ref).max() <= 1e-10 * np.abs(ref).max()
