"""Learned-proposal sampler: BF16 tensor-core GEMM and network gradients against
references, exactness of the Metropolised sampler's law, and what training gains.

Tolerances: GEMM vs float64 products of the same bf16 inputs, 1e-5 relative (FP32
accumulation); network loss 1e-5 and gradients 2e-3 relative in norm against the
bf16-rounding float64 restatement; sampled laws chi-square p > 0.01."""
import math

import numpy as np
import pytest
import torch

from _stats import chi2_pvalue
from oracle import mlp_ref
from perceval_gb300.learned import ProposalMLP, ess, exact_moments, log_abs_perm2, run_mis
from perceval_gb300.utils import fock_rank
from perceval_gb300.utils.matrix import random_unitary

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,ta,tb,epi", [(200, 96, 64, 0, 0, 0), (130, 257, 100, 0, 0, 2), (64, 128, 300, 0, 1, 0),
                                             (96, 72, 333, 1, 1, 0), (1, 900, 512, 0, 0, 1),
                                             (512, 384, 1024, 0, 0, 0), (300, 200, 136, 0, 0, 2),
                                             # more tiles than SMs: every persistent CTA walks several
                                             # tiles through both accumulators and wraps the load ring
                                             (7680, 900, 512, 0, 0, 2), (4096, 1024, 1024, 0, 0, 0),
                                             # transposed operands by TMA (MN-major tiles): the
                                             # backward GEMMs' shapes, ragged edges in every dimension
                                             (7680, 512, 904, 0, 1, 0), (512, 904, 7680, 1, 0, 0),
                                             (1000, 520, 776, 1, 1, 2), (200, 136, 72, 1, 0, 1)])
def test_gemm_bf16(native, M, N, K, ta, tb, epi):
    g = torch.Generator().manual_seed(M + N + K)
    A = torch.randn(K, M, generator=g) if ta else torch.randn(M, K, generator=g)
    B = torch.randn(K, N, generator=g) if tb else torch.randn(N, K, generator=g)
    bias = torch.randn(N, generator=g)
    Ab, Bb = A.to(torch.bfloat16), B.to(torch.bfloat16)
    Ad, Bd = Ab.double(), Bb.double()
    ref = (Ad.T if ta else Ad) @ (Bd if tb else Bd.T)
    if epi:
        ref = ref + bias.double()
    pre = ref.clone()
    if epi == 2:
        ref = 0.5 * ref * (1 + torch.erf(ref / math.sqrt(2)))
    C = torch.empty(M, N, device="cuda")
    Cpre = torch.empty(M, N, device="cuda")
    native.gemm_bf16(Ab.cuda().contiguous(), Bb.cuda().contiguous(), M, N, K, M if ta else K, N if tb else K,
                     transA=ta, transB=tb, bias=bias.cuda(), epilogue=epi, C=C, Cpre=Cpre if epi == 2 else None)
    assert torch.allclose(C.cpu().double(), ref, rtol=1e-5, atol=1e-5 * ref.abs().max().item())
    if epi == 2:
        assert torch.allclose(Cpre.cpu().double(), pre, rtol=1e-5, atol=1e-5 * pre.abs().max().item())


def _params(net):
    return {"mode_emb": net.mode_emb.cpu().double().numpy(), "pos_emb": net.pos_emb.cpu().double().numpy(),
            "W": [w.cpu().double().numpy() for w in net.W], "b": [b.cpu().double().numpy() for b in net.b],
            "Wo": net.Wo.cpu().double().numpy(), "bo": net.bo.cpu().double().numpy()}


def test_network_gradients_vs_reference(native):
    m, n = 24, 5
    net = ProposalMLP(m, n, D=32, H=64, layers=3, seed=3)
    for p in net.b + [net.bo]:
        p.normal_(0, 0.1)
    rng = np.random.default_rng(0)
    seq = rng.integers(0, m, size=(37, n)).astype(np.int32)
    loss, grads = net.loss_and_grads(torch.from_numpy(seq).cuda())
    rloss, rg = mlp_ref.forward_backward(_params(net), seq)
    assert abs(loss - rloss) <= 1e-5 * abs(rloss)
    ref = [rg["mode_emb"], rg["pos_emb"]] + rg["W"] + rg["b"] + [rg["Wo"], rg["bo"]]
    for got, want in zip(grads, ref):
        got = got.cpu().double().numpy()
        assert np.linalg.norm(got - want) <= 2e-3 * np.linalg.norm(want) + 1e-12


def test_sampled_log_q_consistent(native):
    net = ProposalMLP(10, 4, D=16, H=32, layers=3, seed=1)
    seq, logq = net.sample(300, seed=7)
    again = net.log_q(seq)
    assert torch.allclose(logq, again, atol=1e-4)
    assert int(seq.min()) >= 0 and int(seq.max()) < 10


def test_mis_law_is_exact(native, oracle):
    # whatever the proposal (here untrained), the chain's multisets follow |Perm|^2 / prod s!
    m, n = 6, 3
    U = random_unitary(m, seed=4)
    inp = [1, 1, 1, 0, 0, 0]
    probs, _ = oracle.slos(U, inp)
    net = ProposalMLP(m, n, D=16, H=32, layers=3, seed=2)
    # one state per chain, after 200 steps: independent draws, the start (a draw from
    # the proposal) forgotten
    res = run_mis(net, U, inp, chains=3000, steps=200, seed=5, batch=8192)
    st = res.samples[:, -1]
    counts = np.bincount([fock_rank(s) for s in st], minlength=len(probs))
    assert chi2_pvalue(counts, probs) > 0.01
    assert 0 < res.accept_rate <= 1


def test_training_gains_over_untrained(native):
    # a proposal trained on exact samples accepts more and mixes faster than the same
    # network untrained, on the same unitary and budget
    m, n = 16, 4
    U = random_unitary(m, seed=8)
    inp = [1] * n + [0] * (m - n)
    Ud = torch.from_numpy(U).cuda()
    train = native.cc2017_sample(Ud, inp, 6000, seed=11).cpu().numpy()
    base = ProposalMLP(m, n, D=32, H=128, layers=3, seed=0)
    trained = ProposalMLP(m, n, D=32, H=128, layers=3, seed=0)
    losses = trained.train(train, epochs=8, batch=256, lr=2e-3)
    assert losses[-1] < losses[0]
    r0 = run_mis(base, U, inp, chains=64, steps=200, seed=1)
    r1 = run_mis(trained, U, inp, chains=64, steps=200, seed=1)
    e0 = np.mean([ess(x) for x in r0.log_pi])
    e1 = np.mean([ess(x) for x in r1.log_pi])
    assert r1.accept_rate > r0.accept_rate + 0.05
    assert e1 > e0


def test_exact_moments_match_slos(oracle):
    m, n = 6, 3
    U = random_unitary(m, seed=9)
    inp = [0, 1, 1, 0, 1, 0]
    probs, _ = oracle.slos(U, inp)
    states = np.array(oracle.fock_states(m, n))
    A, E2 = exact_moments(U, inp)
    assert np.allclose(A, probs @ states, atol=1e-12)
    assert np.allclose(E2, np.einsum("r,ri,rj->ij", probs, states, states), atol=1e-12)


def test_tvd_estimate_matches_enumeration(native, oracle):
    # m = 6, n = 3: all 216 photon sequences enumerated; the Monte-Carlo estimate from exact
    # samples agrees within 5 standard errors
    import itertools
    from perceval_gb300.learned import tvd_estimate
    m, inp = 6, [1, 0, 1, 0, 1, 0]
    U = random_unitary(m, seed=12)
    net = ProposalMLP(m, 3, D=16, H=32, layers=3, seed=2)
    seqs = np.array(list(itertools.product(range(m), repeat=3)), dtype=np.int32)
    cols = np.array([0, 2, 4])
    lp = log_abs_perm2(torch.from_numpy(U).cuda(), cols, torch.from_numpy(seqs).cuda()) - math.log(6)
    lq = net.log_q(torch.from_numpy(seqs).cuda()).cpu().numpy()
    exact = 0.5 * np.abs(np.exp(lp) - np.exp(lq)).sum()
    assert abs(np.exp(lp).sum() - 1) < 1e-12 and abs(np.exp(lq).sum() - 1) < 1e-5
    samples = oracle.cc2017(U, inp, 20000, seed=4)
    est, se = tvd_estimate(net, U, inp, samples, seed=1)
    assert abs(est - exact) < 5 * se + 1e-3, (est, se, exact)


@pytest.mark.parametrize("inp", [[1, 0, 1, 0, 1, 0], [2, 0, 1, 0, 0, 0]])
def test_exact_empirical_tvd_matches_enumeration(native, oracle, inp):
    # m = 6, n = 3: every output's probability from the oracle's SLOS; the empirical TVD of
    # GPU exact samples (sorted modes recovered from occupations on the device) computed
    # without enumeration equals the enumerated one, for a few and for many samples
    from perceval_gb300.learned import counts_to_sorted_modes, exact_empirical_tvd
    from perceval_gb300.utils.states import fock_rank_array
    m, n = 6, 3
    U = random_unitary(m, seed=13)
    p, _ = oracle.slos(U, inp)
    x = native.cc2017_sample(torch.from_numpy(U).cuda(), inp, 4000, seed=21)
    for N in (7, 4000):
        occ = x[:N].cpu().numpy()
        f = np.bincount(fock_rank_array(occ), minlength=len(p)) / N
        want = 0.5 * np.abs(p - f).sum()
        got = exact_empirical_tvd(U, inp, counts_to_sorted_modes(x[:N], n).cpu().numpy())
        assert got["samples"] == N and got["distinct_outputs"] == int((f > 0).sum())
        assert abs(got["tvd"] - want) < 1e-12, (got, want)
        assert abs(got["observed_mass"] - p[f > 0].sum()) < 1e-12


def test_early_stopping_keeps_the_best_epoch(native):
    # 200 samples, 12 epochs: the held-out NLL rises once the network memorises; training
    # keeps the epoch with the lowest held-out NLL, never worse than the start
    m, n = 24, 4
    U = random_unitary(m, seed=30)
    inp = [1] * n + [0] * (m - n)
    data = native.cc2017_sample(torch.from_numpy(U).cuda(), inp, 400, seed=31).cpu().numpy()
    net = ProposalMLP(m, n, D=32, H=256, layers=3, seed=1)
    net.train(data[:200], epochs=12, batch=32, lr=3e-3, val=data[200:], seed=4)
    assert len(net.val_nll) == 13
    assert net.val_nll[net.best_epoch] == min(net.val_nll) <= net.val_nll[0]
    assert abs(net.nll(data[200:], seed=5) - net.val_nll[net.best_epoch]) < 1e-5
