"""Learned-proposal Metropolised independence sampler for boson sampling.

There is no counterpart in the reference; its exact sampler (Clifford & Clifford,
perceval/backends/_clifford2017.py) is both the fallback and the point of comparison here.

Target.  For n photons in input modes ``in`` and a unitary U, an output *sequence*
r = (r_1..r_n) of modes (one per photon, order kept) gets

    pi(r) = |Perm(U[r, in])|^2 / n!

so that the multiset of r has the boson-sampling probability |Perm|^2 / prod s!: every
ordering of a multiset is equally likely.  The permanent is the exact Glynn kernel in
native FP64 (permanent plans, pcvl_perm_plan_*), so the acceptance ratios are FP64
throughout.

Proposal.  An autoregressive network q(r) = prod_k q(r_k | r_<k): the input row of
step k is pos_emb[k] + sum_{l<k} mode_emb[r_l] (mode embedding dim D), followed by
three GELU layers of width H and a linear map to logits over the m modes.  Weights
are BF16 for the tensor-core GEMMs (pcvl_gemm_bf16, FP32 accumulation) with FP32
master copies updated by Adam; every forward, backward and update step runs in this
library's kernels.  The network is trained by maximum likelihood on exact samples
of the GPU Clifford & Clifford sampler, each given a uniformly random photon order
(a draw from pi).

Sampler.  Proposals are independent of the chain state, so a batch of P proposals
is drawn at once (network + pcvl_sample_step) and scored at once (P permanents);
the accept/reject scan with acceptance min(1, pi(r') q(r) / (pi(r) q(r'))) runs on
the host in FP64.  The stationary law is pi exactly, whatever the network.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native

BF16 = torch.bfloat16


def _init(shape, fan_in, gen) -> torch.Tensor:
    return (torch.randn(*shape, generator=gen, dtype=torch.float64) / math.sqrt(fan_in)).float()


class ProposalMLP:
    """Autoregressive proposal over output modes (see the module docstring)."""

    def __init__(self, m: int, n: int, D: int = 128, H: int = 512, layers: int = 3, seed: int = 0):
        _native.load()
        self.m, self.n, self.D, self.H, self.L = m, n, D, H, layers
        gen = torch.Generator().manual_seed(seed)
        dev = torch.device("cuda")
        self.mode_emb = (_init((m, D), 1.0, gen) * 0.1).to(dev)
        self.pos_emb = (_init((n, D), 1.0, gen) * 0.1).to(dev)
        dims = [D] + [H] * layers
        self.W = [_init((dims[i + 1], dims[i]), dims[i], gen).to(dev) for i in range(layers)]
        self.b = [torch.zeros(dims[i + 1], device=dev) for i in range(layers)]
        self.Wo = _init((m, H), H, gen).to(dev) * 0.5
        self.bo = torch.zeros(m, device=dev)
        self.params = [self.mode_emb, self.pos_emb] + self.W + self.b + [self.Wo, self.bo]
        self.Wb = [w.to(BF16) for w in self.W]
        self.Wob = self.Wo.to(BF16)
        self._adam = [(torch.zeros_like(p), torch.zeros_like(p)) for p in self.params]
        self._step = 0

    # ------------------------------------------------------------------ forward
    def _forward_rows(self, h0b: torch.Tensor, R: int, keep: bool):
        """Hidden stack and logits for R input rows (bf16 R x D)."""
        acts_b, pres = [h0b], []
        x = h0b
        for i in range(self.L):
            out_b = torch.empty(R, self.H, dtype=BF16, device="cuda")
            pre = torch.empty(R, self.H, device="cuda") if keep else None
            _native.gemm_bf16(x, self.Wb[i], R, self.H, x.shape[1], x.shape[1], x.shape[1], bias=self.b[i],
                              epilogue=2, Cb=out_b, Cpre=pre)
            acts_b.append(out_b)
            pres.append(pre)
            x = out_b
        logits = torch.empty(R, self.m, device="cuda")
        _native.gemm_bf16(x, self.Wob, R, self.m, self.H, self.H, self.H, bias=self.bo, epilogue=1, C=logits)
        return logits, acts_b, pres

    def logits(self, seq: torch.Tensor) -> torch.Tensor:
        """Logits of every step of every sequence (S*n x m, row s*n + k)."""
        S = seq.shape[0]
        h0 = torch.empty(S * self.n, self.D, dtype=BF16, device="cuda")
        _native.bag_embed(seq, S, self.n, -1, self.mode_emb, self.pos_emb, self.D, h0)
        return self._forward_rows(h0, S * self.n, False)[0]

    def log_q(self, seq: torch.Tensor) -> torch.Tensor:
        """log q(r) of each sequence (float64, on the device)."""
        S = seq.shape[0]
        lg = self.logits(seq)
        lp = torch.empty(S * self.n, device="cuda")
        _native.softmax_xent(lg, S * self.n, self.m, target=seq.reshape(-1), logp_target=lp)
        return lp.view(S, self.n).double().sum(dim=1)

    # ------------------------------------------------------------------ training
    def loss_and_grads(self, seq: torch.Tensor):
        """Mean negative log-likelihood per photon and the gradient of every parameter."""
        S, n, D, H, m = seq.shape[0], self.n, self.D, self.H, self.m
        R = S * n
        h0 = torch.empty(R, D, dtype=BF16, device="cuda")
        _native.bag_embed(seq, S, n, -1, self.mode_emb, self.pos_emb, D, h0)
        logits, acts_b, pres = self._forward_rows(h0, R, True)
        lp = torch.empty(R, device="cuda")
        dlog = torch.empty(R, m, device="cuda")
        dlog_b = torch.empty(R, m, dtype=BF16, device="cuda")
        _native.softmax_xent(logits, R, m, target=seq.reshape(-1), scale=1.0 / R, logp_target=lp, grad=dlog,
                             gradb=dlog_b)
        loss = -float(lp.double().mean())
        grads = {}
        # output layer
        gWo = torch.empty(m, H, device="cuda")
        _native.gemm_bf16(dlog_b, acts_b[-1], m, H, R, m, H, transA=1, transB=1, C=gWo)
        gbo = torch.empty(m, device="cuda")
        _native.colsum(dlog, R, m, m, gbo)
        da = torch.empty(R, H, device="cuda")
        _native.gemm_bf16(dlog_b, self.Wob, R, H, m, m, H, transB=1, C=da)
        gW, gb = [None] * self.L, [None] * self.L
        for i in range(self.L - 1, -1, -1):
            dz = torch.empty(R, H, device="cuda")
            dz_b = torch.empty(R, H, dtype=BF16, device="cuda")
            _native.gelu_backward(da, pres[i], out=dz, outb=dz_b)
            fan_in = acts_b[i].shape[1]
            gW[i] = torch.empty(H, fan_in, device="cuda")
            _native.gemm_bf16(dz_b, acts_b[i], H, fan_in, R, H, fan_in, transA=1, transB=1, C=gW[i])
            gb[i] = torch.empty(H, device="cuda")
            _native.colsum(dz, R, H, H, gb[i])
            da = torch.empty(R, fan_in, device="cuda")
            _native.gemm_bf16(dz_b, self.Wb[i], R, fan_in, H, H, fan_in, transB=1, C=da)
        gmode = torch.zeros_like(self.mode_emb)
        gpos = torch.zeros_like(self.pos_emb)
        _native.bag_embed_backward(seq, S, n, da, D, gmode, gpos)
        return loss, [gmode, gpos] + gW + gb + [gWo, gbo]

    def adam_step(self, grads, lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        self._step += 1
        bf = [None, None] + self.Wb + [None] * self.L + [self.Wob, None]
        for p, g, (m1, m2), wb in zip(self.params, grads, self._adam, bf):
            _native.adam(p, g, m1, m2, lr, b1, b2, eps, self._step, wb)

    def _snapshot(self):
        return [p.clone() for p in self.params], [w.clone() for w in self.Wb], self.Wob.clone()

    def _restore(self, snap):
        ps, wbs, wob = snap
        for p, v in zip(self.params, ps):
            p.copy_(v)
        for w, v in zip(self.Wb, wbs):
            w.copy_(v)
        self.Wob.copy_(wob)

    def nll(self, samples: np.ndarray, seed: int = 0, batch: int = 1024) -> float:
        """Mean negative log-likelihood per photon of output samples (counts per mode),
        each given a uniformly random photon order."""
        seqs = np.stack(counts_to_sequences(samples, np.random.default_rng(seed))).astype(np.int32)
        tot = 0.0
        for i in range(0, len(seqs), batch):
            tot -= float(self.log_q(torch.from_numpy(seqs[i:i + batch]).cuda()).sum())
        return tot / (len(seqs) * self.n)

    def train(self, samples: np.ndarray, epochs: int = 5, batch: int = 256, lr: float = 1e-3, seed: int = 0,
              log=None, val: np.ndarray | None = None) -> list[float]:
        """Maximum likelihood on sequences made from output samples (counts per mode),
        each photon order drawn uniformly at random.  With held-out samples ``val`` the
        parameters of the epoch with the lowest held-out NLL are kept (the starting point
        counts as epoch 0), so training cannot leave the proposal worse on fresh samples
        than it found it; ``self.val_nll`` records the held-out NLL per epoch."""
        rng = np.random.default_rng(seed)
        seqs = counts_to_sequences(samples, rng)
        losses = []
        self.val_nll, self.best_epoch = [], 0
        best = None
        if val is not None:
            self.val_nll.append(self.nll(val, seed=seed + 1))
            best = self._snapshot()
        for ep in range(epochs):
            order = rng.permutation(len(seqs))
            tot, cnt = 0.0, 0
            for i in range(0, len(seqs), batch):
                idx = order[i:i + batch]
                # fresh random photon order every epoch (the target is order-symmetric)
                sb = np.stack([rng.permutation(seqs[j]) for j in idx]).astype(np.int32)
                loss, grads = self.loss_and_grads(torch.from_numpy(sb).cuda())
                self.adam_step(grads, lr=lr)
                tot += loss * len(idx)
                cnt += len(idx)
            losses.append(tot / cnt)
            if val is not None:
                self.val_nll.append(self.nll(val, seed=seed + 1))
                if self.val_nll[-1] < min(self.val_nll[:-1]):
                    best, self.best_epoch = self._snapshot(), ep + 1
            if log:
                log(f"epoch {ep}: nll/photon {losses[-1]:.4f}" +
                    (f", held-out {self.val_nll[-1]:.4f}" if val is not None else ""))
        if best is not None:
            self._restore(best)
        return losses

    # ------------------------------------------------------------------ sampling
    def sample(self, S: int, seed: int, chain0: int = 0) -> tuple[torch.Tensor, torch.Tensor]:
        """S sequences from q and their log q (float64), all on the device."""
        seq = torch.zeros(S, self.n, dtype=torch.int32, device="cuda")
        logq = torch.zeros(S, dtype=torch.float64, device="cuda")
        h0 = torch.empty(S, self.D, dtype=BF16, device="cuda")
        for k in range(self.n):
            _native.bag_embed(seq, S, self.n, k, self.mode_emb, self.pos_emb, self.D, h0)
            lg = self._forward_rows(h0, S, False)[0]
            _native.sample_step(lg, S, self.m, k, seed, chain0, seq, self.n, logq)
        return seq, logq


def counts_to_sequences(samples: np.ndarray, rng: np.random.Generator) -> list[np.ndarray]:
    """Output counts (N x m) -> mode sequences with a uniformly random photon order."""
    out = []
    for row in np.asarray(samples):
        s = np.repeat(np.arange(len(row)), row)
        out.append(rng.permutation(s))
    return out


def sequences_to_counts(seq: np.ndarray, m: int) -> np.ndarray:
    """Occupation counts (rows x m) of photon sequences (rows x n)."""
    seq = np.asarray(seq)
    rows = seq.reshape(-1, seq.shape[-1])
    out = np.zeros((rows.shape[0], m), dtype=np.int32)
    np.add.at(out, (np.repeat(np.arange(rows.shape[0]), rows.shape[1]), rows.reshape(-1).astype(np.int64)), 1)
    return out.reshape(seq.shape[:-1] + (m,))


_PERM_PLANS: dict = {}


def _perm_plan(S: int, n: int) -> "_native.PermPlan":
    """Cached permanent plan (one CUDA graph) for S packed n x n matrices: proposal
    batches repeat the same shape every round."""
    key = (S, n, torch.cuda.current_device())
    plan = _PERM_PLANS.get(key)
    if plan is None:
        if len(_PERM_PLANS) >= 8:
            _PERM_PLANS.pop(next(iter(_PERM_PLANS))).close()
        plan = _native.PermPlan(np.arange(S, dtype=np.int64) * n * n, np.full(S, n, np.int32), precision="fp64")
        _PERM_PLANS[key] = plan
    return plan


def log_abs_perm2(U_dev: torch.Tensor, cols: np.ndarray, seq: torch.Tensor) -> np.ndarray:
    """log |Perm(U[seq_s, cols])|^2 for every sequence (exact FP64 permanents)."""
    S, n = seq.shape
    colsd = torch.as_tensor(cols, dtype=torch.long, device=U_dev.device)
    mats = U_dev[seq.long()][:, :, colsd].contiguous()  # S x n x n
    out = _perm_plan(S, n)(mats.view(-1))
    a = out.abs().cpu().numpy()
    with np.errstate(divide="ignore"):
        return 2.0 * np.log(a)


def counts_to_sorted_modes(counts: torch.Tensor, n: int) -> torch.Tensor:
    """Photon modes in ascending order (rows x n, int64) of occupation counts (rows x m, on
    any device): photon p sits in the first mode whose cumulative count exceeds p."""
    cum = counts.to(torch.int64).cumsum(1)
    return torch.stack([(cum <= p).sum(1) for p in range(n)], dim=1)


def exact_empirical_tvd(U: np.ndarray, input_state, sequences: np.ndarray, chunk: int = 1 << 20) -> dict:
    """Exact total variation distance between the empirical distribution of sampled outputs
    (rows of photon modes, in any order) and the boson-sampling law
    p(s) = |Perm(U[s, t])|^2 / (prod s! prod t!), without enumerating the outputs: every
    observed output's p(s) from an exact FP64 permanent, the unobserved outputs' mass as
    1 - sum of the observed p(s), so TVD = (sum_observed |p(s) - f(s)| + 1 - sum_observed p(s)) / 2.
    Outputs are identified by their sorted modes packed into one int64 (n log2(m) <= 63 bits)."""
    m = U.shape[0]
    inp = np.asarray(input_state)
    n = int(inp.sum())
    bits = max(1, int(m - 1).bit_length())
    if bits * n > 63:
        raise ValueError("outputs do not fit a 63-bit key")
    if n == 0:  # the vacuum is the only output
        N = int(np.asarray(sequences).shape[0])
        return {"samples": N, "distinct_outputs": int(N > 0), "observed_mass": float(N > 0), "tvd": float(N == 0)}
    seq = np.sort(np.asarray(sequences).reshape(-1, n).astype(np.int64), axis=1)
    shifts = np.arange(n, dtype=np.int64) * bits
    keys = np.bitwise_or.reduce(seq << shifts, axis=1)
    uniq, counts = np.unique(keys, return_counts=True)
    N, D = seq.shape[0], len(uniq)
    modes = (uniq[:, None] >> shifts) & ((1 << bits) - 1)
    # prod s!: the product of the positions within each run of equal (sorted) modes
    run = np.ones(D, dtype=np.int64)
    sfact = np.ones(D)
    for j in range(1, n):
        run = np.where(modes[:, j] == modes[:, j - 1], run + 1, 1)
        sfact *= run
    tfact = float(np.prod([math.factorial(int(t)) for t in inp]))
    U_dev = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    V = U_dev[:, torch.as_tensor(np.repeat(np.arange(m), inp), dtype=torch.long, device=U_dev.device)]
    p = np.empty(D)
    for a in range(0, D, chunk):
        rows = torch.from_numpy(np.ascontiguousarray(modes[a:a + chunk])).to(U_dev.device)
        S = rows.shape[0]
        mats = V[rows].contiguous()  # S x n x n: rows = output modes, columns = input photons
        out = torch.empty(S, dtype=torch.complex128, device=U_dev.device)
        _native.permanent_batch(mats.view(-1), np.arange(S, dtype=np.int64) * n * n, np.full(S, n, np.int32), out)
        p[a:a + S] = (out.abs() ** 2).cpu().numpy()
    p /= sfact * tfact
    seen = float(p.sum())
    tvd = 0.5 * (float(np.abs(p - counts / N).sum()) + max(0.0, 1.0 - seen))
    return {"samples": int(N), "distinct_outputs": int(D), "observed_mass": seen, "tvd": tvd}


@dataclass
class MISResult:
    sequences: np.ndarray          # chain states as photon sequences, chains x steps x n
    m: int
    accept_rate: float
    proposals: int
    seconds: float
    log_pi: np.ndarray = field(default_factory=lambda: np.zeros(0))

    @property
    def samples(self) -> np.ndarray:
        """Chain states as occupation counts, chains x steps x m."""
        return sequences_to_counts(self.sequences, self.m)


def run_mis(proposal: ProposalMLP, U: np.ndarray, input_state, chains: int, steps: int, seed: int = 0,
            batch: int = 512) -> MISResult:
    """Independent-proposal Metropolis-Hastings chains targeting pi (exact law)."""
    import time
    m = U.shape[0]
    cols = np.repeat(np.arange(m), np.asarray(input_state))
    U_dev = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    total = chains * (steps + 1)
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    seqs, logq, logpi = [], [], []
    for start in range(0, total, batch):
        cnt = min(batch, total - start)
        s, lq = proposal.sample(cnt, seed, chain0=start)
        seqs.append(s.cpu().numpy())
        logq.append(lq.cpu().numpy())
        logpi.append(log_abs_perm2(U_dev, cols, s))
    torch.cuda.synchronize()
    seq = np.concatenate(seqs).reshape(chains, steps + 1, -1)
    lq = np.concatenate(logq).reshape(chains, steps + 1)
    lp = np.concatenate(logpi).reshape(chains, steps + 1)
    # the accept / reject scan, all chains at once (uniform u[c, t] in the order of a
    # chain-by-chain scan)
    u = np.log(rng.random((chains, steps)))
    lw = lp - lq
    cur = np.zeros(chains, dtype=np.int64)  # index of each chain's current proposal
    cur_lw = lw[:, 0].copy()
    state_idx = np.empty((chains, steps), dtype=np.int64)
    state_lp = np.empty((chains, steps))
    accepted = 0
    for t in range(steps):
        acc = u[:, t] < lw[:, t + 1] - cur_lw
        accepted += int(acc.sum())
        cur = np.where(acc, t + 1, cur)
        cur_lw = np.where(acc, lw[:, t + 1], cur_lw)
        state_idx[:, t] = cur
        state_lp[:, t] = cur_lw
    states = seq[np.arange(chains)[:, None], state_idx]
    secs = time.perf_counter() - t0
    return MISResult(states, m, accepted / (chains * steps), total, secs, state_lp)


def tvd_estimate(proposal: "ProposalMLP", U: np.ndarray, input_state, exact_counts: np.ndarray,
                 seed: int = 0) -> tuple[float, float]:
    """Total-variation distance between the proposal q and the target pi on photon
    sequences, TVD = E_{r ~ pi}[max(0, 1 - q(r) / pi(r))], estimated without bias from
    exact samples (counts) given a uniformly random photon order (a draw from pi); exact
    pi(r) = |Perm|^2 / n! from FP64 permanents.  Returns (estimate, standard
    error).  It bounds the distance between the two laws on output multisets from above."""
    rng = np.random.default_rng(seed)
    m = U.shape[0]
    n = int(np.sum(input_state))
    cols = np.repeat(np.arange(m), np.asarray(input_state))
    seqs = np.stack(counts_to_sequences(exact_counts, rng)).astype(np.int32)
    U_dev = torch.from_numpy(np.ascontiguousarray(U)).cuda()
    seq_d = torch.from_numpy(seqs).cuda()
    log_pi = log_abs_perm2(U_dev, cols, seq_d) - math.lgamma(n + 1)
    log_q = proposal.log_q(seq_d).cpu().numpy()
    with np.errstate(over="ignore"):
        v = np.maximum(0.0, 1.0 - np.exp(log_q - log_pi))
    return float(v.mean()), float(v.std(ddof=1) / math.sqrt(len(v)))


def ess(x: np.ndarray) -> float:
    """Effective sample size of one chain's scalar series (Geyer's initial positive
    sequence estimator of the integrated autocorrelation time)."""
    x = np.asarray(x, dtype=np.float64)
    N = len(x)
    if N < 4 or np.var(x) == 0:
        return float(N)
    xc = x - x.mean()
    f = np.fft.rfft(xc, n=2 * N)
    acf = np.fft.irfft(f * np.conj(f))[:N] / (np.arange(N, 0, -1))
    acf /= acf[0]
    tau = 1.0
    for t in range(1, N - 1, 2):
        pair = acf[t] + acf[t + 1]
        if pair <= 0:
            break
        tau += 2 * pair
    return N / tau


def exact_moments(U: np.ndarray, input_state) -> tuple[np.ndarray, np.ndarray]:
    """Exact E[n_i] and E[n_i n_j] of the output occupations for single-photon inputs:
    E[n_i] = A_i = sum_k |U_ik|^2 and, for i != j,
    E[n_i n_j] = A_i A_j + |sum_k conj(U_ik) U_jk|^2 - 2 sum_k |U_ik|^2 |U_jk|^2,
    E[n_i^2]  = A_i + 2 A_i^2 - 2 sum_k |U_ik|^4   (sums over occupied input modes k)."""
    inp = np.asarray(input_state)
    assert inp.max() <= 1, "closed forms are for single-photon inputs"
    V = np.asarray(U)[:, inp == 1]
    P = np.abs(V) ** 2
    A = P.sum(axis=1)
    G = V.conj() @ V.T
    E2 = np.outer(A, A) + np.abs(G) ** 2 - 2 * (P @ P.T)
    np.fill_diagonal(E2, A + 2 * A ** 2 - 2 * (P ** 2).sum(axis=1))
    return A, E2
