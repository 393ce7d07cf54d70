"""numpy float64 restatement of the proposal network.  TEST INFRASTRUCTURE ONLY.

Same architecture as perceval_gb300.learned.ProposalMLP (bag-of-modes + position
embedding, GELU layers, linear logits, mean NLL per photon).  GEMM inputs are rounded
to bfloat16 exactly where the GPU rounds them (embedding rows, activations, weights,
logit gradients, pre-activation gradients), and everything else is float64, so GPU
and reference differ only by FP32 accumulation and transcendental rounding.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float64 -> bfloat16 (round to nearest even) -> float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1 + erf(x / np.sqrt(2)))


def gelu_grad(x):
    return 0.5 * (1 + erf(x / np.sqrt(2))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)


def forward_backward(params: dict, seq: np.ndarray):
    """params: mode_emb (m,D), pos_emb (n,D), W[i] (out,in), b[i], Wo (m,H), bo.
    Returns (loss, grads dict with the same keys)."""
    S, n = seq.shape
    me, pe, W, b, Wo, bo = (params[k] for k in ("mode_emb", "pos_emb", "W", "b", "Wo", "bo"))
    D = me.shape[1]
    R = S * n
    h0 = np.zeros((R, D))
    for s in range(S):
        acc = np.zeros(D)
        for k in range(n):
            h0[s * n + k] = pe[k] + acc
            acc = acc + me[seq[s, k]]
    acts = [bf16(h0)]
    pres = []
    for Wi, bi in zip(W, b):
        z = acts[-1] @ bf16(Wi).T + bi
        pres.append(z)
        acts.append(bf16(gelu(z)))
    logits = acts[-1] @ bf16(Wo).T + bo
    mx = logits.max(axis=1, keepdims=True)
    lse = mx[:, 0] + np.log(np.exp(logits - mx).sum(axis=1))
    tgt = seq.reshape(-1)
    loss = -np.mean(logits[np.arange(R), tgt] - lse)
    p = np.exp(logits - lse[:, None])
    dlog = p.copy()
    dlog[np.arange(R), tgt] -= 1
    dlog /= R
    g = {"bo": dlog.sum(axis=0), "Wo": bf16(dlog).T @ acts[-1]}
    da = bf16(dlog) @ bf16(Wo)
    gW, gb = [None] * len(W), [None] * len(W)
    for i in range(len(W) - 1, -1, -1):
        dz = da * gelu_grad(pres[i])
        gb[i] = dz.sum(axis=0)
        gW[i] = bf16(dz).T @ acts[i]
        da = bf16(dz) @ bf16(W[i])
    g["W"], g["b"] = gW, gb
    gme, gpe = np.zeros_like(me), np.zeros_like(pe)
    for s in range(S):
        for k in range(n):
            gpe[k] += da[s * n + k]
            for l in range(k):
                gme[seq[s, l]] += da[s * n + k]
    g["mode_emb"], g["pos_emb"] = gme, gpe
    return loss, g
