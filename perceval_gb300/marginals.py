"""Exact one- and two-mode marginal distributions of boson sampling outputs.

No counterpart in the reference; they measure a sampler's accuracy at sizes where the
full output distribution cannot be enumerated (n = 30 photons on m = 900 modes has
about 10^56 outputs).

Input: one photon in each of the modes t_1..t_n; V = U[:, t] (m x n, orthonormal
columns).  The probability generating function of the output occupations is a
permanent:

    E[prod_j z_j^{n_j}] = Perm(A(z)),   A(z)_{kl} = sum_j z_j conj(V_jk) V_jl,

since expanding Perm(A(z)) over output assignments gives sum_s |Perm(V_s)|^2 / s!
prod z^s.  With every z_j = 1 except z_i = x (and z_j = y), A = I + (x - 1) conj(v_i)
v_i^T (+ (y - 1) conj(v_j) v_j^T), v_i = row i of V: a rank-one (rank-two)
perturbation of the identity, whose permanent is a sum over principal submatrices.

One mode.  Perm(I + X c r^T) = sum_S X^|S| |S|! prod_{k in S} c_k r_k, so with
q_k = |V_ik|^2, G(x) = sum_t t! e_t(q) (x - 1)^t, e_t the elementary symmetric
polynomials, and P(n_i = a) = sum_{t >= a} t! e_t(q) C(t, a) (-1)^(t - a).

Two modes.  Perm(I + X a b^T + Y c d^T) with a = conj(v_i), b = v_i, c = conj(v_j),
d = v_j: a principal submatrix S contributes, for every split of its rows into T (the
X term) and S \\ T (the Y term) and of its columns into T' and S \\ T' with
|T'| = |T| = t, the weight t! (|S| - t)! prod over S of one of a_k b_k (k in T and T'),
a_k d_k (T, not T'), c_k b_k (not T, T'), c_k d_k (neither).  A dynamic programme over
the n photons with state (|T|, |S \\ T|, |T'|) sums these; then G(x, y) =
sum_{t,u} t! u! D[t, u, t] (x - 1)^t (y - 1)^u and the coefficients of x^a y^b are
P(n_i = a, n_j = b).

Arithmetic: the alternating binomial sums are taken in exact rational arithmetic
(Python fractions over the binary values of the float64 inputs) when ``exact=True``,
else in float64 (which suffices when the t! e_t terms decrease, as for n << m).
Pinned against brute-force enumeration at n <= 6 in the tests.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np


def _input_columns(U: np.ndarray, input_state) -> np.ndarray:
    inp = np.asarray(input_state)
    assert inp.max() <= 1, "the generating functions here are for single-photon inputs"
    return np.asarray(U)[:, inp == 1]


def _elementary_symmetric(q: np.ndarray) -> np.ndarray:
    """e_0..e_n of the values q (float64 or object arrays)."""
    n = len(q)
    e = np.zeros(n + 1, dtype=q.dtype)
    e[0] = 1
    for v in q:
        e[1:] = e[1:] + v * e[:-1]
    return e


def one_mode_marginal(U: np.ndarray, input_state, i: int, exact: bool = False) -> np.ndarray:
    """P(n_i = a) for a = 0..n."""
    V = _input_columns(U, input_state)
    n = V.shape[1]
    q = np.abs(V[i]) ** 2
    if exact:
        q = np.array([Fraction(float(v)) for v in q], dtype=object)
    e = _elementary_symmetric(q)
    g = [math.factorial(t) * e[t] for t in range(n + 1)]
    out = []
    for a in range(n + 1):
        s = sum(g[t] * math.comb(t, a) * (-1) ** (t - a) for t in range(a, n + 1))
        out.append(float(s))
    return np.array(out)


def _two_mode_table(V: np.ndarray, i: int, j: int, exact: bool):
    """D[t, u, t'] of the module docstring (complex), for modes i != j."""
    n = V.shape[1]
    a, b = np.conj(V[i]), V[i]
    c, d = np.conj(V[j]), V[j]
    terms = [(a * b), (a * d), (c * b), (c * d)]
    if exact:
        def fr(z):
            return (Fraction(float(z.real)), Fraction(float(z.imag)))
        terms = [[fr(z) for z in t] for t in terms]
        D = {(0, 0, 0): (Fraction(1), Fraction(0))}
        for k in range(n):
            nxt = dict(D)
            for (t, u, tp), (re, im) in D.items():
                for (dt, du, dtp), w in (((1, 0, 1), terms[0][k]), ((1, 0, 0), terms[1][k]),
                                        ((0, 1, 1), terms[2][k]), ((0, 1, 0), terms[3][k])):
                    key = (t + dt, u + du, tp + dtp)
                    r2, i2 = re * w[0] - im * w[1], re * w[1] + im * w[0]
                    o = nxt.get(key, (Fraction(0), Fraction(0)))
                    nxt[key] = (o[0] + r2, o[1] + i2)
            D = nxt
        return D
    D = np.zeros((n + 1, n + 1, n + 1), dtype=np.complex128)
    D[0, 0, 0] = 1
    for k in range(n):
        new = D.copy()
        new[1:, :, 1:] += terms[0][k] * D[:-1, :, :-1]
        new[1:, :, :] += terms[1][k] * D[:-1, :, :]
        new[:, 1:, 1:] += terms[2][k] * D[:, :-1, :-1]
        new[:, 1:, :] += terms[3][k] * D[:, :-1, :]
        D = new
    return D


def two_mode_marginal(U: np.ndarray, input_state, i: int, j: int, exact: bool = False) -> np.ndarray:
    """P(n_i = a, n_j = b) as an (n + 1) x (n + 1) array (zero where a + b > n)."""
    assert i != j
    V = _input_columns(U, input_state)
    n = V.shape[1]
    D = _two_mode_table(V, i, j, exact)
    f = [math.factorial(t) for t in range(n + 1)]
    if exact:
        g = {}
        for (t, u, tp), (re, _) in D.items():
            if tp == t:
                g[(t, u)] = g.get((t, u), Fraction(0)) + re * f[t] * f[u]
        out = np.zeros((n + 1, n + 1))
        for a_ in range(n + 1):
            for b_ in range(n + 1 - a_):
                s = Fraction(0)
                for (t, u), v in g.items():
                    if t >= a_ and u >= b_:
                        s += v * math.comb(t, a_) * math.comb(u, b_) * (-1) ** (t - a_ + u - b_)
                out[a_, b_] = float(s)
        return out
    tt = np.arange(n + 1)
    G = np.real(D[tt[:, None], tt[None, :], tt[:, None]]) * np.outer(f, f).astype(float)  # G[t, u]
    C = np.array([[math.comb(t, a_) * (-1) ** (t - a_) if t >= a_ else 0 for t in range(n + 1)]
                  for a_ in range(n + 1)], dtype=float)  # C[a, t]
    out = C @ G @ C.T
    mask = np.add.outer(tt, tt) > n
    out[mask] = 0.0
    return out


def empirical_one_mode(samples: np.ndarray, i: int, n: int) -> np.ndarray:
    return np.bincount(samples[:, i].astype(np.int64), minlength=n + 1)[:n + 1] / len(samples)


def empirical_two_mode(samples: np.ndarray, i: int, j: int, n: int) -> np.ndarray:
    out = np.zeros((n + 1, n + 1))
    np.add.at(out, (samples[:, i].astype(np.int64), samples[:, j].astype(np.int64)), 1.0)
    return out / len(samples)
