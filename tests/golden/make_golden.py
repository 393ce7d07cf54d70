"""Generates tests/golden/golden_values.json: high-precision golden vectors.

Permanents and SLOS amplitudes of small seeded inputs, evaluated with mpmath at 40
significant digits by Ryser's formula over exact subsets (independent of both the
CPU oracle's and the GPU kernels' Gray-code and float-float arithmetic).  Run from
the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import itertools
import json
import math
from pathlib import Path

import mpmath
import numpy as np

mpmath.mp.dps = 40
HERE = Path(__file__).resolve().parent


def haar(n: int, seed: int) -> np.ndarray:
    rs = np.random.RandomState(seed)
    u = rs.randn(n, n) + 1j * rs.randn(n, n)
    q, r = np.linalg.qr(u)
    return q @ np.diag(np.sign(np.diagonal(np.real(r))))


def perm_mp(a: np.ndarray) -> mpmath.mpc:
    n = a.shape[0]
    if n == 0:
        return mpmath.mpc(1)
    A = [[mpmath.mpc(complex(a[i, j]).real, complex(a[i, j]).imag) for j in range(n)] for i in range(n)]
    tot = mpmath.mpc(0)
    for mask in range(1, 1 << n):
        cols = [j for j in range(n) if mask >> j & 1]
        p = mpmath.mpc(1)
        for i in range(n):
            p *= mpmath.fsum(A[i][j] for j in cols)
        tot += -p if (len(cols) & 1) else p
    return -tot if n & 1 else tot


def fock_states(m: int, n: int):
    if m == 1:
        return [(n,)]
    out = []
    for a in range(n, -1, -1):
        out.extend((a,) + t for t in fock_states(m - 1, n - a))
    return out


def c2l(z) -> list[str]:
    return [mpmath.nstr(mpmath.re(z), 25), mpmath.nstr(mpmath.im(z), 25)]


def main():
    out = {"about": __doc__.strip().splitlines()[0], "permanents": [], "slos": []}
    rng = np.random.default_rng(2024)
    for n in range(1, 11):
        for kind in ("gaussian", "haar_sub"):
            if kind == "gaussian":
                a = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / math.sqrt(2)
            else:
                u = haar(3 * n, seed=n)
                rows = rng.choice(3 * n, n, replace=False)
                cols = rng.choice(3 * n, n, replace=False)
                a = u[np.ix_(rows, cols)]
            out["permanents"].append({"n": n, "kind": kind,
                                      "matrix": [[v.real, v.imag] for v in a.reshape(-1)],
                                      "perm": c2l(perm_mp(a))})
    for m, inp, seed in [(5, (1, 1, 1, 0, 0), 7), (5, (2, 0, 1, 0, 0), 7), (4, (0, 3, 0, 1), 11)]:
        u = haar(m, seed)
        n = sum(inp)
        amps = []
        pin = math.prod(math.factorial(v) for v in inp)
        for s in fock_states(m, n):
            rows = [j for j, v in enumerate(s) for _ in range(v)]
            cols = [i for i, v in enumerate(inp) for _ in range(v)]
            p = perm_mp(u[np.ix_(rows, cols)])
            f = math.prod(math.factorial(v) for v in s) * pin
            amps.append(c2l(p / mpmath.sqrt(f)))
        out["slos"].append({"m": m, "input": list(inp), "unitary_seed": seed,
                            "unitary": [[v.real, v.imag] for v in u.reshape(-1)],
                            "states": [list(s) for s in fock_states(m, n)], "amplitudes": amps})
    (HERE / "golden_values.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
