"""Generates tests/golden/perm_large.json: permanents of seeded Haar submatrices at the
single-matrix sizes where the CPU oracle takes minutes (n = 32), for the GPU parity
tests to compare against without running the oracle at test time.

The matrix is the n x n submatrix (rows and columns drawn without replacement with
numpy default_rng(seed)) of the 1024 x 1024 Haar unitary made as the reference makes it
(perceval/utils/matrix.py:141-173, numpy legacy seed 0).  It is stored element by
element, so the test does not depend on the platform's QR.  The permanent is the C
oracle's FP64 Glynn sum (Neumaier-compensated); its Ryser sum is stored beside it as a
cross-check (Ryser's alternating subset sum cancels far more: at n = 32 the two agree to
about 2e-8 relative, and the generator requires 1e-6).  Run from the repository root
(about 1-2 minutes on 8 cores):  python tests/golden/make_perm_fixtures.py
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

CASES = ((32, 32),)  # (n, seed of the row/column draw)


def haar(n: int, seed: int) -> np.ndarray:
    rs = np.random.RandomState(seed)
    u = rs.randn(n, n) + 1j * rs.randn(n, n)
    q, r = np.linalg.qr(u)
    return q @ np.diag(np.sign(np.diagonal(np.real(r))))


def main():
    from oracle import oracle
    oracle.build()
    U = haar(1024, 0)
    out = {"generator": "tests/golden/make_perm_fixtures.py", "cases": []}
    for n, seed in CASES:
        rng = np.random.default_rng(seed)
        a = np.ascontiguousarray(U[np.ix_(rng.choice(1024, n, False), rng.choice(1024, n, False))])
        t0 = time.time()
        g = oracle.perm(a, "glynn")
        t1 = time.time()
        r = oracle.perm(a, "ryser")
        t2 = time.time()
        rel = abs(g - r) / abs(g)
        assert rel < 1e-6, f"oracle Glynn and Ryser disagree at n={n}: {rel:.2e}"
        out["cases"].append({"n": n, "seed": seed,
                             "matrix": [[float(v.real), float(v.imag)] for v in a.reshape(-1)],
                             "perm_glynn": [g.real, g.imag], "perm_ryser": [r.real, r.imag],
                             "glynn_ryser_rel_diff": rel, "oracle_threads": oracle.num_threads(),
                             "oracle_seconds": {"glynn": round(t1 - t0, 1), "ryser": round(t2 - t1, 1)}})
        print(f"n={n}: perm {g:.17g}  Glynn-Ryser {rel:.2e}  ({t1 - t0:.1f} s + {t2 - t1:.1f} s)")
    (HERE / "perm_large.json").write_text(json.dumps(out))


if __name__ == "__main__":
    main()
