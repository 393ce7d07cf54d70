"""Seeded Haar-random unitaries, generated exactly as the reference generates them.

perceval/utils/matrix.py:141-173: ``U = randn(n, n) + 1j * randn(n, n)`` drawn from
numpy's legacy global generator (real block first), then ``Q, R = qr(U)`` and
``Q @ diag(sign(Re diag R))``.  Every workload's inputs come from here on the host
(numpy, not the torch generator) and are copied to the device.
"""
from __future__ import annotations

import numpy as np


def unitarize_matrix(u: np.ndarray) -> np.ndarray:
    """Make a square complex matrix unitary by QR with a phase-fixed R diagonal."""
    q, r = np.linalg.qr(u)
    d = np.sign(np.diagonal(np.real(r)))
    return q @ np.diag(d)


def random_unitary(n: int, seed: int | None = None) -> np.ndarray:
    """n x n Haar-random complex128 unitary from numpy's legacy generator.

    With ``seed`` given, ``np.random.seed(seed)`` is called first (the reference's
    ``random_seed`` seeds numpy the same way, perceval/utils/_random.py:36-58).
    """
    if seed is not None:
        np.random.seed(seed)
    u = np.random.randn(n, n) + 1j * np.random.randn(n, n)
    return unitarize_matrix(u)


def is_unitary(u: np.ndarray, tol: float = 1e-10) -> bool:
    u = np.asarray(u)
    return u.shape[0] == u.shape[1] and np.allclose(u @ u.conj().T, np.eye(u.shape[0]), atol=tol)


class Matrix:
    """Namespace mirroring ``perceval.utils.Matrix`` static constructors."""

    random_unitary = staticmethod(random_unitary)

    @staticmethod
    def eye(n: int) -> np.ndarray:
        return np.eye(n, dtype=complex)
