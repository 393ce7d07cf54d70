"""Circuit and unitary components.

Unitary conventions, restated from the reference:

* ``BS`` (perceval/components/unitary_components.py:142-183): with c = cos(theta/2),
  s = sin(theta/2) and the template T of the convention
  (Rx: [[1, i], [i, 1]], Ry: [[1, -1], [1, 1]], H: [[1, 1], [1, -1]]),
  U = [[T00 e^{i(tl+tr)} c, T01 e^{i(tr+bl)} s], [T10 e^{i(tl+br)} s, T11 e^{i(bl+br)} c]].
* ``PS`` (:262-270): [[e^{i phi}]].
* ``PERM`` (:475-484): U[perm[i], i] = 1.
* ``Circuit.compute_unitary`` (perceval/components/linear_circuit.py:487-503): each
  component's unitary is embedded into the identity on its modes and left-multiplied,
  U = U_k ... U_2 U_1.
"""
from __future__ import annotations

import math
from enum import IntEnum

import numpy as np

from .parameter import Parameter


def _param(name: str, v, min_v=None, max_v=None) -> Parameter:
    if isinstance(v, Parameter):
        if v.min_v is None:
            v.min_v, v.max_v = min_v, max_v
        return v
    p = Parameter(name, v, min_v, max_v)
    p.fixed = True
    return p


def _free(params) -> list[Parameter]:
    return [p for p in params if not getattr(p, "fixed", False)]


class ACircuit:
    """Base of every linear component: m modes and a unitary."""

    requires_polarization = False

    def __init__(self, m: int, name: str | None = None):
        self._m = m
        self._name = name

    @property
    def m(self) -> int:
        return self._m

    @property
    def name(self) -> str:
        return self._name or type(self).__name__

    def _compute_unitary(self) -> np.ndarray:
        raise NotImplementedError

    def compute_unitary(self, use_symbolic: bool = False) -> np.ndarray:
        if use_symbolic:
            raise NotImplementedError("symbolic unitaries are not supported by perceval_gb300")
        return self._compute_unitary()

    @property
    def U(self) -> np.ndarray:
        return self.compute_unitary()

    def get_parameters(self) -> list[Parameter]:
        return []

    def __floordiv__(self, other):
        c = Circuit(self.m)
        c.add(0, self)
        return c // other


class BSConvention(IntEnum):
    Rx = 0
    Ry = 1
    H = 2


_BS_TEMPLATE = {
    BSConvention.Rx: np.array([[1, 1j], [1j, 1]], dtype=complex),
    BSConvention.Ry: np.array([[1, -1], [1, 1]], dtype=complex),
    BSConvention.H: np.array([[1, 1], [1, -1]], dtype=complex),
}


class BS(ACircuit):
    """Beam splitter with angle theta and four phases (tl, bl, tr, br)."""

    def __init__(self, theta=math.pi / 2, phi_tl=0, phi_bl=0, phi_tr=0, phi_br=0,
                 convention: BSConvention = BSConvention.Rx):
        super().__init__(2)
        self._convention = convention
        self._theta = _param("theta", theta, 0, 4 * math.pi)
        self._phi_tl = _param("phi_tl", phi_tl, 0, 2 * math.pi)
        self._phi_bl = _param("phi_bl", phi_bl, 0, 2 * math.pi)
        self._phi_tr = _param("phi_tr", phi_tr, 0, 2 * math.pi)
        self._phi_br = _param("phi_br", phi_br, 0, 2 * math.pi)

    @staticmethod
    def H(theta=math.pi / 2, phi_tl=0, phi_bl=0, phi_tr=0, phi_br=0):
        return BS(theta, phi_tl, phi_bl, phi_tr, phi_br, convention=BSConvention.H)

    @staticmethod
    def Rx(theta=math.pi / 2, phi_tl=0, phi_bl=0, phi_tr=0, phi_br=0):
        return BS(theta, phi_tl, phi_bl, phi_tr, phi_br, convention=BSConvention.Rx)

    @staticmethod
    def Ry(theta=math.pi / 2, phi_tl=0, phi_bl=0, phi_tr=0, phi_br=0):
        return BS(theta, phi_tl, phi_bl, phi_tr, phi_br, convention=BSConvention.Ry)

    @staticmethod
    def r_to_theta(r: float) -> float:
        return 2 * math.acos(math.sqrt(r))

    @property
    def name(self) -> str:
        return f"BS.{self._convention.name}"

    def _compute_unitary(self) -> np.ndarray:
        th = float(self._theta)
        c, s = math.cos(th / 2), math.sin(th / 2)
        tl, bl, tr, br = (float(p) for p in (self._phi_tl, self._phi_bl, self._phi_tr, self._phi_br))
        u = _BS_TEMPLATE[self._convention].copy()
        u[0, 0] *= np.exp(1j * (tl + tr)) * c
        u[0, 1] *= np.exp(1j * (tr + bl)) * s
        u[1, 1] *= np.exp(1j * (bl + br)) * c
        u[1, 0] *= np.exp(1j * (tl + br)) * s
        return u

    def get_parameters(self):
        return _free((self._theta, self._phi_tl, self._phi_bl, self._phi_tr, self._phi_br))


class PS(ACircuit):
    """Phase shifter exp(i phi) on one mode."""

    def __init__(self, phi):
        super().__init__(1)
        self._phi = _param("phi", phi, 0, 2 * math.pi)

    def _compute_unitary(self) -> np.ndarray:
        return np.array([[np.exp(1j * float(self._phi))]], dtype=complex)

    def get_parameters(self):
        return _free((self._phi,))


class Unitary(ACircuit):
    """Arbitrary unitary component (perceval/components/unitary_components.py:423-447)."""

    def __init__(self, U, name: str | None = None):
        U = np.asarray(U, dtype=complex)
        assert U.ndim == 2 and U.shape[0] == U.shape[1], "Unitary must be a square matrix"
        super().__init__(U.shape[0], name)
        self._u = U

    def _compute_unitary(self) -> np.ndarray:
        return self._u.copy()


class PERM(Unitary):
    """Mode permutation: photon in mode i goes to mode perm[i]."""

    def __init__(self, perm: list[int]):
        assert sorted(perm) == list(range(len(perm))), f"{perm} is not a permutation"
        u = np.zeros((len(perm), len(perm)), dtype=complex)
        for i, v in enumerate(perm):
            u[v, i] = 1
        super().__init__(u, "PERM")


class Barrier(ACircuit):
    """Visual alignment only: identity."""

    def __init__(self, m: int, visible: bool = True):
        super().__init__(m)

    def _compute_unitary(self) -> np.ndarray:
        return np.eye(self.m, dtype=complex)


class Circuit(ACircuit):
    """Ordered list of (modes, component); unitary = left-multiplied product."""

    def __init__(self, m: int, name: str | None = None):
        super().__init__(m, name)
        self._components: list[tuple[tuple[int, ...], ACircuit]] = []

    def add(self, port, component: ACircuit, merge: bool = False):
        if isinstance(port, int):
            port = tuple(range(port, port + component.m))
        port = tuple(port)
        assert len(port) == component.m, "port width and component size mismatch"
        assert port == tuple(range(port[0], port[0] + len(port))), "ports must be consecutive"
        assert port[-1] < self.m, "component exceeds circuit size"
        if merge and isinstance(component, Circuit):
            for r, c in component._components:
                self._components.append((tuple(p + port[0] for p in r), c))
        else:
            self._components.append((port, component))
        return self

    def __floordiv__(self, other):
        if isinstance(other, tuple):
            port, comp = other
        else:
            port, comp = 0, other
        return self.add(port, comp, merge=True)

    def __iter__(self):
        return iter(self._components)

    def ncomponents(self) -> int:
        return len(self._components)

    def _compute_unitary(self) -> np.ndarray:
        u = np.eye(self.m, dtype=complex)
        for r, c in self._components:
            cu = c.compute_unitary()
            lo, hi = r[0], r[-1] + 1
            # left-multiply the embedded component: only rows lo:hi change
            u[lo:hi, :] = cu @ u[lo:hi, :]
        return u

    def get_parameters(self) -> list[Parameter]:
        seen, out = set(), []
        for _, c in self._components:
            for p in c.get_parameters():
                if id(p) not in seen:
                    seen.add(id(p))
                    out.append(p)
        return out
