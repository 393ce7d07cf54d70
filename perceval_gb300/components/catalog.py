"""The catalog items that the backend tests and workloads use.

* ``mzi phase last`` (perceval/components/core_catalog/mzi.py:88-100):
  BS(theta_a) // (1, PS(phi_a)) // BS(theta_b) // (1, PS(phi_b)).
* ``mzi phase first`` (mzi.py:69-85):
  (0, PS(phi_a)) // BS(theta_a) // (0, PS(phi_b)) // BS(theta_b).
* ``postprocessed cz`` (perceval/components/core_catalog/postprocessed_cz.py:49-57) and
  ``postprocessed cnot`` (postprocessed_cnot.py:49-54), 6 modes, heralds on 4 and 5.
"""
from __future__ import annotations

import math

from .circuit import BS, PS, PERM, Circuit
from .parameter import Parameter


def _handle(v, default_name):
    if v is None:
        return Parameter(default_name)
    if isinstance(v, str):
        return Parameter(v)
    return v


class _MZI:
    def __init__(self, name: str, phase_last: bool):
        self.name = name
        self._phase_last = phase_last

    def build_circuit(self, phi_a=None, phi_b=None, theta_a=math.pi / 2, theta_b=math.pi / 2, i=None):
        if i is not None:
            phi_a, phi_b = f"phi_a{i}", f"phi_b{i}"
        phi_a = _handle(phi_a, "phi_a")
        phi_b = _handle(phi_b, "phi_b")
        if self._phase_last:
            return (Circuit(2, name="MZI") // BS(theta=theta_a) // (1, PS(phi=phi_a))
                    // BS(theta=theta_b) // (1, PS(phi=phi_b)))
        return (Circuit(2, name="MZI") // (0, PS(phi=phi_a)) // BS(theta=theta_a)
                // (0, PS(phi=phi_b)) // BS(theta=theta_b))

    def generate(self, i: int):
        return self.build_circuit(i=i)


class _PostProcessedCZ:
    name = "postprocessed cz"

    def build_circuit(self, **kwargs) -> Circuit:
        theta_13 = BS.r_to_theta(1 / 3)
        return (Circuit(6, name="PostProcessed CZ")
                .add(1, PERM([2, 1, 3, 0]))
                .add((0, 1), BS.H(theta_13))
                .add((2, 3), BS.H(theta_13))
                .add((4, 5), BS.H(theta_13))
                .add(1, PERM([3, 1, 0, 2])))


class _PostProcessedCNOT:
    name = "postprocessed cnot"

    def build_circuit(self, **kwargs) -> Circuit:
        return (Circuit(6, name="PostProcessed CNOT")
                .add((2, 3), BS.H())
                .add(0, _PostProcessedCZ().build_circuit(), merge=True)
                .add((2, 3), BS.H()))


catalog = {
    "mzi phase last": _MZI("mzi phase last", True),
    "mzi phase first": _MZI("mzi phase first", False),
    "postprocessed cz": _PostProcessedCZ(),
    "postprocessed cnot": _PostProcessedCNOT(),
}
