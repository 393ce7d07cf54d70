"""Builds the circuits of tests/golden/reference_kats.json from their op lists."""
import math

from perceval_gb300.components import BS, PS, Circuit, GenericInterferometer, catalog


def build(m: int, ops) -> Circuit:
    c = Circuit(m)
    for op in ops:
        kind, port = op[0], op[1]
        if kind == "BS.H":
            c.add(port, BS.H(*op[2:]))
        elif kind == "BS.Rx":
            c.add(port, BS.Rx(*op[2:]))
        elif kind == "PS":
            c.add(port, PS(op[2]))
        elif kind == "catalog":
            c.add(port, catalog[op[2]].build_circuit(), merge=True)
        elif kind == "identity_mesh":
            gi = GenericInterferometer(op[2], catalog["mzi phase last"].generate)
            gi.set_identity_mode()
            c.add(port, gi, merge=True)
        else:
            raise ValueError(kind)
    return c
