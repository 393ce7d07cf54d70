"""Linear-optics circuits, restated only as far as the backends need a unitary.

The reference builds the m x m unitary of a circuit by left-multiplying the embedded
unitaries of its components in order (perceval/components/linear_circuit.py:487-503,
535-547).  Components restated here: ``BS`` with its three conventions
(perceval/components/unitary_components.py:42-190), ``PS`` (:244-270), ``PERM``
(:464-484), ``Unitary`` (:423-447), ``Barrier``; ``GenericInterferometer`` rectangle
(perceval/components/generic_interferometer.py:150-165) and the catalog items the
tests and workloads use (``mzi phase last``/``mzi phase first``,
perceval/components/core_catalog/mzi.py:69-100; ``postprocessed cz``/``cnot``).
"""
from .parameter import Parameter, P
from .circuit import ACircuit, Circuit, BS, BSConvention, PS, PERM, Unitary, Barrier
from .interferometer import GenericInterferometer, InterferometerShape
from .catalog import catalog
from .mesh import clements_mesh_unitary, clements_mesh_phase_count

__all__ = ["Parameter", "P", "ACircuit", "Circuit", "BS", "BSConvention", "PS", "PERM",
           "Unitary", "Barrier", "GenericInterferometer", "InterferometerShape", "catalog",
           "clements_mesh_unitary", "clements_mesh_phase_count"]
