"""GB300-native linear-optics hot path behind Perceval's backend API.

Backends ``SLOS``, ``Naive``, ``NaiveApprox`` and ``CliffordClifford2017`` run hand-written sm_103a
CUDA kernels through the C ABI of ``lib/libpcvl_gb300.so`` (declared in
``include/pcvl_gb300.h``); there is no CPU fallback.  ``Simulator`` and ``SamplesProvider``
batch the many input states of a mixture into those backends.
"""
from .backends import (BACKEND_LIST, ABackend, ASamplingBackend, AStrongSimulationBackend, BackendFactory,
                       Clifford2017Backend, NaiveApproxBackend, NaiveBackend, SLAPBackend, SLOSBackend)
from .components import BS, PERM, PS, Circuit, GenericInterferometer, Unitary, catalog
from .simulators import SamplesProvider, Simulator
from .utils import (BasicState, BSCount, BSDistribution, BSSamples, FockState, StateVector, Matrix,
                    allstate_iterator, random_seed)

__version__ = "0.1.0"
