"""Backend registry and factory (perceval/backends/__init__.py:39-62).

``BackendFactory.get_backend(name)`` returns a GPU backend for the names of the hot
path ("SLOS", "SLAP", "Naive", "NaiveApprox", "CliffordClifford2017"); an unknown name logs a
warning and falls back to SLOS, as in the reference.
"""
import logging

from ._abstract_backends import ABackend, ASamplingBackend, AStrongSimulationBackend, IFFBackend
from ._clifford2017 import Clifford2017Backend
from ._naive import NaiveBackend
from ._naive_approx import NaiveApproxBackend
from ._slap import SLAPBackend
from ._slos import SLOSBackend

BACKEND_LIST = {
    "CliffordClifford2017": Clifford2017Backend,
    "Naive": NaiveBackend,
    "NaiveApprox": NaiveApproxBackend,
    "SLAP": SLAPBackend,
    "SLOS": SLOSBackend,
}


class BackendFactory:
    @staticmethod
    def get_backend(backend_name: str = "SLOS", **kwargs) -> ABackend:
        if backend_name in BACKEND_LIST:
            return BACKEND_LIST[backend_name](**kwargs)
        logging.getLogger("perceval_gb300.user").warning('Backend "%s" not found. Falling back on SLOS',
                                                         backend_name)
        return BACKEND_LIST["SLOS"](**kwargs)

    @staticmethod
    def list():
        return list(BACKEND_LIST.keys())


__all__ = ["ABackend", "ASamplingBackend", "AStrongSimulationBackend", "BACKEND_LIST", "BackendFactory", "IFFBackend",
           "Clifford2017Backend", "NaiveApproxBackend", "NaiveBackend", "SLAPBackend", "SLOSBackend"]
