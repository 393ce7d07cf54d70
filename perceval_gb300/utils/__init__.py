"""State containers, enumeration, seeded unitaries and seeding."""
from .states import (BasicState, BSCount, BSDistribution, BSSamples, FockState, FSMask, StateVector,
                     allstate_iterator, fock_rank, fock_space_array, fock_space_size, fock_unrank,
                     max_photon_state_iterator)
from .matrix import Matrix, random_unitary, unitarize_matrix
from ._random import random_seed
from .globals import global_params

__all__ = ["BasicState", "BSCount", "BSDistribution", "BSSamples", "FockState", "FSMask", "StateVector",
           "allstate_iterator", "fock_rank", "fock_space_array", "fock_space_size", "fock_unrank",
           "max_photon_state_iterator", "Matrix", "random_unitary", "unitarize_matrix", "random_seed",
           "global_params"]
