"""Seeding, mirroring ``perceval.utils.random_seed`` (perceval/utils/_random.py:36-58).

``random_seed(seed)`` seeds Python's ``random``, numpy's legacy generator and the
GPU samplers' Philox key; a ``None`` seed draws a fresh key.  The samplers number
their samples from a process-wide counter, so consecutive calls draw fresh samples
and a given seed reproduces the same sequence.
"""
from __future__ import annotations

import random
import threading

import numpy as np

_lock = threading.Lock()
_seed = random.getrandbits(64)
_next_sample = 0


def random_seed(seed: int | None = None):
    global _seed, _next_sample
    random.seed(seed)
    np.random.seed(seed if seed is None else seed % (2**32))
    with _lock:
        _seed = random.getrandbits(64) if seed is None else int(seed) & (2**64 - 1)
        _next_sample = 0


def take_samples(count: int) -> tuple[int, int]:
    """Reserve ``count`` sample counters: returns (seed, first sample index)."""
    global _next_sample
    with _lock:
        first = _next_sample
        _next_sample += int(count)
        return _seed, first
