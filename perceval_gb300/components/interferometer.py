"""Rectangular (Clements) and triangular generic interferometers.

Placement follows perceval/components/generic_interferometer.py:150-176: in the
rectangle, column i (i = 0..depth-1) holds components on mode pairs (j, j+1) for
j = i % 2, i % 2 + 2, ... < m - 1, numbered in that order; the triangle adds, for
i = 1..m-1, components on (j-1, j) for j = i down to 1.
"""
from __future__ import annotations

import math
from enum import Enum
from typing import Callable

from .circuit import ACircuit, Circuit


class InterferometerShape(Enum):
    RECTANGLE = 0
    TRIANGLE = 1


class GenericInterferometer(Circuit):
    def __init__(self, m: int, fun_gen: Callable[[int], ACircuit],
                 shape: InterferometerShape = InterferometerShape.RECTANGLE, depth: int | None = None,
                 phase_shifter_fun_gen: Callable[[int], ACircuit] | None = None,
                 phase_at_output: bool = False):
        super().__init__(m)
        self._depth_per_mode = [0] * m
        if phase_shifter_fun_gen and not phase_at_output:
            for i in range(m):
                self.add(i, phase_shifter_fun_gen(i), merge=True)
        if shape == InterferometerShape.RECTANGLE:
            max_depth = m if depth is None else depth
            idx = 0
            for i in range(max_depth):
                for j in range(i % 2, m - 1, 2):
                    if depth is not None and (self._depth_per_mode[j] == depth
                                              or self._depth_per_mode[j + 1] == depth):
                        continue
                    self.add((j, j + 1), fun_gen(idx), merge=True)
                    self._depth_per_mode[j] += 1
                    self._depth_per_mode[j + 1] += 1
                    idx += 1
        elif shape == InterferometerShape.TRIANGLE:
            idx = 0
            for i in range(1, m):
                for j in range(i, 0, -1):
                    if depth is not None and (self._depth_per_mode[j - 1] == depth
                                              or self._depth_per_mode[j] == depth):
                        continue
                    self.add((j - 1, j), fun_gen(idx), merge=True)
                    self._depth_per_mode[j - 1] += 1
                    self._depth_per_mode[j] += 1
                    idx += 1
        else:
            raise NotImplementedError(f"Shape {shape} not supported")
        if phase_shifter_fun_gen and phase_at_output:
            for i in range(m):
                self.add(i, phase_shifter_fun_gen(i), merge=True)

    @property
    def mzi_depths(self) -> list[int]:
        return self._depth_per_mode

    def set_identity_mode(self):
        """All free parameters to pi: photons exit on the mode they entered."""
        for p in self.get_parameters():
            p.set_value(math.pi)
