"""Named circuit parameters (numeric only; the symbolic mode is not supported by this package)."""
from __future__ import annotations

import math


class Parameter:
    """A named real parameter, optionally bounded, with a value that can be set later."""

    def __init__(self, name: str, value: float | None = None, min_v: float | None = None,
                 max_v: float | None = None, periodic: bool = True):
        self.name = name
        self._value = None if value is None else float(value)
        self.min_v = min_v
        self.max_v = max_v
        self._periodic = periodic

    @property
    def defined(self) -> bool:
        return self._value is not None

    def set_value(self, v: float, force: bool = False):
        v = float(v)
        if self._periodic and self.min_v is not None and self.max_v is not None and not force:
            span = self.max_v - self.min_v
            if span > 0 and not (self.min_v <= v <= self.max_v):
                v = self.min_v + math.fmod(v - self.min_v, span)
                if v < self.min_v:
                    v += span
        self._value = v

    def reset(self):
        self._value = None

    def __float__(self) -> float:
        if self._value is None:
            raise ValueError(f"parameter {self.name} has no value")
        return self._value

    def __repr__(self) -> str:
        return f"Parameter(name='{self.name}', value={self._value})"


P = Parameter
