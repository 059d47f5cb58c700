"""Boundary condition objects accepted by ``GPU_domain.set_boundary``.

The reference's GPU path evaluates two ANUGA boundary types on the device,
``Reflective_boundary`` and ``Dirichlet_boundary``
(src/anuga_cuda/gpu_domain_advanced.py:2006-2108), and raises for any other.
Both are provided here with the same constructor arguments, plus one
time-dependent stage boundary evaluated on the device.
"""
from __future__ import annotations

import math

from . import _lib

__all__ = ["Reflective_boundary", "Dirichlet_boundary", "Time_stage_sine_boundary"]


class Boundary:
    type: int = -1

    def params(self):
        return (0.0, 0.0, 0.0, 0.0)

    def tag_struct(self):
        t = _lib.BoundaryTag_t()
        t.type = self.type
        for i, v in enumerate(self.params()):
            t.p[i] = float(v)
        return t


class Reflective_boundary(Boundary):
    """Reflective wall: edge stage copied, momentum mirrored about the edge
    normal (evaluate_segment.cu:3-76)."""

    type = _lib.BC_REFLECTIVE

    def __init__(self, domain=None):
        self.domain = domain

    def __repr__(self):
        return "Reflective_boundary"


class Dirichlet_boundary(Boundary):
    """Fixed conserved values [stage, xmomentum, ymomentum]
    (evaluate_segment.cu:80-115).  A fourth value (elevation, ANUGA's
    evolved-quantities form) is accepted and ignored: the flux extends the
    bed to the boundary."""

    type = _lib.BC_DIRICHLET

    def __init__(self, dirichlet_values=None):
        if dirichlet_values is None or len(dirichlet_values) < 3:
            raise ValueError("Dirichlet_boundary needs [stage, xmomentum, ymomentum]")
        self.dirichlet_values = [float(v) for v in dirichlet_values]

    def params(self):
        return tuple(self.dirichlet_values[:3]) + (0.0,)

    def __repr__(self):
        return f"Dirichlet_boundary({self.dirichlet_values})"


class Time_stage_sine_boundary(Boundary):
    """Time-dependent stage  mean + amplitude*sin(2*pi*t/period + phase)
    with zero momentum, evaluated on the device at the model time of each
    update_boundary (e.g. a tide on an open edge)."""

    type = _lib.BC_TIME_STAGE_SINE

    def __init__(self, domain=None, amplitude=1.0, period=600.0, mean=0.0, phase=0.0):
        if not period:
            raise ValueError("period must be nonzero")
        self.domain = domain
        self.amplitude, self.period, self.mean, self.phase = (
            float(amplitude), float(period), float(mean), float(phase))

    def params(self):
        return (self.mean, self.amplitude, self.period, self.phase)

    def evaluate(self, t):
        return [self.mean + self.amplitude * math.sin(2 * math.pi * t / self.period + self.phase),
                0.0, 0.0]

    def __repr__(self):
        return (f"Time_stage_sine_boundary(mean={self.mean}, amplitude={self.amplitude}, "
                f"period={self.period}, phase={self.phase})")
