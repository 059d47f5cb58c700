"""Boundary condition objects accepted by ``GPU_domain.set_boundary``.

The reference's GPU path evaluates two ANUGA boundary types on the device,
``Reflective_boundary`` and ``Dirichlet_boundary``
(src/anuga_cuda/gpu_domain_advanced.py:2006-2108), and raises for any other.
Both are provided here with the same constructor arguments, with ANUGA's
two transmissive boundaries, a time-dependent stage boundary and an inflow
hydrograph, all evaluated on the device.
"""
from __future__ import annotations

import math

from . import _lib

__all__ = ["Reflective_boundary", "Dirichlet_boundary", "Time_stage_sine_boundary",
           "Transmissive_boundary", "Transmissive_stage_zero_momentum_boundary",
           "Inflow_hydrograph_boundary", "Time_stage_fourier_boundary"]


class Boundary:
    type: int = -1

    def params(self, mesh=None, tag=None):
        """The four device parameters; ``mesh`` and ``tag`` are the mesh and
        tag name the boundary is attached to."""
        return (0.0, 0.0, 0.0, 0.0)

    def tag_struct(self, mesh=None, tag=None):
        t = _lib.BoundaryTag_t()
        t.type = self.type
        for i, v in enumerate(self.params(mesh, tag)):
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

    def params(self, mesh=None, tag=None):
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

    def params(self, mesh=None, tag=None):
        return (self.mean, self.amplitude, self.period, self.phase)

    def evaluate(self, t):
        return [self.mean + self.amplitude * math.sin(2 * math.pi * t / self.period + self.phase),
                0.0, 0.0]

    def __repr__(self):
        return (f"Time_stage_sine_boundary(mean={self.mean}, amplitude={self.amplitude}, "
                f"period={self.period}, phase={self.phase})")


class Time_stage_fourier_boundary(Boundary):
    """Time-dependent stage given by five coefficients of a truncated
    Fourier series, c0 + c1 sin(wt) + c2 cos(wt) + c3 sin(2wt) + c4 cos(2wt)
    with w = 2 pi / period, and zero momentum: ANUGA's Time_boundary with
    that function of the model time, evaluated on the device (a tide with
    its first overtide on an open edge)."""

    type = _lib.BC_TIME_STAGE_FOURIER

    def __init__(self, domain=None, coefficients=(0.0, 0.0, 0.0, 0.0, 0.0), period=3600.0):
        c = [float(v) for v in coefficients]
        if len(c) != 5:
            raise ValueError("five coefficients c0..c4")
        if not period:
            raise ValueError("period must be nonzero")
        self.domain = domain
        self.coefficients, self.period = c, float(period)

    def params(self, mesh=None, tag=None):
        return tuple(self.coefficients) + (self.period,)

    def evaluate(self, t):
        c, wt = self.coefficients, 2 * math.pi * t / self.period
        return [c[0] + c[1] * math.sin(wt) + c[2] * math.cos(wt) + c[3] * math.sin(2 * wt)
                + c[4] * math.cos(2 * wt), 0.0, 0.0]

    def __repr__(self):
        return f"Time_stage_fourier_boundary(coefficients={self.coefficients}, period={self.period})"


class Transmissive_boundary(Boundary):
    """ANUGA Transmissive_boundary: the boundary takes the inside edge's
    stage and momentum (a zero-gradient outflow)."""

    type = _lib.BC_TRANSMISSIVE

    def __init__(self, domain=None):
        self.domain = domain

    def __repr__(self):
        return "Transmissive_boundary"


class Transmissive_stage_zero_momentum_boundary(Boundary):
    """ANUGA Transmissive_stage_zero_momentum_boundary: inside edge stage,
    zero momentum."""

    type = _lib.BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM

    def __init__(self, domain=None):
        self.domain = domain

    def __repr__(self):
        return "Transmissive_stage_zero_momentum_boundary"


class Inflow_hydrograph_boundary(Boundary):
    """A triangular inflow hydrograph through one tagged boundary segment:
    discharge Q(t) rises linearly from 0 at ``start`` to ``peak`` (m^3/s)
    over ``rise`` seconds and falls back to 0 over ``fall`` seconds (default
    ``2*rise``).  Q is spread evenly over the tag's edge length ``width``
    (taken from the mesh when not given) as unit discharge q = Q/width,
    entering along the inward normal with the inside edge's stage, or at
    critical depth (q^2/g)^(1/3) above the edge bed where that is higher
    (a dry or shallow inflow edge)."""

    type = _lib.BC_INFLOW_HYDROGRAPH

    def __init__(self, domain=None, peak=100.0, rise=600.0, fall=None, start=0.0, width=None):
        if not (peak >= 0 and rise > 0):
            raise ValueError("peak must be >= 0 and rise > 0")
        self.domain = domain
        self.peak, self.rise = float(peak), float(rise)
        self.fall = float(2 * rise if fall is None else fall)
        if not self.fall > 0:
            raise ValueError("fall must be > 0")
        self.start = float(start)
        self.width = None if width is None else float(width)

    def discharge(self, t):
        """Q(t) in m^3/s."""
        s = t - self.start
        if s <= 0:
            return 0.0
        if s < self.rise:
            return self.peak * (s / self.rise)
        if s < self.rise + self.fall:
            return self.peak * (1.0 - (s - self.rise) / self.fall)
        return 0.0

    def params(self, mesh=None, tag=None):
        width = self.width
        if width is None:
            if mesh is None or tag is None:
                raise ValueError("Inflow_hydrograph_boundary needs width or a mesh tag")
            width = mesh.tag_length(tag)
        if not width > 0:
            raise ValueError("inflow segment has zero length")
        return (self.peak / width, self.rise, self.fall, self.start)

    def __repr__(self):
        return (f"Inflow_hydrograph_boundary(peak={self.peak}, rise={self.rise}, "
                f"fall={self.fall}, start={self.start})")
