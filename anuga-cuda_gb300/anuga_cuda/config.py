"""Numerical parameters of the evolve step.

ANUGA keeps these in ``anuga/config.py`` and reads them as Domain
attributes; the reference does not vendor that file (it reads the same set
into ``struct domain``, src/anuga_HMPP/sw_domain_fun.h:57-120).  The values
below are stated explicitly and are passed unchanged to both the GPU library
and the CPU oracle, so results do not depend on any installed ANUGA.
"""
from __future__ import annotations

import dataclasses


@dataclasses.dataclass
class Parameters:
    g: float = 9.8
    epsilon: float = 1.0e-12
    H0: float = 1.0e-3
    minimum_allowed_height: float = 1.0e-3
    maximum_allowed_speed: float = 0.0
    beta_w: float = 0.9
    beta_w_dry: float = 0.9
    beta_uh: float = 0.9
    beta_uh_dry: float = 0.9
    beta_vh: float = 0.9
    beta_vh_dry: float = 0.9
    alpha_balance: float = 2.0
    CFL: float = 1.0
    evolve_max_timestep: float = 1.0e100
    evolve_min_timestep: float = 1.0e-6
    tight_slope_limiters: int = 1
    use_centroid_velocities: int = 1
    optimise_dry_cells: int = 1
    extrapolate_velocity_second_order: int = 1
    use_sloped_mannings: int = 0
    max_smallsteps: int = 50
    default_order: int = 2
    optimised_gradient_limiter: int = 1
    use_edge_limiter: int = 0
    flow_algorithm: int = 0            # 1: ANUGA's 'tsunami' distribute

    def replace(self, **kw) -> "Parameters":
        return dataclasses.replace(self, **kw)

    def as_tuple(self):
        return tuple(getattr(self, f.name) for f in dataclasses.fields(self))


DEFAULT = Parameters()
