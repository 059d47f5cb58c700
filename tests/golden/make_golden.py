"""Generate the golden fixtures of the CPU oracle from the reference's own
ANUGA C kernels.

Run where the reference sources are present (they are compiled by
``make -C oracle ref`` from src/anuga_HMPP/shallow_water_ext.c and
quantity.c):

    python tests/golden/make_golden.py

For each case the fixture stores the mesh arrays, the initial state, the
output of every reference kernel applied once (protect, second-order
extrapolation, balance, vertex-to-edge interpolation, central-upwind fluxes,
gravity_wb, Manning friction, the semi-implicit update) and the conserved
state and timestep after each of ``STEPS`` Euler steps driven by those
kernels in the reference's call order (src/anuga_cuda/
gpu_domain_advanced.py:2476-2675), and the same after each of ``RK_STEPS``
RK2 and RK3 steps (ANUGA's evolve_one_rk2_step / evolve_one_rk3_step driving
the reference's kernels and its _saxpy_centroid_values).  The time-step rule and the boundary
conditions have no C-callable counterpart in the reference and come from the
oracle's restatement (src/anuga_HMPP/evolve.c:115-160,
src/anuga_cuda/evaluate_segment/evaluate_segment.cu:3-115).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "anuga-cuda_gb300")]

from anuga_cuda import DEFAULT, scenarios  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
STEPS = 40
SAVED_STEPS = (0, 1, 4, 19, 39)   # conserved state stored after these steps
RK_STEPS = 12                      # Runge-Kutta runs (rk2, rk3)
RK_SAVED_STEPS = (0, 3, 11)
MESH_KEYS = ["neighbours", "neighbour_edges", "surrogate_neighbours", "number_of_boundaries",
             "tri_full_flag", "normals", "edgelengths", "radii", "areas", "vertex_coordinates",
             "centroid_coordinates", "boundary_cells", "boundary_edges", "boundary_tag"]
STATE_KEYS = ["stage_centroid_values", "xmom_centroid_values", "ymom_centroid_values",
              "bed_centroid_values", "friction_centroid_values", "stage_vertex_values",
              "xmom_vertex_values", "ymom_vertex_values", "bed_vertex_values",
              "bed_edge_values"]


def four_triangles():
    """The 4-triangle mesh of the reference's only known-answer test
    (src/anuga_cuda/anuga_gpu/mytest.py:11-34): a central triangle with three
    neighbours that each have two boundary edges; here with a wet/dry
    initial state so that every branch runs."""
    from anuga_cuda.boundaries import Dirichlet_boundary, Reflective_boundary
    from anuga_cuda.mesh import Mesh
    pts = np.array([[0.0, 0.0], [0.0, 2.0], [2.0, 0.0], [0.0, 4.0], [2.0, 2.0], [4.0, 0.0]])
    tris = np.array([[1, 0, 2], [1, 2, 4], [4, 2, 5], [3, 1, 4]])
    mesh = Mesh(pts, tris, None, reorder=False)
    bnd = {kk: ("left" if k == 0 else "exterior") for kk in mesh.boundary for k in [kk[0]]}
    mesh = Mesh(pts, tris, bnd, reorder=False)
    N = mesh.number_of_elements
    V = mesh.vertex_coordinates.reshape(-1, 3, 2)
    z = -1.0 + 0.3 * V[..., 0] + 0.1 * V[..., 1]
    zc = z.mean(axis=1)
    w = np.maximum(zc, np.array([0.2, -0.1, 0.05, -0.6]))
    return scenarios.Scenario(
        name="four_triangles", mesh=mesh, elevation_vertex=z, stage_centroid=w,
        xmom_centroid=np.array([0.1, -0.05, 0.0, 0.02]), ymom_centroid=np.array([0.0, 0.03, -0.01, 0.0]),
        friction=np.full(N, 0.03),
        boundaries={"left": Dirichlet_boundary([0.3, 0.0, 0.0]), "exterior": Reflective_boundary()})


def single_triangle():
    """One triangle, three boundary edges (the number_of_boundaries == 3
    branch)."""
    from anuga_cuda.boundaries import Reflective_boundary
    from anuga_cuda.mesh import Mesh
    mesh = Mesh(np.array([[0.0, 0.0], [3.0, 0.0], [0.0, 2.0]]), np.array([[0, 1, 2]]), None,
                reorder=False)
    V = mesh.vertex_coordinates.reshape(-1, 3, 2)
    z = -0.5 + 0.1 * V[..., 0]
    return scenarios.Scenario(
        name="single_triangle", mesh=mesh, elevation_vertex=z,
        stage_centroid=np.array([0.4]), xmom_centroid=np.array([0.2]),
        ymom_centroid=np.array([-0.1]), friction=np.array([0.02]),
        boundaries={"exterior": Reflective_boundary()})


def cases():
    yield "four_triangles", four_triangles(), DEFAULT
    yield "single_triangle", single_triangle(), DEFAULT
    yield "basin_wetdry", scenarios.small_basin(12, 10, seed=1), DEFAULT.replace(
        beta_w_dry=0.2, beta_uh_dry=0.1, beta_vh_dry=0.3)
    yield "basin_momentum_limiter", scenarios.small_basin(9, 7, seed=7), DEFAULT.replace(
        extrapolate_velocity_second_order=0, tight_slope_limiters=0,
        use_centroid_velocities=0, use_sloped_mannings=1)
    yield "harbour_small", scenarios.tidal_harbour(target_triangles=1500, seed=11,
                                                   points="bridson"), DEFAULT
    yield "basin_edge_limiter", scenarios.small_basin(9, 7, seed=8), DEFAULT.replace(
        use_edge_limiter=1, beta_w=0.8, beta_uh=1.1, beta_vh=1.3)
    yield "channel_vertex_limiter", scenarios.channel_inflow(14, 5, seed=1), DEFAULT.replace(
        optimised_gradient_limiter=0)
    yield "basin_tsunami", scenarios.small_basin(11, 8, seed=9), DEFAULT.replace(
        flow_algorithm=1, beta_w_dry=0.4, beta_uh_dry=0.3, beta_vh_dry=0.2)


def ref_step(R, od, finaltime=-1.0):
    D = od.D
    t0 = D.time
    ft = R.compute_fluxes(od)
    R.gravity_wb(od)
    R.manning_friction(od)
    D.flux_timestep = ft
    od.update_timestep(finaltime)
    rc = R.update(od, D.timestep)
    assert rc == 0
    D.time = t0 + D.timestep
    ref_distribute(R, od)


def ref_distribute(R, od):
    """distribute_to_vertices_and_edges (gpu_domain_advanced.py:1744-2001)
    with the reference's kernels, then the boundary values."""
    p = od.params
    if p.flow_algorithm == 1:
        # the 'tsunami' branch: protect_swb2 and the edge extrapolation
        R.protect_swb2(od)
        assert R.extrapolate_second_order_edge_sw(od) == 0
        od.update_boundary()
        return
    R.protect(od)
    if od.D.order == 1:
        od.extrapolate_first_order()
    elif p.use_edge_limiter:
        assert R.limit_by_neighbours(od, True) == 0
    elif p.optimised_gradient_limiter:
        R.extrapolate_second_order_sw(od)
    else:
        assert R.limit_by_neighbours(od, False) == 0
    R.balance_deep_and_shallow(od)
    R.interpolate_to_edges(od)
    od.update_boundary()


def ref_stage(R, od):
    """A Runge-Kutta stage after the first: the step's dt is kept."""
    R.compute_fluxes(od)
    R.gravity_wb(od)
    R.manning_friction(od)
    assert R.update(od, od.D.timestep) == 0


def ref_rk_step(R, od, method, finaltime=-1.0):
    """ANUGA's evolve_one_rk2_step / evolve_one_rk3_step (restated driver)
    on the reference's kernels, backup as a copy (the reference's
    backup_conserved_quantities is a device memcpy) and the reference's
    _saxpy_centroid_values, then the evolve loop's time update and
    distribute."""
    D = od.D
    t0 = D.time
    for q in ("stage", "xmom", "ymom"):
        od.arrays[q + "_centroid_backup"][:] = od.arrays[q + "_centroid_values"]
    ft = R.compute_fluxes(od)
    R.gravity_wb(od)
    R.manning_friction(od)
    D.flux_timestep = ft
    od.update_timestep(finaltime)
    assert R.update(od, D.timestep) == 0
    D.time = D.time + D.timestep
    ref_distribute(R, od)
    ref_stage(R, od)
    if method == "rk2":
        R.saxpy_conserved_quantities(od, 0.5, 0.5)
    else:
        R.saxpy_conserved_quantities(od, 0.25, 0.75)
        D.time = t0 + D.timestep * 0.5
        ref_distribute(R, od)
        ref_stage(R, od)
        R.saxpy_conserved_quantities(od, 2.0 / 3.0, 1.0 / 3.0)
    D.time = t0 + D.timestep
    ref_distribute(R, od)


def make(name, sc, params):
    R = O.ReferenceKernels()
    od = O.OracleDomain(sc.mesh, params, sc.oracle_tags())
    sc.apply_to_oracle(od)
    out = {}
    for k in MESH_KEYS:
        out["mesh/" + k] = np.asarray(getattr(sc.mesh, k)).copy()
    out["tags/type"] = np.array([t for t, _ in sc.oracle_tags()], dtype=np.int64)
    out["tags/p"] = np.array([p for _, p in sc.oracle_tags()], dtype=np.float64)
    for k in STATE_KEYS:
        out["init/" + k] = od.arrays[k].copy()
    # one application of each kernel, in distribute/flux order
    R.protect(od)
    out["k/protect/stage"] = od.arrays["stage_centroid_values"].copy()
    out["k/protect/xmom"] = od.arrays["xmom_centroid_values"].copy()
    out["k/protect/ymom"] = od.arrays["ymom_centroid_values"].copy()
    R.extrapolate_second_order_sw(od)
    for q in ("stage", "xmom", "ymom"):
        out[f"k/extrapolate/{q}_vertex"] = od.arrays[q + "_vertex_values"].copy()
    R.balance_deep_and_shallow(od)
    for q in ("stage", "xmom", "ymom"):
        out[f"k/balance/{q}_vertex"] = od.arrays[q + "_vertex_values"].copy()
    R.interpolate_to_edges(od)
    for q in ("stage", "xmom", "ymom"):
        out[f"k/interpolate/{q}_edge"] = od.arrays[q + "_edge_values"].copy()
    od.update_boundary()
    out["k/flux/timestep"] = np.array([R.compute_fluxes(od)])
    for q in ("stage", "xmom", "ymom"):
        out[f"k/flux/{q}_explicit"] = od.arrays[q + "_explicit_update"].copy()
    R.gravity_wb(od)
    for q in ("xmom", "ymom"):
        out[f"k/gravity/{q}_explicit"] = od.arrays[q + "_explicit_update"].copy()
    R.manning_friction(od)
    for q in ("xmom", "ymom"):
        out[f"k/friction/{q}_semi"] = od.arrays[q + "_semi_implicit_update"].copy()
    dt = 0.5 * out["k/flux/timestep"][0]
    out["k/update/dt"] = np.array([dt])
    assert R.update(od, dt) == 0
    for q in ("stage", "xmom", "ymom"):
        out[f"k/update/{q}"] = od.arrays[q + "_centroid_values"].copy()

    if params.flow_algorithm == 1:
        # the 'tsunami' distribute kernels once, from the initial state
        od = O.OracleDomain(sc.mesh, params, sc.oracle_tags())
        sc.apply_to_oracle(od)
        R.protect_swb2(od)
        for q in ("stage", "xmom", "ymom"):
            out[f"k/protect_swb2/{q}"] = od.arrays[q + "_centroid_values"].copy()
        assert R.extrapolate_second_order_edge_sw(od) == 0
        for q in ("stage", "xmom", "ymom"):
            out[f"k/edge_extrapolate/{q}_edge"] = od.arrays[q + "_edge_values"].copy()
            out[f"k/edge_extrapolate/{q}_vertex"] = od.arrays[q + "_vertex_values"].copy()

    # a fresh run of STEPS Euler steps from the initial state
    od = O.OracleDomain(sc.mesh, params, sc.oracle_tags())
    sc.apply_to_oracle(od)
    od.evolve_start(1.0e300)   # restated set-up: distribute, time, distribute, boundary
    D = od.D
    for s in range(STEPS):
        ref_step(R, od)
        out[f"run/{s}/dt"] = np.array([D.timestep])
        out[f"run/{s}/time"] = np.array([D.time])
        if s in SAVED_STEPS:
            for q in ("stage", "xmom", "ymom"):
                out[f"run/{s}/{q}"] = od.arrays[q + "_centroid_values"].copy()
    for q in ("stage", "xmom", "ymom"):
        out[f"run/final/{q}_vertex"] = od.arrays[q + "_vertex_values"].copy()
    out["run/final/mass"] = np.array([od.mass()])

    # fresh runs of RK_STEPS Runge-Kutta steps
    for method in ("rk2", "rk3"):
        od = O.OracleDomain(sc.mesh, params, sc.oracle_tags())
        sc.apply_to_oracle(od)
        od.evolve_start(1.0e300)
        D = od.D
        for s in range(RK_STEPS):
            ref_rk_step(R, od, method)
            out[f"{method}/{s}/dt"] = np.array([D.timestep])
            out[f"{method}/{s}/time"] = np.array([D.time])
            if s in RK_SAVED_STEPS:
                for q in ("stage", "xmom", "ymom"):
                    out[f"{method}/{s}/{q}"] = od.arrays[q + "_centroid_values"].copy()
    out["params"] = np.array(params.as_tuple(), dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: N={sc.mesh.number_of_elements} final time {D.time:.6f} "
          f"order {D.order}")


if __name__ == "__main__":
    O.build(ref=True)
    if not O.reference_available():
        sys.exit("reference kernels not built: needs the reference sources")
    for name, sc, params in cases():
        make(name, sc, params)
