/*
 * swgpu.h -- C ABI of libswgpu.so, the GB300 (sm_103a) shallow-water evolve
 * step for ANUGA unstructured triangle meshes.
 *
 * The reference (budiaji/anuga-cuda) exposes this path as a Python subclass
 * of anuga.Domain whose overridden methods launch one PyCUDA kernel each
 * (src/anuga_cuda/gpu_domain_advanced.py).  Each entry point below replaces
 * one of those methods or the device-array management behind them; the
 * comment on each names the reference code it stands in for.  The Python
 * package anuga_cuda (GPU_domain) binds these through ctypes.
 *
 * Conventions
 *   - Every function returns an int status: SWGPU_OK (0) or a SWGPU_E*
 *     code.  swgpu_last_error() gives the message of the last failure on a
 *     handle.  Nothing in the library aborts, traps or exits.
 *   - Host arrays use ANUGA's layout: triangle k, edge/vertex i at [3k+i],
 *     normals and vertex coordinates at [6k+2i] (x) and [6k+2i+1] (y),
 *     indices as int64 (ANUGA's `long`).  The library copies them; it never
 *     keeps a host pointer after a call returns.
 *   - A handle owns all device memory and one CUDA stream.  It must be used
 *     from one host thread at a time.  Several handles may share a device.
 */
#ifndef SWGPU_H
#define SWGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWGPU_ABI_VERSION 2

/* ---- status codes --------------------------------------------------- */
enum swgpu_status {
    SWGPU_OK = 0,
    SWGPU_EINVAL = 1,          /* bad argument (null pointer, size, enum)   */
    SWGPU_ECUDA = 2,           /* a CUDA runtime call failed                */
    SWGPU_ENOMEM = 3,          /* device allocation failed                  */
    SWGPU_EDENOMINATOR = 4,    /* semi-implicit denominator <= 0 (_update)  */
    SWGPU_ESMALLSTEP = 5,      /* timestep below minimum even at order 1    */
    SWGPU_ENONFINITE = 6,      /* NaN or Inf in the flux timestep           */
    SWGPU_EBED = 7,            /* discontinuous bed across an edge          */
    SWGPU_EBOUNDARY = 8,       /* unknown boundary type                     */
    SWGPU_EOVERSHOOT = 9,      /* model time overshot finaltime             */
    SWGPU_EMESH = 10,          /* inconsistent mesh arrays                  */
    SWGPU_ETIMEOUT = 11        /* a bounded device-side wait ran out; the   */
                               /* handle is unusable from then on: every    */
                               /* later call fails, destroy it              */
};

/* ---- precision of the evolve path ------------------------------------ */
enum swgpu_precision {
    SWGPU_FP64 = 0,   /* every operation in FP64, in the reference's order  */
    SWGPU_MIXED = 1   /* FP32 flux/limiter/extrapolation, FP64 update, depth
                         at wet/dry fronts, mass and model time             */
};

/* ---- timestepping methods (Domain.set_timestepping_method) ----------- */
enum swgpu_timestepping {
    SWGPU_EULER = 1,  /* forward Euler (the default)                       */
    SWGPU_RK2 = 2,    /* two-stage Runge-Kutta, Q = Q/2 + E(E(Q))/2         */
    SWGPU_RK3 = 3     /* three-stage strong-stability-preserving RK         */
};

/* ---- quantity ids (Domain.quantities keys) --------------------------- */
enum swgpu_quantity {
    SWGPU_STAGE = 0,
    SWGPU_XMOMENTUM = 1,
    SWGPU_YMOMENTUM = 2,
    SWGPU_ELEVATION = 3,
    SWGPU_FRICTION = 4,
    SWGPU_HEIGHT = 5,      /* derived: update_other_quantities */
    SWGPU_XVELOCITY = 6,   /* derived */
    SWGPU_YVELOCITY = 7    /* derived */
};

/* ---- boundary condition types ---------------------------------------- */
enum swgpu_boundary_type {
    SWGPU_BC_REFLECTIVE = 0,     /* anuga Reflective_boundary              */
    SWGPU_BC_DIRICHLET = 1,      /* anuga Dirichlet_boundary (w, uh, vh)   */
    SWGPU_BC_TIME_STAGE_SINE = 2, /* stage = p0 + p1*sin(2*pi*t/p2 + p3),
                                    momentum 0, t = model time             */
    SWGPU_BC_TRANSMISSIVE = 3,   /* anuga Transmissive_boundary: the inside
                                    edge's stage and momentum              */
    SWGPU_BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM = 4, /* anuga
                                    Transmissive_stage_zero_momentum_boundary */
    SWGPU_BC_INFLOW_HYDROGRAPH = 5, /* triangular hydrograph of unit discharge
                                    q(t) (p0 peak in m^2/s, p1 rise, p2 fall,
                                    p3 start time) entering along the inward
                                    normal; stage the inside edge's, or
                                    critical depth (q^2/g)^(1/3) above the
                                    edge bed where higher; no reference
                                    counterpart                            */
    SWGPU_BC_TIME_STAGE_FOURIER = 6 /* stage = p0 + p1*sin(wt) + p2*cos(wt)
                                    + p3*sin(2wt) + p4*cos(2wt), w =
                                    2*pi/p5, momentum 0, t = model time (an
                                    ANUGA Time_boundary of that function)  */
};

typedef struct {
    int64_t type;      /* swgpu_boundary_type */
    double p[8];       /* parameters, see swgpu_boundary_type (unused
                          entries ignored) */
} swgpu_boundary_tag;

/* Mesh arrays (anuga Mesh / struct domain in src/anuga_HMPP/sw_domain.h:16-180).
 * neighbours[3k+i] = triangle across edge i, or -(m+1) for boundary slot m.
 * surrogate_neighbours = neighbours with boundary entries replaced by k.
 * tri_full_flag may be NULL (all triangles full). */
typedef struct {
    int64_t number_of_elements;
    int64_t number_of_boundary_elements;
    const int64_t *neighbours;            /* [3N] */
    const int64_t *neighbour_edges;       /* [3N] */
    const int64_t *surrogate_neighbours;  /* [3N] */
    const int64_t *number_of_boundaries;  /* [N]  */
    const int64_t *tri_full_flag;         /* [N] or NULL */
    const double *normals;                /* [6N] */
    const double *edgelengths;            /* [3N] */
    const double *radii;                  /* [N]  */
    const double *areas;                  /* [N]  */
    const double *vertex_coordinates;     /* [6N] */
    const double *centroid_coordinates;   /* [2N] */
    const int64_t *boundary_cells;        /* [Nb] triangle of boundary slot m */
    const int64_t *boundary_edges;        /* [Nb] edge of boundary slot m     */
    const int64_t *boundary_tag;          /* [Nb] index into the tag table    */
} swgpu_mesh;

/* ANUGA numerical parameters (Domain attributes; the reference reads the
 * same set, src/anuga_HMPP/sw_domain_fun.h:57-120). */
typedef struct {
    double g;
    double epsilon;
    double H0;
    double minimum_allowed_height;
    double maximum_allowed_speed;
    double beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry;
    double alpha_balance;
    double CFL;
    double evolve_max_timestep;
    double evolve_min_timestep;
    int64_t tight_slope_limiters;
    int64_t use_centroid_velocities;
    int64_t optimise_dry_cells;
    int64_t extrapolate_velocity_second_order;
    int64_t use_sloped_mannings;
    int64_t max_smallsteps;
    int64_t default_order;
    int64_t optimised_gradient_limiter;  /* nonzero: extrapolate_second_order_sw
                                            (the default); 0: per-quantity
                                            limit by vertex (FP64 only) */
    int64_t use_edge_limiter;            /* nonzero: per-quantity limit by edge
                                            (FP64 only; gpu_domain_advanced.py:
                                            1815-1860) */
    int64_t flow_algorithm;              /* 0: the default distribute; 1: the
                                            'tsunami' one (protect_swb2 + edge
                                            extrapolation, no balance; :1755-1812;
                                            FP64 only) */
} swgpu_params;

/* Evolve state kept on the device (Domain time bookkeeping,
 * gpu_domain_advanced.py:2476-2675). */
typedef struct {
    double time;
    double yieldtime;
    double finaltime;          /* <= 0: none */
    double timestep;           /* last dt */
    double flux_timestep;      /* last CFL flux timestep (before CFL factor) */
    double recorded_max_timestep;
    double recorded_min_timestep;
    int64_t order;             /* current _order_ */
    int64_t smallsteps;
    int64_t number_of_steps;   /* since last yield */
    int64_t total_steps;       /* since evolve_start */
    int64_t stop_reason;       /* 0 none, 1 yield, 2 finaltime, 3 step budget, 4 error */
    int64_t status;            /* swgpu_status of a device-side failure */
} swgpu_state;

/* ---- lifetime --------------------------------------------------------- */

/* Allocates the device copy of the mesh and all quantity arrays on the
 * current CUDA device and renumbers nothing (the caller's triangle order is
 * kept).  Replaces allocate_device_array + asynchronous_transfer
 * (gpu_domain_advanced.py:582-903) and equip_kernel_functions (:186-507). */
int swgpu_create(const swgpu_mesh *mesh, const swgpu_params *params,
                 int precision, void **handle_out);

/* Batched ensemble: nscen independent scenarios in one handle, advanced
 * together by one device-resident loop (one graph of fused steps over all
 * of them), each with its own time, timestep, yield/final times and stop
 * state.  mesh is the scenarios' meshes concatenated: scenario s owns
 * triangles [scenario_offsets[s], scenario_offsets[s+1]) (offsets[0] = 0,
 * offsets[nscen] = number_of_elements, every offset a multiple of 256 --
 * pad a scenario with isolated triangles), its neighbour, surrogate and
 * boundary indices are global, and no triangle has a neighbour in another
 * scenario.  Boundary tags and quantities are set with the single-domain
 * calls on the concatenated arrays.  Per-method calls that reduce a single
 * timestep (compute_fluxes, update_conserved_quantities) are refused.  No
 * counterpart in the reference (which runs one domain per process). */
int swgpu_create_ensemble(const swgpu_mesh *mesh, const int64_t *scenario_offsets, int nscen,
                          const swgpu_params *params, int precision, void **handle_out);

/* Number of scenarios of a handle (1 for swgpu_create handles). */
int swgpu_ensemble_size(void *handle, int *nscen);

/* Evolve state of one scenario (swgpu_get_state reads scenario 0). */
int swgpu_ensemble_get_state(void *handle, int scenario, swgpu_state *state);

/* Per-scenario finaltime (<= 0: none) after swgpu_evolve_start, which gives
 * every scenario the same one.  swgpu_evolve_run then returns when every
 * scenario has stopped (final time, yield, step budget or error). */
int swgpu_ensemble_set_finaltimes(void *handle, const double *finaltimes);

/* Water volume of each scenario, each equal to swgpu_mass of that scenario
 * run alone. */
int swgpu_ensemble_mass(void *handle, double *masses);

/* Launch shape of the fused evolve step: the autotuner's knobs.  Results do
 * not depend on it (every per-triangle operation and every reduction order
 * is the same for every shape).  flux_block: threads per block of the FP64
 * flux, or triangles per TMA tile of the mixed flux (64, 128, 256);
 * update_block, distribute_block: 128, 256 or 512 (at most 256 for an
 * ensemble); steps_per_graph: 1..64 steps captured per CUDA graph.  No
 * counterpart in the reference (its block sizes are fixed per kernel,
 * gpu_domain_advanced.py:186-507). */
typedef struct {
    int32_t flux_block;
    int32_t update_block;
    int32_t distribute_block;
    int32_t steps_per_graph;
    int32_t flux_pipelined;   /* mixed flux: persistent blocks, double-buffered TMA
                                 tiles (flux_block 64 or 128) */
    int32_t dependent_launch; /* mixed kernels: each step kernel is launched as a
                                 programmatic dependent of the previous one, so
                                 its blocks start (and fetch the static planes)
                                 during that kernel's last wave */
} swgpu_launch_config;

int swgpu_get_launch_config(void *handle, swgpu_launch_config *config);
int swgpu_set_launch_config(void *handle, const swgpu_launch_config *config);

/* Per-triangle tracking over the device-resident loop: the maximum depth
 * since the call and the first model time (end of a whole step) at which
 * the depth exceeded threshold (-1: not yet).  on = 0 stops tracking.  The
 * targets of the surrogate model; no counterpart in the reference. */
int swgpu_set_tracking(void *handle, int on, double threshold);
int swgpu_get_tracking(void *handle, float *max_depth, float *arrival_time);

/* ---- BF16 MLP surrogate (swgpu_mlp_*) ---------------------------------
 * A 16 -> 256 -> 256 -> 256 -> 3 ReLU network predicting per (scenario,
 * triangle) row the normalised maximum depth, the normalised arrival time
 * and the 90% quantile of the first output's absolute error, from 9 scenario
 * parameters and the triangle's centroid, bed and distance to the inflow.
 * BF16 weights and activations, FP32 accumulation; every layer of width
 * 256 runs as tcgen05.mma tiles (128 rows x 256 units) accumulating in
 * tensor memory, in the forward and the backward pass; FP32 master weights
 * trained by Adam.  params is the flat FP32 vector W1 [16][256], b1 [256],
 * W2 [256][256], b2, W3 [256][256], b3, W4 [256][3], b4 [3]
 * (swgpu_mlp_num_params() floats, in-major weights); the feature map is
 * (raw - mean) * inv_std over 16 features (the last 3 are zero).  Handles
 * use the current device and their own stream; a handle whose kernel
 * reports SWGPU_ETIMEOUT is unusable (every later call fails).  No
 * counterpart in the reference. */
int swgpu_mlp_num_params(void);
int swgpu_mlp_create(const float *params, const float *feature_mean,
                     const float *feature_inv_std, void **mlp_out);
int swgpu_mlp_destroy(void *mlp);
const char *swgpu_mlp_last_error(void *mlp);
/* tri [ntri][4]: centroid x, y, bed and distance to the inflow; scen
 * [nscen][9]; targets [nscen][ntri][2] (normalised depth and arrival; may
 * be NULL for prediction only). */
int swgpu_mlp_set_data(void *mlp, const float *tri, int64_t ntri, const float *scen,
                       int64_t nscen, const float *targets);
/* rows row0 .. row0+nrows-1 (row = scenario * ntri + triangle) into a
 * DEVICE buffer out [nrows][3]; *elapsed_ms (may be NULL) = device time. */
int swgpu_mlp_predict(void *mlp, int64_t row0, int64_t nrows, float *out_device,
                      float *elapsed_ms);
/* Outputs [nrows][3], gradient of the loss (flat like params) and loss of
 * the given rows, without updating: mean over rows of
 * w_depth (y0 - t0)^2 + w_arrival (y1 - t1)^2 + w_error rho(|y0 - t0| - y2),
 * rho(u) = u (0.9 - [u < 0]) the pinball loss of the 90% quantile, with
 * |y0 - t0| held constant (the error estimate learns that quantile of the
 * depth output's error without changing it). */
int swgpu_mlp_gradients(void *mlp, const int64_t *rows, int64_t nrows, float w_depth,
                        float w_arrival, float w_error, float *outputs, float *grad,
                        float *loss);
/* steps Adam steps on random batches of batch rows (seeded). */
int swgpu_mlp_train(void *mlp, int steps, int64_t batch, uint64_t seed, float lr,
                    float w_depth, float w_arrival, float w_error, float *last_loss,
                    float *elapsed_ms);
int swgpu_mlp_get_params(void *mlp, float *params);

/* Frees everything the handle owns.  No counterpart in the reference (its
 * PyCUDA allocations are released by the garbage collector). */
int swgpu_destroy(void *handle);

/* Message for the last failing call on this handle (never NULL). */
const char *swgpu_last_error(void *handle);

/* Device and build description, e.g. "NVIDIA GB300 sm_103 (libswgpu 1)". */
int swgpu_device_info(char *buf, int buflen);

/* ---- quantities and boundaries --------------------------------------- */

/* Uploads one quantity (Quantity.set_values + the H2D copy of
 * asynchronous_transfer).  centroid may not be NULL; vertex / edge may be
 * NULL (left unchanged).  Uploading stage or momentum marks the vertex and
 * edge values stale until the next distribute. */
int swgpu_set_quantity(void *handle, int quantity, const double *centroid,
                       const double *vertex, const double *edge);

/* Downloads one quantity (the reference's copy_back path).  Any output
 * pointer may be NULL.  Derived quantities (height, velocities) are
 * computed on demand from the conserved ones (update_other_quantities,
 * gpu_domain_advanced.py:2114-2151). */
int swgpu_get_quantity(void *handle, int quantity, double *centroid,
                       double *vertex, double *edge);

/* Boundary values of slot m for stage/xmomentum/ymomentum/elevation, and
 * for height/xvelocity/yvelocity as of the last
 * swgpu_update_other_quantities. */
int swgpu_get_boundary_values(void *handle, int quantity, double *out);

/* explicit_update (stage/xmom/ymom) or semi_implicit_update (xmom/ymom). */
int swgpu_get_explicit_update(void *handle, int quantity, double *out);

/* max_speed per triangle from the last swgpu_compute_fluxes (FP64 handles;
 * the copy_back of gpu_domain_advanced.py:923 for the degenerate-timestep
 * protection). */
int swgpu_get_max_speed(void *handle, double *out);
int swgpu_get_semi_implicit_update(void *handle, int quantity, double *out);

/* Installs the boundary tag table (Domain.set_boundary).  Every tag index
 * used by mesh->boundary_tag must be < ntags. */
int swgpu_set_boundary_tags(void *handle, const swgpu_boundary_tag *tags,
                            int ntags);

/* ---- per-method entry points (gpu_domain_advanced.py) ---------------- */

/* protect_against_infinitesimal_and_negative_heights (:1003-1055). */
int swgpu_protect(void *handle);

/* distribute_to_vertices_and_edges (:1744-2001): protect, extrapolation of
 * the current order (extrapolate_second_order_sw :1061-1161 or
 * extrapolate_first_order), balance_deep_and_shallow (:957-995) and
 * interpolate_from_vertices_to_edges (:1975-1986). */
int swgpu_distribute_to_vertices_and_edges(void *handle);

/* update_boundary (:2006-2108), evaluated at the handle's model time. */
int swgpu_update_boundary(void *handle);

/* compute_fluxes (:1595-1696): central-upwind flux and gravity_wb into
 * explicit_update; returns the minimum flux timestep (the host min of the
 * reference's timestep_array, :1684) in *flux_timestep. */
int swgpu_compute_fluxes(void *handle, double *flux_timestep);

/* compute_forcing_terms -> manning_friction_implicit (:1255-1324). */
int swgpu_compute_forcing_terms(void *handle);

/* manning_friction_explicit (:1330-1388): the same Manning friction term
 * S * momentum added to the explicit updates of x and y momentum (FP64
 * handles). */
int swgpu_manning_friction_explicit(void *handle);

/* extrapolate_second_order_sw (:1061-1161): centroid velocities (when
 * extrapolate_velocity_second_order) and the limited second-order
 * reconstruction of stage and momentum at the vertices, with no protect
 * and no balance; vertex values only (FP64 handles, default flow
 * algorithm). */
int swgpu_extrapolate_second_order_sw(void *handle);

/* balance_deep_and_shallow (:957-995) on the current vertex values (FP64
 * handles). */
int swgpu_balance_deep_and_shallow(void *handle);

/* update_conserved_quantities (:1412-1442) with the given dt. */
int swgpu_update_conserved_quantities(void *handle, double timestep);

/* update_other_quantities (:2114-2151) materialised for download. */
int swgpu_update_other_quantities(void *handle);

/* backup_conserved_quantities (:1449-1478): device copies of the centroid
 * stage, xmomentum and ymomentum (FP64 handles). */
int swgpu_backup_conserved_quantities(void *handle);

/* saxpy_conserved_quantities (:1484-1519; kernel
 * saxpy_centroid_values/saxpy_centroid_values.cu:1-12):
 * Q = a*Q + b*backup for the three conserved quantities (FP64 handles). */
int swgpu_saxpy_conserved_quantities(void *handle, double a, double b);

/* Domain.set_timestepping_method (numbered as src/utilities/utility.py:
 * 256-261): the steps of swgpu_evolve_run / swgpu_evolve_one_step become
 * ANUGA's evolve_one_euler_step, evolve_one_rk2_step or evolve_one_rk3_step
 * (dispatched at gpu_domain_advanced.py:2566-2573), every stage of an RK step
 * with the timestep chosen by its first. */
int swgpu_set_timestepping_method(void *handle, int method);

/* Total water volume sum(area*(stage-elevation)) (FP64 reduction). */
int swgpu_mass(void *handle, double *mass);

/* ---- evolve (the device-resident loop) ------------------------------- */

/* Read / overwrite the device-side time bookkeeping (set_time, _order_,
 * yieldtime, ...). */
int swgpu_get_state(void *handle, swgpu_state *state);
int swgpu_set_state(void *handle, const swgpu_state *state);

/* The set-up half of Domain.evolve (:2476-2551): distribute, time reset,
 * counters, second distribute, update_boundary. */
int swgpu_evolve_start(void *handle, double starttime, double yieldstep,
                       double finaltime);

/* The hot loop of Domain.evolve (:2555-2675): Euler steps with the
 * timestep computed on the device, until the next yield time, the final
 * time, or max_steps steps (max_steps <= 0: no limit).  Steps run as CUDA
 * graphs of several steps; the host synchronises only between graphs.
 * On return *state holds the device state; stop_reason says why it
 * stopped.  After a yield, call again to continue (the library advances
 * yieldtime by yieldstep). */
int swgpu_evolve_run(void *handle, int64_t max_steps, swgpu_state *state);

/* One Euler step exactly as evolve_one_euler_step (:2178-2191) followed
 * by the time update, distribute and update_boundary of the loop body,
 * issued kernel by kernel without a graph (for tests and co-testing). */
int swgpu_evolve_one_step(void *handle, swgpu_state *state);

/* swgpu_evolve_run with CUDA events recorded on the handle's stream before
 * the first and after the last graph of the run: *elapsed_ms is the device
 * time of the whole run.  No reference counterpart (the reference times its
 * evolve loop with host clocks, gpu_domain_advanced.py:2418-2436, 2678-2688). */
int swgpu_evolve_run_timed(void *handle, int64_t max_steps, swgpu_state *state,
                           double *elapsed_ms);

/* Runs nsteps Euler steps kernel by kernel (no graph) with a CUDA event
 * around each kernel and returns the summed device time of each: ms[0]
 * flux + gravity, ms[1] update, ms[2] extrapolation/balance/boundary, ms[3]
 * the mixed path's step clock (0 for FP64 handles, whose flux kernel
 * evaluates the clock itself); ms holds 4 doubles.  For per-kernel
 * rooflines.  No reference counterpart (the reference's per-kernel times
 * come from the legacy command-line profiler). */
int swgpu_profile_steps(void *handle, int64_t nsteps, double *ms);

/* Synchronises the handle's stream. */
int swgpu_synchronize(void *handle);

/* ---- allocation-free entry point -------------------------------------- */

/* Water volume sum(areas[k] * (stage[k] - elevation[k])), k < n, written to
 * *volume, for callers that cannot allocate device memory when they need it:
 * code running inside a CUDA stream capture (cudaMalloc is not capturable),
 * code whose device memory belongs to a pool it does not control, and
 * time-critical loops that must avoid cudaMalloc's implicit synchronisation.
 * No counterpart in the reference.
 *
 * All five pointers are DEVICE pointers owned by the caller; stream may be
 * NULL (the legacy default stream).  The call only enqueues work: *volume is
 * ready when the stream reaches it.  It allocates nothing: its scratch is a
 * 128 KiB file-scope __device__ array that every GPU loading the library
 * holds until the process exits, which limits n to 4,194,304 (larger n:
 * SWGPU_EINVAL).  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  All calls on a device share the one
 * array, so calls that overlap on the GPU (different streams or threads
 * without ordering) race; calls ordered on one stream do not.  The sum is
 * taken in swgpu_mass's order: given an FP64 handle's own centroid arrays in
 * that handle's triangle order, the result is bit-identical to its
 * swgpu_mass (a mixed-precision handle's swgpu_mass sums area times its FP64
 * depth instead).  A CUDA error already pending when the call is made is
 * reported (SWGPU_ECUDA) and left pending; nothing is launched.  The scratch
 * address belongs to the device's context at the first call: do not call
 * cudaDeviceReset afterwards.  Errors: swgpu_last_error(NULL). */
int swgpu_water_volume_noalloc(const double *areas, const double *stage,
                               const double *elevation, int64_t n, double *volume,
                               void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SWGPU_H */
