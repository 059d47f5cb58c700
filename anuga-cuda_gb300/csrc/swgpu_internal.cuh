// swgpu_internal.cuh -- device data structures shared by the evolve kernels
// and the C ABI layer of libswgpu.so.
//
// Device layout (HBM): every per-triangle array is structure-of-arrays with
// triangle index fastest, so a warp's 32 consecutive triangles read 32
// consecutive words.  Per-edge / per-vertex data are three planes of N
// ([i*N + k] for edge or vertex i of triangle k); normals and vertex
// coordinates are six planes ([2i*N + k] = x, [(2i+1)*N + k] = y).
// Indices are int32.  The caller's triangle order is kept; meshes built by
// anuga_cuda.mesh are already Morton ordered so neighbour gathers stay local.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "swgpu.h"

namespace swgpu {

constexpr int kBlock = 256;

// neighbour packing: interior edge -> (n << 2) | m (m = edge index in n);
// boundary edge -> -(slot + 1), as in ANUGA's neighbours array.
__host__ __device__ inline int pack_neighbour(int n, int m) { return (n << 2) | m; }

// Threads per block of the fused-step kernels (the autotuner's knobs;
// results do not depend on them).  flux: FP64 block size, or the mixed
// flux's TMA tile (64, 128, 256); update, distribute: 128, 256 or 512.
struct LaunchShape {
    int flux, update, distribute;
    int pipelined;  // mixed flux: persistent double-buffered blocks (tiles of 64 or 128)
    int sms;        // multiprocessors of the device (persistent grid size)
    int pdl;        // mixed kernels launched as programmatic dependents of the previous one
};

struct DevMesh {
    int N, Nb;
    int n_launch;  // triangles the fused-step kernels are launched over: N, or for an
                   // ensemble the scenarios still running (they come first)
    LaunchShape shape;
    const int *nbr;            // [3][N] packed neighbour / boundary slot
    const int *surr;           // [3][N] surrogate neighbours
    const uint8_t *nb;         // [N] number_of_boundaries
    const uint8_t *order;      // [N] flux summation order (2 bits per position)
    const uint8_t *full;       // [N] tri_full_flag
    const double *normals;     // [6][N]
    const double *len;         // [3][N]
    const double *radii;       // [N]
    const double *areas;       // [N]
    const double *vxy;         // [6][N]
    const double *cxy;         // [2][N]
    const int *bcell, *bedge, *btag;   // [Nb]
    // ensembles: scenario of each 256-triangle block (scenarios start on
    // 256-triangle boundaries); nullptr for a single mesh
    const int *blk_scen;
};

// FP64 state (both precisions keep the conserved centroid state in FP64).
struct DevState {
    double *w, *uh, *vh, *zc, *fric;          // [N] centroid values
    double *uvel, *vvel;                      // [N] centroid velocities (extrapolation input)
    double *wv, *uhv, *vhv, *zv, *ze;         // [3][N] vertex values; bed edge values
    double *we, *uhe, *vhe;                   // [3][N] edge values (materialised on demand)
    double *wb, *uhb, *vhb, *zb;              // [Nb] boundary values
    double *ew, *euh, *evh;                   // [N] explicit_update
    double *suh, *svh;                        // [N] semi_implicit_update
    double *max_speed;                        // [N]
    double *hc, *uc, *vc;                     // [N] derived centroid quantities
    double *hb, *ub, *vb;                     // [Nb] derived boundary quantities
    double *partials;                         // [grid] reduction scratch
    float *hmax, *tarr;                       // [N] tracking: maximum depth since reset,
                                              // first time depth exceeded the threshold
                                              // (negative: not yet); null when off
    double *bw, *buh, *bvh;                   // [N] backups of the conserved state for
                                              // Runge-Kutta steps (bw: stage in FP64,
                                              // depth in the mixed precision)
};

// Mixed-precision state.  The conserved state is FP64 depth h = w - z (so
// depth at wet/dry fronts never comes from a difference of two large
// stages) and FP64 momentum.  Everything the flux, limiter and
// extrapolation read is FP32 and, where the shallow-water terms cancel,
// stored as a deviation: centroid stage and depth, edge STAGE JUMPS from
// the centroid (not absolute edge values), and bed offsets from the
// centroid bed, so that hydrostatic pressure and bed-slope terms never
// subtract two large FP32 numbers.
struct DevMixed {
    int S;                         // stride of the padded planes: N rounded up to 64, so
                                   // that every plane and every tile of 64-512 triangles
                                   // starts on a multiple of 64 elements (TMA-aligned)
    double *hd;                    // [N] FP64 depth (conserved)
    float2 *ws;                    // [S] centroid stage as an FP32 pair, x hi + y lo
    float *hf;                     // [S] centroid depth
    float2 *vel;                   // [S] centroid velocities, x u + y v
    float4 *es;                    // [3][S] edge state: x depth, y stage jump from the
                                   // centroid, z/w momentum (one 16-byte load per edge)
    float *hbf, *uhbf, *vhbf;      // [Nb] boundary depth and momentum
    float *wjb;                    // [Nb] boundary stage minus the owner's edge stage
    float2 *ewu;                   // [S] explicit_update of depth (x) and x momentum (y)
    float *evh;                    // [S] explicit_update of y momentum
    float2 *nrm;                   // [3][S] unit normals (x, y)
    int2 *lnb;                     // [3][S] per edge: x the length (float bits), y the packed
                                   // neighbour of DevMesh::nbr
    float2 *rad;                   // [S] x radius, y 1/area
    float2 *gc;                    // [3][S] vertex-jump coefficients of vertex i (dq1, dq2)
    float *dzv;                    // [3][S] bed vertex minus bed centroid
    float *dze;                    // [3][S] bed edge minus bed centroid
    float4 *ust;                   // [S] the update's static data: x Manning n, y mean(bed
                                   // vertex) minus bed centroid, z/w bed centroid as an
                                   // FP32 pair hi + lo

    int *surrp;                    // [3][S] DevMesh::surr in padded planes (TMA-staged)
    uint8_t *kind;                 // [S] 0 aux triangle, 1 one neighbour (slot<<2), 2 flat;
                                   // | 16: the triangle has a boundary edge
};

struct DevParams {
    double g, epsilon, H0, minimum_allowed_height, maximum_allowed_speed;
    double beta_w, beta_w_dry, beta_uh, beta_uh_dry, beta_vh, beta_vh_dry;
    double alpha_balance, CFL, evolve_max_timestep, evolve_min_timestep;
    int tight_slope_limiters, use_centroid_velocities, optimise_dry_cells;
    int extrapolate_velocity_second_order, use_sloped_mannings;
    int max_smallsteps, default_order;
    int limiter;  // kLimiterOptimised, kLimiterVertex or kLimiterEdge
    int flow_algorithm;  // 0 default, 1 'tsunami' (protect_swb2 + edge extrapolation)
    double track_threshold;  // depth that counts as arrival
    // FP32 copies for the mixed kernels (set on the host; FP64 arithmetic
    // on GB300 runs at 1/64 of the FP32 rate, so none is done per thread)
    float f_g, f_eps, f_H0, f_h0, f_lim, f_mah, f_mas, f_max_dt, f_alpha;
    float f_beta_w, f_beta_w_dry, f_beta_uh, f_beta_uh_dry, f_beta_vh, f_beta_vh_dry;
};

struct BcTag {
    int type;
    double p[8];
};

// Whole-run summary for the host's polling: how many scenarios (Ctrl
// blocks) have halted, and the first device status among them.
struct RunSummary {
    int halted;
    int status;
};

// Device-resident evolve bookkeeping, one per scenario.  FP64 path: written by the
// last block of the update kernel (time, order, counters) and the last block of
// the distribute kernel (halt).  Mixed path: the step clock kernel publishes the
// clock, the first block of the scenario in the distribute commits the stage.
// Read by every kernel at entry.
struct __align__(16) Ctrl {
    unsigned long long ftmin_bits;  // minimum flux timestep of this step (bits of a positive double)
    double time, yieldtime, finaltime, yieldstep, timestep, flux_timestep;
    double rec_max, rec_min, time_epsilon;
    long long order, smallsteps, steps_since_yield, total_steps;
    long long budget;               // steps left in this run; < 0 = unlimited
    int halt;                       // nonzero: kernels return at entry
    int halt_pending;               // stop reason raised by update, applied after distribute
    int stop_reason;
    int status;                     // first device-side failure (swgpu_status)
    unsigned int done_update, done_distribute, done_flux;
    int clk_small_error;            // the step's update_timestep, evaluated once
    double clk_dt, clk_ftmin;       // after the flux grid (FP64: its last block;
    long long clk_order, clk_smallsteps;  // mixed: step_clock_mixed) and read by
                                          // the update and distribute kernels
    double clk_t0;                  // model time when that clock was evaluated
    double step_t0;                 // time at the start of a Runge-Kutta step
    unsigned int blocks_flux;       // blocks of this scenario in one flux launch
    unsigned int blocks_update;     // ... in one update launch
    unsigned int blocks_distribute; // ... in one distribute launch
    RunSummary *summary;            // shared by all scenarios of a handle
    unsigned int *halt_bits;        // one bit per scenario, set when it halts
    int scen;                       // this scenario's index
};

enum StopReason { kStopNone = 0, kStopYield = 1, kStopFinal = 2, kStopBudget = 3, kStopError = 4 };

// Kernel option flags
enum : int {
    kFused = 1,           // part of the device-resident loop (reads/writes Ctrl)
    kWriteEdges = 2,      // distribute materialises edge values
    kWriteBoundary = 4,   // distribute evaluates boundary conditions
    kFrictionInline = 8,  // update computes Manning friction itself
    kWriteMaxSpeed = 16,  // flux writes max_speed
    kNoTimestep = 32,     // flux skips the timestep reduction (later Runge-Kutta stages)
    kTrack = 64,          // update records maximum depth and arrival time (whole steps)
    kExtrapolateOnly = 128,  // FP64 distribute: the second-order extrapolation alone
                             // (extrapolate_second_order_sw), no balance, vertex values only
};

// One stage of a fused step.  An Euler step is one stage; ANUGA's RK2 and
// RK3 steps (Generic_Domain.evolve_one_rk2_step / evolve_one_rk3_step) are
// two and three Euler stages that all use the dt chosen by the first, with
// Q = a*Q + b*backup after the later ones.
enum StageKind : int {
    kStageEuler = 0,  // the whole step: commit it
    kStageFirst = 1,  // back up Q before the update; then time = t0 + dt
    kStageMid = 2,    // Q = a*Q + b*backup; then time = t0 + tfrac*dt
    kStageLast = 3,   // Q = a*Q + b*backup; commit the step (time = t0 + dt)
};
struct Stage {
    int kind;
    double a, b, tfrac;
};
constexpr Stage kEulerStage = {kStageEuler, 1.0, 0.0, 1.0};

// second-order reconstruction of distribute_to_vertices_and_edges
// (gpu_domain_advanced.py:1815-1943)
enum Limiter : int {
    kLimiterOptimised = 0,  // extrapolate_second_order_sw (optimised_gradient_limiter)
    kLimiterVertex = 1,     // per quantity, extrapolate_second_order_and_limit_by_vertex
    kLimiterEdge = 2,       // per quantity, ..._and_limit_by_edge (use_edge_limiter)
};

__host__ __device__ inline double pos_inf() { return 1.0e300 * 1.0e300; }

// ---------------------------------------------------------------- launches
// FP64 path (swgpu_fp64.cu)
void launch_prepare_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                         Ctrl *ctrl, cudaStream_t st);
void launch_distribute_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                            const BcTag *tags, Ctrl *ctrl, int flags, cudaStream_t st);
void launch_boundary_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                          const BcTag *tags,
                          Ctrl *ctrl, cudaStream_t st);
void launch_flux_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                      Ctrl *ctrl, int flags, cudaStream_t st);
// Manning friction (S * momentum) added to the semi-implicit updates, or with
// explicit_target to the explicit updates (manning_friction_explicit)
void launch_forcing_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                         bool explicit_target, cudaStream_t st);
// centroid velocities uh / max(h, minimum_allowed_height) alone (the head of
// the stand-alone extrapolate_second_order_sw; no protect)
void launch_velocities_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                            cudaStream_t st);
// balance_deep_and_shallow on the stored vertex values
void launch_balance_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                         cudaStream_t st);
void launch_update_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                        Ctrl *ctrl, double dt, int flags, const Stage &stage,
                        cudaStream_t st);
// tracking arrays to (0, -1)
void launch_track_reset(const DevMesh &M, const DevState &S, cudaStream_t st);
// saxpy_conserved_quantities: Q = a*Q + b*backup for stage and momenta
void launch_saxpy_fp64(const DevMesh &M, const DevState &S, double a, double b,
                       cudaStream_t st);
void launch_interpolate_fp64(const DevMesh &M, const DevState &S, cudaStream_t st);
void launch_other_quantities(const DevMesh &M, const DevState &S, cudaStream_t st);
void launch_mass(const DevMesh &M, const DevState &S, double *out, cudaStream_t st);
// one volume partial per 256-triangle block into S.partials
void launch_mass_partials(const DevMesh &M, const DevState &S, cudaStream_t st);

// Mixed path (swgpu_mixed.cu)
// with kFused, the stage `stage` is committed by the distribute (see
// distribute_mixed); stand-alone calls pass kEulerStage
void launch_distribute_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                             const DevParams &P, const BcTag *tags, Ctrl *ctrl,
                             int flags, const Stage &stage, cudaStream_t st);
void launch_flux_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                       const DevParams &P, Ctrl *ctrl, int flags, cudaStream_t st);
// the step's clock from the fused mixed flux's minimum, per scenario;
// launched between that flux and the update of a stage that takes a new dt
void launch_step_clock_mixed(const DevParams &P, Ctrl *ctrl, int nscen, bool pdl,
                             cudaStream_t st);
void launch_update_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                         const DevParams &P, Ctrl *ctrl, int flags, const Stage &stage,
                         cudaStream_t st);
// stand-alone distribute head: (optionally) depth from the FP64 stage, then
// protect and the FP32 centroid copies
void launch_prepare_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                          const DevParams &P, int from_stage, cudaStream_t st);
// FP64 stage / vertex / edge values from the mixed state, for downloads
void launch_vertices_from_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                                cudaStream_t st);
// FP64 centroid stage only (w = h + z), for centroid downloads and the
// derived quantities
void launch_stage_from_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                             cudaStream_t st);
void launch_mass_mixed(const DevMesh &M, const DevState &S, const DevMixed &X, double *out,
                       cudaStream_t st);
void launch_mass_partials_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                                cudaStream_t st);

inline int grid_for(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace swgpu
