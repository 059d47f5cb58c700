// swgpu_device.cuh -- device helpers shared by the FP64 and mixed kernels:
// comparisons with the reference's min/max semantics, the boundary
// condition formulas, the device-side update_timestep, last-block-done
// bookkeeping and the block minimum of the flux timestep.
#pragma once

#include "swgpu_internal.cuh"

namespace swgpu {

// src/anuga_HMPP/util_ext.h:45-59: plain comparisons, second argument on
// ties (so the sign of a zero result follows the reference, unlike fmax).
__device__ __forceinline__ double omax(double x, double y) { return x > y ? x : y; }
__device__ __forceinline__ double omin(double x, double y) { return x < y ? x : y; }
__device__ __forceinline__ float omaxf(float x, float y) { return x > y ? x : y; }
__device__ __forceinline__ float ominf(float x, float y) { return x < y ? x : y; }

__device__ __forceinline__ void set_status(Ctrl *ctrl, int code) {
    atomicCAS(&ctrl->status, 0, code);
}

// Unit discharge of a triangular hydrograph (peak, rise, fall, start): 0
// before start, linear to peak over rise, linear back to 0 over fall.
__device__ __forceinline__ double hydrograph(const double p[4], double t) {
    const double s = t - p[3];
    if (s <= 0.0) return 0.0;
    if (s < p[1]) return p[0] * (s / p[1]);
    if (s < p[1] + p[2]) return p[0] * (1.0 - (s - p[1]) / p[2]);
    return 0.0;
}

// Boundary value of one boundary edge from the owning triangle's edge
// values (reflective: src/anuga_cuda/evaluate_segment/evaluate_segment.cu:3-76;
// Dirichlet: :80-115; ANUGA's transmissive boundaries: the inside edge
// values, with or without momentum; the time-dependent stage and the inflow
// hydrograph and the Fourier stage have no reference GPU counterpart: the hydrograph's unit
// discharge q(t) enters along the inward normal with the inside edge's
// stage, or critical depth (q^2/g)^(1/3) above the edge bed ze where that
// is higher, i.e. on a dry or shallow edge).  Returns false for an unknown
// type.
__device__ __forceinline__ bool eval_boundary(const BcTag &T, double time, double we,
                                              double uhe, double vhe, double n1,
                                              double n2, double ze, double g, double &wb,
                                              double &uhb, double &vhb) {
    if (T.type == SWGPU_BC_REFLECTIVE) {
        const double r1 = -uhe * n1 - vhe * n2;
        const double r2 = -uhe * n2 + vhe * n1;
        wb = we;
        uhb = n1 * r1 - n2 * r2;
        vhb = n2 * r1 + n1 * r2;
        return true;
    }
    if (T.type == SWGPU_BC_DIRICHLET) {
        wb = T.p[0];
        uhb = T.p[1];
        vhb = T.p[2];
        return true;
    }
    if (T.type == SWGPU_BC_TIME_STAGE_SINE) {
        const double two_pi = 6.283185307179586;
        wb = T.p[0] + T.p[1] * sin(two_pi * time / T.p[2] + T.p[3]);
        uhb = 0.0;
        vhb = 0.0;
        return true;
    }
    if (T.type == SWGPU_BC_TIME_STAGE_FOURIER) {
        const double wt = 6.283185307179586 * time / T.p[5];
        wb = T.p[0] + T.p[1] * sin(wt) + T.p[2] * cos(wt) + T.p[3] * sin(2.0 * wt) +
             T.p[4] * cos(2.0 * wt);
        uhb = 0.0;
        vhb = 0.0;
        return true;
    }
    if (T.type == SWGPU_BC_TRANSMISSIVE) {
        wb = we;
        uhb = uhe;
        vhb = vhe;
        return true;
    }
    if (T.type == SWGPU_BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM) {
        wb = we;
        uhb = 0.0;
        vhb = 0.0;
        return true;
    }
    if (T.type == SWGPU_BC_INFLOW_HYDROGRAPH) {
        const double q = hydrograph(T.p, time);
        wb = omax(we, ze + cbrt(q * q / g));
        uhb = -q * n1;
        vhb = -q * n2;
        return true;
    }
    return false;
}

// Boundary types whose stage is the edge's own (no stage jump across the edge).
__host__ __device__ inline bool boundary_keeps_edge_stage(int type) {
    return type == SWGPU_BC_REFLECTIVE || type == SWGPU_BC_TRANSMISSIVE ||
           type == SWGPU_BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM;
}

// Snapshot of the time bookkeeping taken at kernel entry.
struct StepClock {
    double dt;          // timestep of this step
    double ftmin;       // flux timestep (minimum over edges)
    long long order;    // _order_ after this step's update_timestep
    long long smallsteps;
    int small_error;    // ran below the minimum step at order 1
};

// ANUGA Generic_Domain.update_timestep as restated in
// src/anuga_HMPP/evolve.c:115-160 (finaltime clamp as finaltime - time).
// Each block evaluates it on the same snapshot and gets the same dt.
__device__ __forceinline__ StepClock device_update_timestep(const Ctrl *c, const DevParams &P) {
    StepClock s;
    s.ftmin = __longlong_as_double((long long)c->ftmin_bits);
    double dt = omin(P.CFL * s.ftmin, P.evolve_max_timestep);
    s.order = c->order;
    s.smallsteps = c->smallsteps;
    s.small_error = 0;
    if (dt < P.evolve_min_timestep) {
        s.smallsteps += 1;
        if (s.smallsteps > P.max_smallsteps) {
            s.smallsteps = 0;
            if (s.order == 1) {
                dt = P.evolve_min_timestep;
                s.small_error = 1;
            } else {
                s.order = 1;
            }
        }
    } else {
        s.smallsteps = 0;
        if (s.order == 1 && P.default_order == 2) s.order = 2;
    }
    if (c->finaltime > 0 && c->time + dt > c->finaltime) dt = c->finaltime - c->time;
    if (c->time + dt > c->yieldtime) dt = c->yieldtime - c->time;
    s.dt = dt;
    return s;
}

// The step's clock as published by publish_step_clock.
__device__ __forceinline__ StepClock published_step_clock(const Ctrl *c) {
    StepClock s;
    s.dt = c->clk_dt;
    s.ftmin = c->clk_ftmin;
    s.order = c->clk_order;
    s.smallsteps = c->clk_smallsteps;
    s.small_error = c->clk_small_error;
    return s;
}

// The control block of the scenario that owns this block's triangles
// (the block's first triangle is blockIdx.x * blockDim.x).
__device__ __forceinline__ Ctrl *block_ctrl(Ctrl *base, const DevMesh &M) {
    return M.blk_scen ? base + M.blk_scen[(blockIdx.x * blockDim.x) >> 8] : base;
}

// Called by thread 0 of each block after the block's work; returns true in
// exactly one of the scenario's `blocks` blocks, the last to finish (all
// other blocks' writes are then visible).  The counter is reset for the
// next launch.
__device__ __forceinline__ bool last_block_done(unsigned int *counter, unsigned int blocks) {
    __threadfence();
    const unsigned int prev = atomicAdd(counter, 1u);
    if (prev == blocks - 1) {
        __threadfence();
        *counter = 0;
        return true;
    }
    return false;
}

// Once all atomicMins of the step are done (FP64: the flux kernel's last
// block; mixed: step_clock_mixed, after the flux grid): evaluate
// update_timestep once and publish it for the update kernel.
__device__ __forceinline__ void publish_step_clock(Ctrl *c, const DevParams &P) {
    const StepClock s = device_update_timestep(c, P);
    c->clk_dt = s.dt;
    c->clk_ftmin = s.ftmin;
    c->clk_order = s.order;
    c->clk_smallsteps = s.smallsteps;
    c->clk_small_error = s.small_error;
    c->clk_t0 = c->time;
}

// Block-wide minimum of a positive double, then one atomicMin on its bit
// pattern (positive IEEE doubles order like their bits) only when it lowers
// the running minimum.  In the fused loop the last block then publishes the
// step's clock.
template <int BLOCK = kBlock>
__device__ __forceinline__ void block_min_timestep(double t, Ctrl *ctrl) {
    __shared__ double wmin[BLOCK / 32];
    for (int o = 16; o > 0; o >>= 1) t = omin(t, __shfl_xor_sync(0xffffffffu, t, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmin[warp] = t;
    __syncthreads();
    if (warp == 0) {
        t = lane < (int)(blockDim.x >> 5) ? wmin[lane] : pos_inf();
        for (int o = 16; o > 0; o >>= 1) t = omin(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (lane == 0) {
            const unsigned long long bits = (unsigned long long)__double_as_longlong(t);
            if (!(t >= 0.0)) {
                set_status(ctrl, SWGPU_ENONFINITE);  // NaN reached the timestep
            } else if (bits < *(volatile unsigned long long *)&ctrl->ftmin_bits) {
                atomicMin(&ctrl->ftmin_bits, bits);
            }
        }
    }
}

// FP32 variant for the mixed flux: the reduction stays in FP32 and only the
// block's minimum is widened for the atomic.  Non-negative floats (+inf
// included) order as their bit patterns read as integers, so each warp takes
// the minimum with one integer warp reduction; a NaN or negative timestep
// maps to -1, which wins the minimum and raises the status.
// ftmin_seen: the running minimum as read earlier by the block (default:
// read it here, after the reduction).
__device__ __forceinline__ int timestep_key(float t) {
    return t >= 0.0f ? (__float_as_int(t) & 0x7fffffff) : -1;
}
template <int BLOCK = kBlock>
__device__ __forceinline__ void block_min_timestep_f(float t, Ctrl *ctrl,
                                                     const unsigned long long *ftmin_seen =
                                                         nullptr) {
    __shared__ int wmin[BLOCK / 32];
    int key = __reduce_min_sync(0xffffffffu, timestep_key(t));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmin[warp] = key;
    __syncthreads();
    if (warp == 0) {
        key = lane < (int)(blockDim.x >> 5) ? wmin[lane] : __float_as_int(3.0e38f);
        key = __reduce_min_sync(0xffffffffu, key);
        if (lane == 0) {
            if (key < 0) {
                set_status(ctrl, SWGPU_ENONFINITE);
            } else {
                const double td = (double)__int_as_float(key);
                const unsigned long long bits = (unsigned long long)__double_as_longlong(td);
                const unsigned long long seen =
                    ftmin_seen ? *ftmin_seen : *(volatile unsigned long long *)&ctrl->ftmin_bits;
                if (bits < seen) atomicMin(&ctrl->ftmin_bits, bits);
            }
        }
    }
}

__device__ __forceinline__ int ctrl_halted(const Ctrl *c) {
    return *(volatile const int *)&c->halt;
}

// The halt flag read after griddepcontrol.wait, when no kernel still running
// can change it: a plain load, served from L1 for all but the first warp of
// each SM (a volatile load from every warp would queue on the one L2 line
// that holds the control block).
__device__ __forceinline__ int ctrl_halt_settled(const Ctrl *c) { return c->halt; }

// Commit the new time and counters and decide whether the loop stops after
// this step's distribute (FP64: the update kernel's last block; mixed: the
// first block of the scenario in the distribute, through commit_stage).
__device__ __forceinline__ void commit_step(Ctrl *c, const StepClock &s, const DevParams &P) {
    c->rec_max = omax(s.dt, c->rec_max);
    c->rec_min = omin(s.dt, c->rec_min);
    c->order = s.order;
    c->smallsteps = s.smallsteps;
    c->flux_timestep = s.ftmin;
    c->timestep = s.dt;
    c->time = c->time + s.dt;
    c->steps_since_yield += 1;
    c->total_steps += 1;
    c->ftmin_bits = (unsigned long long)__double_as_longlong(P.evolve_max_timestep);
    int reason = kStopNone;
    if (s.small_error) set_status(c, SWGPU_ESMALLSTEP);
    if (c->status != 0) {
        reason = kStopError;
    } else if (c->finaltime > 0 && c->time >= c->finaltime - c->time_epsilon) {
        if (c->time > c->finaltime) set_status(c, SWGPU_EOVERSHOOT);
        c->time = c->finaltime;
        reason = c->status ? kStopError : kStopFinal;
    } else if (c->time >= c->yieldtime) {
        reason = kStopYield;
    }
    if (reason == kStopNone && c->budget > 0) {
        c->budget -= 1;
        if (c->budget == 0) reason = kStopBudget;
    }
    if (reason != kStopNone) c->halt_pending = reason;
}

// The stage commit of a fused step, per stage kind (FP64: the update
// kernel's last block; mixed: the distribute's first block).  The
// first Runge-Kutta stage records the step's clock (the distribute that
// follows reads the order) and moves time to t0 + dt, the middle RK3 stage
// to t0 + dt/2; the last stage commits the step from t0 as an Euler step
// does (time = t0 + dt, the evolve loop's set_time(initial_time + timestep)).
__device__ __forceinline__ void commit_stage(Ctrl *c, const StepClock &s, const DevParams &P,
                                             const Stage &stg) {
    if (stg.kind == kStageFirst) {
        c->step_t0 = c->time;
        c->order = s.order;
        c->smallsteps = s.smallsteps;
        c->time = c->time + s.dt;
    } else if (stg.kind == kStageMid) {
        c->time = c->step_t0 + s.dt * stg.tfrac;
    } else {
        if (stg.kind == kStageLast) c->time = c->step_t0;
        commit_step(c, s, P);
    }
}

// Maximum depth and arrival time of triangle k after a whole step that
// ends at time t_end (stages before the last of a Runge-Kutta step do not
// count).
__device__ __forceinline__ void track_depth(const DevState &S, int k, double h, double t_end,
                                            double threshold) {
    const float hf = (float)h;
    if (hf > S.hmax[k]) S.hmax[k] = hf;
    if (h > threshold && S.tarr[k] < 0.0f) S.tarr[k] = (float)t_end;
}

// Model time at the end of the step a stage belongs to, read by every
// block before the stage is committed.
__device__ __forceinline__ double step_end_time(const Ctrl *c, const StepClock &s,
                                                const Stage &stg) {
    return (stg.kind == kStageLast ? c->step_t0 : c->time) + s.dt;
}

// Last block of the distribute kernel: a pending stop takes effect.
__device__ __forceinline__ void apply_pending_halt(Ctrl *c) {
    if (c->halt_pending) {
        c->stop_reason = c->halt_pending;
        c->halt = 1;
        c->halt_pending = 0;
        if (c->status) atomicCAS(&c->summary->status, 0, c->status);
        atomicOr(&c->halt_bits[c->scen >> 5], 1u << (c->scen & 31));
        __threadfence();
        atomicAdd(&c->summary->halted, 1);
    }
}

// Mixed path: the stage commit (in the distribute's first block of the
// scenario) announces a stop decided by commit_step at once (stop reason,
// summary, halt bit), and halt = 2 means "stopped after this step's
// distribute": the mixed distribute skips only halt == 1, every other mixed
// kernel any nonzero halt, and the next step's clock kernel turns 2 into 1.
__device__ __forceinline__ void announce_halt(Ctrl *c) {
    if (c->halt_pending) {
        c->stop_reason = c->halt_pending;
        c->halt = 2;
        c->halt_pending = 0;
        if (c->status) atomicCAS(&c->summary->status, 0, c->status);
        atomicOr(&c->halt_bits[c->scen >> 5], 1u << (c->scen & 31));
        __threadfence();
        atomicAdd(&c->summary->halted, 1);
    }
}

}  // namespace swgpu
