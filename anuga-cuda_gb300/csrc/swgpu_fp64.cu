// swgpu_fp64.cu -- FP64 evolve kernels (the parity path).
//
// Every floating-point operation is performed in the order of the
// reference's ANUGA C kernels so that the results agree bit for bit with
// them on the same mesh (the file is compiled with --fmad=false: no
// contraction into FMA).  On GB300 this path is bound by the FP64 pipe, not
// by HBM: ~600 dependent FP64 operations per triangle-step.
//
// One Euler step of the device-resident loop is three kernels:
//   flux_fp64       central-upwind fluxes of the three edges (triangle
//                   centric, neighbour edge values gathered), summed in
//                   ANUGA's order, gravity_wb, per-triangle CFL timestep ->
//                   block min -> atomicMin into Ctrl
//   update_fp64     the step's update_timestep (evaluated once by the flux
//                   kernel's last block), Manning
//                   friction, the semi-implicit conserved update, protect,
//                   centroid velocities for the next extrapolation; the last
//                   block advances the model time
//   distribute_fp64 second-order limited extrapolation, balance_deep_and_
//                   shallow, boundary conditions of the triangle's boundary
//                   edges; vertex values stored, edge values derived on use
#include <cstdio>

#include "swgpu_device.cuh"

namespace swgpu {

// ---------------------------------------------------------------- flux ---

// src/anuga_HMPP/shallow_water_ext.c:214-242 (_compute_speed).
__device__ __forceinline__ double limited_speed(double &uh, double &h, double eps, double h0,
                                                double lim) {
    double u;
    if (h < lim) {
        if (h < eps) {
            h = 0.0;
            u = 0.0;
        } else {
            u = uh / (h + h0 / h);
        }
        uh = u * h;
    } else {
        u = uh / h;
    }
    return u;
}

// src/anuga_HMPP/shallow_water_ext.c:302-441 (_flux_function_central).
// Returns false if the bed is discontinuous across the edge.
__device__ __forceinline__ bool central_flux(double wl, double uhl_in, double vhl_in, double wr,
                                             double uhr_in, double vhr_in, double zl, double zr,
                                             double n1, double n2, const DevParams &P, double h0,
                                             double lim, double &f0, double &f1, double &f2,
                                             double &ms) {
    // rotate into the edge frame (_rotate, :36-53)
    const double al = n1 * uhl_in + n2 * vhl_in;
    const double bl = -n2 * uhl_in + n1 * vhl_in;
    const double ar = n1 * uhr_in + n2 * vhr_in;
    const double br = -n2 * uhr_in + n1 * vhr_in;
    if (fabs(zl - zr) > 1.0e-10) return false;
    const double z = 0.5 * (zl + zr);
    const double g = P.g, eps = P.epsilon;

    double hl = wl - z, uhl = al;
    const double ul = limited_speed(uhl, hl, eps, h0, lim);
    double hr = wr - z, uhr = ar;
    const double ur = limited_speed(uhr, hr, eps, h0, lim);
    double vhl = bl, vhr = br;
    limited_speed(vhl, hl, eps, h0, lim);
    limited_speed(vhr, hr, eps, h0, lim);

    const double cl = sqrt(g * hl);
    const double cr = sqrt(g * hr);
    double smax = omax(ul + cl, ur + cr);
    if (smax < 0.0) smax = 0.0;
    double smin = omin(ul - cl, ur - cr);
    if (smin > 0.0) smin = 0.0;

    const double fl0 = ul * hl;
    const double fl1 = ul * uhl + 0.5 * g * hl * hl;
    const double fl2 = ul * vhl;
    const double fr0 = ur * hr;
    const double fr1 = ur * uhr + 0.5 * g * hr * hr;
    const double fr2 = ur * vhr;

    const double denom = smax - smin;
    if (denom < eps) {
        f0 = f1 = f2 = 0.0;
        ms = 0.0;
        return true;
    }
    const double inv = 1.0 / denom;
    const double ss = smax * smin;
    double e0 = smax * fl0 - smin * fr0;
    e0 += ss * (wr - wl);
    e0 *= inv;
    double e1 = smax * fl1 - smin * fr1;
    e1 += ss * (ar - al);
    e1 *= inv;
    double e2 = smax * fl2 - smin * fr2;
    e2 += ss * (br - bl);
    e2 *= inv;
    ms = omax(fabs(smax), fabs(smin));
    // rotate back: _rotate(edgeflux, n1, -n2)
    f0 = e0;
    f1 = n1 * e1 + (-n2) * e2;
    f2 = -(-n2) * e1 + n1 * e2;
    return true;
}

struct EdgeFlux {
    double f0, f1, f2;
    bool skip;
};

// Flux of edge i of triangle k (src/anuga_HMPP/shallow_water_ext.c:4553-4640,
// seen from triangle k) and its contribution to the CFL timestep.
template <int I>
__device__ __forceinline__ EdgeFlux edge_flux(const DevMesh &M, const DevState &S,
                                              const DevParams &P, int k, const double (&ew)[3],
                                              const double (&euh)[3], const double (&evh)[3],
                                              const double (&ez)[3], double h0, double lim,
                                              double &t, double &ms_own, int &bad) {
    const int N = M.N;
    EdgeFlux r;
    const int pk = M.nbr[I * N + k];
    double wr, uhr, vhr, zr;
    int n = -1;
    if (pk >= 0) {
        n = pk >> 2;
        const int m = pk & 3;
        if (P.flow_algorithm) {
            wr = S.we[m * N + n];
            uhr = S.uhe[m * N + n];
            vhr = S.vhe[m * N + n];
        } else {
            const int a = (m == 0) ? 1 : 0, b = (m == 2) ? 1 : 2;  // the other two vertices
            wr = 0.5 * (S.wv[a * N + n] + S.wv[b * N + n]);
            uhr = 0.5 * (S.uhv[a * N + n] + S.uhv[b * N + n]);
            vhr = 0.5 * (S.vhv[a * N + n] + S.vhv[b * N + n]);
        }
        zr = S.ze[m * N + n];
    } else {
        const int mb = -pk - 1;
        wr = S.wb[mb];
        uhr = S.uhb[mb];
        vhr = S.vhb[mb];
        zr = ez[I];
    }
    const double wl = ew[I], zl = ez[I];
    if (P.optimise_dry_cells && fabs(wl - zl) < P.epsilon && fabs(wr - zr) < P.epsilon) {
        r.f0 = r.f1 = r.f2 = 0.0;
        r.skip = true;
        return r;
    }
    double ms;
    if (!central_flux(wl, euh[I], evh[I], wr, uhr, vhr, zl, zr, M.normals[(2 * I) * N + k],
                      M.normals[(2 * I + 1) * N + k], P, h0, lim, r.f0, r.f1, r.f2, ms)) {
        bad = 1;
        r.f0 = r.f1 = r.f2 = 0.0;
        r.skip = true;
        return r;
    }
    const double length = M.len[I * N + k];
    r.f0 *= length;
    r.f1 *= length;
    r.f2 *= length;
    r.skip = false;
    // CFL: counted when the triangle that processes this edge first in
    // ANUGA's loop (the lower index of the pair) is full
    const bool full = (n >= 0 && n < k) ? M.full[n] : M.full[k];
    if (full && ms > P.epsilon) {
        t = omin(t, M.radii[k] / ms);
        if (n >= 0) t = omin(t, M.radii[n] / ms);
    }
    if (n < 0 || n > k) ms_own = omax(ms_own, ms);
    return r;
}

__device__ __forceinline__ void pick(int i, const EdgeFlux &a, const EdgeFlux &b,
                                     const EdgeFlux &c, double &f0, double &f1, double &f2,
                                     bool &skip) {
    f0 = i == 0 ? a.f0 : (i == 1 ? b.f0 : c.f0);
    f1 = i == 0 ? a.f1 : (i == 1 ? b.f1 : c.f1);
    f2 = i == 0 ? a.f2 : (i == 1 ? b.f2 : c.f2);
    skip = i == 0 ? a.skip : (i == 1 ? b.skip : c.skip);
}

// compute_fluxes with gravity_wb ('wb_2').  Triangle k sums -flux(k,i) over
// its edges in ANUGA's order: edges to lower-index neighbours first, by
// neighbour index, then its remaining edges by edge index.  The central
// flux is exactly antisymmetric in IEEE arithmetic, so -flux(k,i) equals
// the +flux(n,m) that ANUGA's edge loop adds, and the sums agree bitwise.
template <int BS>
__global__ void __launch_bounds__(BS) flux_fp64(DevMesh M, DevState S, DevParams P,
                                                    Ctrl *ctrl, int flags) {
    ctrl = block_ctrl(ctrl, M);
    if ((flags & kFused) && ctrl_halted(ctrl)) return;
    const int N = M.N;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double t = P.evolve_max_timestep;
    int bad = 0;
    if (k < N) {
        const double h0 = P.H0 * P.H0;
        const double lim = 10 * P.H0;
        double vw[3], vu[3], vv[3], ew[3], euh[3], evh[3], ez[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            vw[i] = S.wv[i * N + k];
            vu[i] = S.uhv[i * N + k];
            vv[i] = S.vhv[i * N + k];
            ez[i] = S.ze[i * N + k];
        }
        if (P.flow_algorithm) {
            // 'tsunami': the extrapolated edge values themselves
#pragma unroll
            for (int i = 0; i < 3; i++) {
                ew[i] = S.we[i * N + k];
                euh[i] = S.uhe[i * N + k];
                evh[i] = S.vhe[i * N + k];
            }
        } else {
            // quantity.c:687-706 (_interpolate_from_vertices_to_edges)
            ew[0] = 0.5 * (vw[1] + vw[2]);
            ew[1] = 0.5 * (vw[0] + vw[2]);
            ew[2] = 0.5 * (vw[0] + vw[1]);
            euh[0] = 0.5 * (vu[1] + vu[2]);
            euh[1] = 0.5 * (vu[0] + vu[2]);
            euh[2] = 0.5 * (vu[0] + vu[1]);
            evh[0] = 0.5 * (vv[1] + vv[2]);
            evh[1] = 0.5 * (vv[0] + vv[2]);
            evh[2] = 0.5 * (vv[0] + vv[1]);
        }

        double ms_own = 0.0;
        const EdgeFlux F0 = edge_flux<0>(M, S, P, k, ew, euh, evh, ez, h0, lim, t, ms_own, bad);
        const EdgeFlux F1 = edge_flux<1>(M, S, P, k, ew, euh, evh, ez, h0, lim, t, ms_own, bad);
        const EdgeFlux F2 = edge_flux<2>(M, S, P, k, ew, euh, evh, ez, h0, lim, t, ms_own, bad);

        const int code = M.order[k];
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            double f0, f1, f2;
            bool skip;
            pick((code >> (2 * j)) & 3, F0, F1, F2, f0, f1, f2, skip);
            if (!skip) {
                a0 -= f0;
                a1 -= f1;
                a2 -= f2;
            }
        }
        const double inv_area = 1.0 / M.areas[k];
        a0 *= inv_area;
        a1 *= inv_area;
        a2 *= inv_area;

        // gravity_wb (src/anuga_HMPP/shallow_water_ext.c:1942-2036)
        {
            const double g = P.g;
            const double x0 = M.vxy[0 * N + k], y0 = M.vxy[1 * N + k];
            const double x1 = M.vxy[2 * N + k], y1 = M.vxy[3 * N + k];
            const double x2 = M.vxy[4 * N + k], y2 = M.vxy[5 * N + k];
            const double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
            double wx = (y2 - y0) * (vw[1] - vw[0]) - (y1 - y0) * (vw[2] - vw[0]);
            wx /= det;
            double wy = (x1 - x0) * (vw[2] - vw[0]) - (x2 - x0) * (vw[1] - vw[0]);
            wy /= det;
            const double avg_h = S.w[k] - S.zc[k];
            a1 += -g * wx * avg_h;
            a2 += -g * wy * avg_h;
            double sidex = 0.0, sidey = 0.0;
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const double hh = ew[i] - ez[i];
                const double fact = -0.5 * g * hh * hh * M.len[i * N + k];
                sidex = sidex + fact * M.normals[(2 * i) * N + k];
                sidey = sidey + fact * M.normals[(2 * i + 1) * N + k];
            }
            const double area = M.areas[k];
            a1 += -sidex / area;
            a2 += -sidey / area;
        }
        S.ew[k] = a0;
        S.euh[k] = a1;
        S.evh[k] = a2;
        if (flags & kWriteMaxSpeed) S.max_speed[k] = ms_own;
    }
    if (bad) set_status(ctrl, SWGPU_EBED);
    if (flags & kNoTimestep) return;  // later Runge-Kutta stage: the step's dt is set
    block_min_timestep<BS>(t, ctrl);
    if ((flags & kFused) && threadIdx.x == 0 && last_block_done(&ctrl->done_flux, ctrl->blocks_flux))
        publish_step_clock(ctrl, P);
}

// ------------------------------------------------------------- update ---

// src/anuga_HMPP/shallow_water_ext.c:1238-1317: Manning friction
// coefficient S of triangle k (0 when it does not apply).
__device__ __forceinline__ double manning_S(const DevMesh &M, const DevState &S,
                                            const DevParams &P, int k, double w, double uh,
                                            double vh, bool &applied) {
    const int N = M.N;
    const double eta = S.fric[k];
    const double eps = P.minimum_allowed_height;
    applied = false;
    if (!(eta > eps)) return 0.0;
    const double z0 = S.zv[k], z1 = S.zv[N + k], z2 = S.zv[2 * N + k];
    double zs = 1.0;
    if (P.use_sloped_mannings) {
        const double x0 = M.vxy[0 * N + k], y0 = M.vxy[1 * N + k];
        const double x1 = M.vxy[2 * N + k], y1 = M.vxy[3 * N + k];
        const double x2 = M.vxy[4 * N + k], y2 = M.vxy[5 * N + k];
        const double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
        double zx = (y2 - y0) * (z1 - z0) - (y1 - y0) * (z2 - z0);
        zx /= det;
        double zy = (x1 - x0) * (z2 - z0) - (x2 - x0) * (z1 - z0);
        zy /= det;
        zs = sqrt(1.0 + zx * zx + zy * zy);
    }
    const double z = (z0 + z1 + z2) / 3.0;
    const double h = w - z;
    if (!(h >= eps)) return 0.0;
    double Sf;
    if (P.use_sloped_mannings)
        Sf = -P.g * eta * eta * zs * sqrt((uh * uh + vh * vh));
    else
        Sf = -P.g * eta * eta * sqrt((uh * uh + vh * vh));
    Sf /= pow(h, 7.0 / 3);
    applied = true;
    return Sf;
}

// compute_forcing_terms for the per-method API: semi_implicit_update += S*q
// (manning_friction_implicit, gpu_domain_advanced.py:1255-1324), or with
// explicit_target explicit_update += S*q (manning_friction_explicit, :1330-1388:
// the same _manning_friction_flat / _sloped kernels given the explicit arrays).
__global__ void __launch_bounds__(kBlock) forcing_fp64(DevMesh M, DevState S, DevParams P,
                                                       int explicit_target) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M.N) return;
    bool applied;
    const double uh = S.uh[k], vh = S.vh[k];
    const double Sf = manning_S(M, S, P, k, S.w[k], uh, vh, applied);
    if (applied) {
        double *xu = explicit_target ? S.euh : S.suh;
        double *yu = explicit_target ? S.evh : S.svh;
        xu[k] += Sf * uh;
        yu[k] += Sf * vh;
    }
}

// src/anuga_HMPP/shallow_water_ext.c:1638-1705 (_protect) on one triangle.
// The 'tsunami' protection (src/anuga_cuda/protect/protect.cu:64-131) of
// triangle k: below max(0.1 (max bed edge - bed centroid), mah) momentum is
// zeroed; a non-positive depth lifts stage to the lowest bed vertex minus
// mah.  Returns the lifted stage floor bmin (or -inf) for the vertex clamp.
__device__ __forceinline__ double protect_swb2_one(const DevParams &P, double zc,
                                                   const double (&zv)[3], double &w, double &uh,
                                                   double &vh) {
    const double mah = P.minimum_allowed_height;
    const double hc = w - zc;
    const double bmax = 0.5 * fmax(zv[0] + zv[1], fmax(zv[1] + zv[2], zv[2] + zv[0]));
    double floor_w = -pos_inf();
    if (hc < fmax(0.1 * (bmax - zc), mah)) {
        uh = 0.0;
        vh = 0.0;
        if (hc <= 0.0) {
            const double bmin = fmin(zv[0], fmin(zv[1], zv[2])) - mah;
            if (w < bmin) {
                w = fmax(w, bmin);
                floor_w = bmin;
            }
        }
    }
    return floor_w;
}

__device__ __forceinline__ void protect_one(const DevParams &P, double zc, double &w, double &uh,
                                            double &vh) {
    const double hc = w - zc;
    if (!(hc < P.minimum_allowed_height)) return;
    if (P.maximum_allowed_speed < P.epsilon) {
        uh = 0.0;
        vh = 0.0;
        if (hc <= 0.0) w = zc;
    } else if (hc <= 0.0) {
        w = zc;
        uh = 0.0;
        vh = 0.0;
    } else {
        const double u = uh / hc, v = vh / hc;
        if (fabs(u) > P.maximum_allowed_speed) uh = (P.maximum_allowed_speed * u / fabs(u)) * hc;
        if (fabs(v) > P.maximum_allowed_speed) vh = (P.maximum_allowed_speed * v / fabs(v)) * hc;
    }
}

// src/anuga_HMPP/quantity.c:769-820 (_update) on one value with a nonzero
// semi-implicit term; returns false if the denominator is not positive.
__device__ __forceinline__ bool semi_update(double &c, double e, double semi, double dt) {
    if (c == 0.0)
        semi = 0.0;
    else
        semi /= c;
    c += dt * e;
    const double den = 1.0 - dt * semi;
    if (den <= 0.0) return false;
    c /= den;
    return true;
}

// update_conserved_quantities (gpu_domain_advanced.py:1412-1442).  Fused:
// dt from the device update_timestep, Manning friction computed here, then
// protect (the first step of the next distribute, moved here: nothing reads
// the centroids in between) and the centroid velocities the next
// extrapolation reads.  API: dt given, semi-implicit terms from
// compute_forcing_terms, no protect.
template <int BS>
__global__ void __launch_bounds__(BS) update_fp64(DevMesh M, DevState S, DevParams P,
                                                      Ctrl *ctrl, double dt_api, int flags,
                                                      Stage stg) {
    const bool fused = flags & kFused;
    ctrl = block_ctrl(ctrl, M);
    if (fused && ctrl_halted(ctrl)) return;
    StepClock clk;
    if (fused) {
        clk = published_step_clock(ctrl);
    } else {
        clk.dt = dt_api;
    }
    const double dt = clk.dt;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int bad = 0, nonfinite = 0;
    if (k < M.N) {
        double w = S.w[k], uh = S.uh[k], vh = S.vh[k];
        if (stg.kind == kStageFirst) {  // backup_conserved_quantities
            S.bw[k] = w;
            S.buh[k] = uh;
            S.bvh[k] = vh;
        }
        double su, sv;
        bool applied;
        if (flags & kFrictionInline) {
            const double Sf = manning_S(M, S, P, k, w, uh, vh, applied);
            su = applied ? Sf * uh : 0.0;
            sv = applied ? Sf * vh : 0.0;
        } else {
            su = S.suh[k];
            sv = S.svh[k];
            applied = (su != 0.0) || (sv != 0.0);
            S.suh[k] = 0.0;
            S.svh[k] = 0.0;
        }
        // stage has no semi-implicit term: its denominator is exactly 1
        w += dt * S.ew[k];
        if (applied) {
            if (!semi_update(uh, S.euh[k], su, dt)) bad = 1;
            if (!semi_update(vh, S.evh[k], sv, dt)) bad = 1;
        } else {
            uh += dt * S.euh[k];
            vh += dt * S.evh[k];
        }
        if (stg.kind == kStageMid || stg.kind == kStageLast) {
            // saxpy_conserved_quantities (quantity.c:749-765)
            w = stg.a * w + stg.b * S.bw[k];
            uh = stg.a * uh + stg.b * S.buh[k];
            vh = stg.a * vh + stg.b * S.bvh[k];
        }
        if (fused) {
            const double zc = S.zc[k];
            if (P.flow_algorithm) {
                // the stage vertex clamp of protect_swb2 is overwritten by the
                // extrapolation that follows in the same step
                const double zv[3] = {S.zv[k], S.zv[M.N + k], S.zv[2 * M.N + k]};
                protect_swb2_one(P, zc, zv, w, uh, vh);
            } else {
                protect_one(P, zc, w, uh, vh);
            }
            if (P.extrapolate_velocity_second_order == 1) {
                const double dk = omax(w - zc, P.minimum_allowed_height);
                S.uvel[k] = uh / dk;
                S.vvel[k] = vh / dk;
            }
        }
        // NaN / Inf anywhere in the new state stops the run
        const double big = 1.0e308;
        if (!(fabs(w) <= big) || !(fabs(uh) <= big) || !(fabs(vh) <= big)) nonfinite = 1;
        S.w[k] = w;
        S.uh[k] = uh;
        S.vh[k] = vh;
        if ((flags & kTrack) && (stg.kind == kStageEuler || stg.kind == kStageLast))
            track_depth(S, k, w - S.zc[k], step_end_time(ctrl, clk, stg), P.track_threshold);
    }
    if (bad) set_status(ctrl, SWGPU_EDENOMINATOR);
    if (nonfinite) set_status(ctrl, SWGPU_ENONFINITE);
    if (fused) {
        __syncthreads();
        if (threadIdx.x == 0 && last_block_done(&ctrl->done_update, ctrl->blocks_update))
            commit_stage(ctrl, clk, P, stg);
    }
}

__global__ void __launch_bounds__(kBlock) track_reset(int N, float *hmax, float *tarr) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    hmax[k] = 0.0f;
    tarr[k] = -1.0f;
}
void launch_track_reset(const DevMesh &M, const DevState &S, cudaStream_t st) {
    track_reset<<<grid_for(M.N), kBlock, 0, st>>>(M.N, S.hmax, S.tarr);
}

// saxpy_conserved_quantities (src/anuga_cuda/saxpy_centroid_values/
// saxpy_centroid_values.cu:1-12, src/anuga_HMPP/quantity.c:749-765) on the
// three conserved quantities: Q = a*Q + b*backup, products then sum, no
// contraction (this unit is built with --fmad=false).
__global__ void __launch_bounds__(kBlock) saxpy_fp64(int N, double a, double b, double *w,
                                                     double *uh, double *vh,
                                                     const double *bw, const double *buh,
                                                     const double *bvh) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    w[k] = a * w[k] + b * bw[k];
    uh[k] = a * uh[k] + b * buh[k];
    vh[k] = a * vh[k] + b * bvh[k];
}

// protect plus the centroid velocities: the head of a stand-alone
// distribute (gpu_domain_advanced.py:1003-1055 and
// extrapolate_velocity_second_order_true, extrapolate_second_order_sw.cu:77-104).
__global__ void __launch_bounds__(kBlock) prepare_fp64(DevMesh M, DevState S, DevParams P) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = M.N;
    if (k >= N) return;
    double w = S.w[k], uh = S.uh[k], vh = S.vh[k];
    const double zc = S.zc[k];
    if (P.flow_algorithm) {
        const double zv[3] = {S.zv[k], S.zv[N + k], S.zv[2 * N + k]};
        const double floor_w = protect_swb2_one(P, zc, zv, w, uh, vh);
        if (floor_w > -pos_inf()) {
#pragma unroll
            for (int i = 0; i < 3; i++) S.wv[i * N + k] = fmax(S.wv[i * N + k], floor_w);
        }
    } else {
        protect_one(P, zc, w, uh, vh);
    }
    S.w[k] = w;
    S.uh[k] = uh;
    S.vh[k] = vh;
    const double dk = omax(w - zc, P.minimum_allowed_height);
    S.uvel[k] = uh / dk;
    S.vvel[k] = vh / dk;
}

// The centroid velocities alone: extrapolate_velocity_second_order_true
// (extrapolate_second_order_sw.cu:77-104) as the stand-alone
// extrapolate_second_order_sw runs it, on the state as it is (no protect).
__global__ void __launch_bounds__(kBlock) velocities_fp64(DevMesh M, DevState S, DevParams P) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M.N) return;
    const double dk = omax(S.w[k] - S.zc[k], P.minimum_allowed_height);
    S.uvel[k] = S.uh[k] / dk;
    S.vvel[k] = S.vh[k] / dk;
}

// --------------------------------------------------------- distribute ---

// src/anuga_HMPP/shallow_water_ext.c:98-148 (find_qmin_and_qmax).
__device__ __forceinline__ void qmin_qmax(double dq0, double dq1, double dq2, double &qmin,
                                          double &qmax) {
    if (dq0 >= 0.0) {
        if (dq1 >= dq2) {
            qmax = (dq1 >= 0.0) ? dq0 + dq1 : dq0;
            qmin = dq0 + dq2;
            if (qmin >= 0.0) qmin = 0.0;
        } else {
            qmax = (dq2 > 0) ? dq0 + dq2 : dq0;
            qmin = dq0 + dq1;
            if (qmin >= 0.0) qmin = 0.0;
        }
    } else {
        if (dq1 <= dq2) {
            qmin = (dq1 < 0.0) ? dq0 + dq1 : dq0;
            qmax = dq0 + dq2;
            if (qmax <= 0.0) qmax = 0.0;
        } else {
            qmin = (dq2 < 0.0) ? dq0 + dq2 : dq0;
            qmax = dq0 + dq1;
            if (qmax <= 0.0) qmax = 0.0;
        }
    }
}

// src/anuga_HMPP/shallow_water_ext.c:151-181 (limit_gradient).
__device__ __forceinline__ void limit_jumps(double (&d)[3], double qmin, double qmax,
                                            double beta) {
    const double TINY = 1.0e-100;
    double r = 1000.0, r0 = 1.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (d[i] < -TINY) r0 = qmin / d[i];
        if (d[i] > TINY) r0 = qmax / d[i];
        r = omin(r0, r);
    }
    const double phi = omin(r * beta, 1.0);
    d[0] = d[0] * phi;
    d[1] = d[1] * phi;
    d[2] = d[2] * phi;
}

// Auxiliary-triangle reconstruction of one quantity
// (src/anuga_HMPP/shallow_water_ext.c:2942-3055).
__device__ __forceinline__ void aux_jumps(double qk, double q0, double q1, double q2, double dx1,
                                          double dy1, double dx2, double dy2, double inv_area2,
                                          const double (&dxv)[3], const double (&dyv)[3],
                                          double beta, double (&out)[3]) {
    const double dq0 = q0 - qk, dq1 = q1 - q0, dq2 = q2 - q0;
    double a = dy2 * dq1 - dy1 * dq2;
    a *= inv_area2;
    double b = dx1 * dq2 - dx2 * dq1;
    b *= inv_area2;
    double d[3];
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] = a * dxv[i] + b * dyv[i];
    double qmin, qmax;
    qmin_qmax(dq0, dq1, dq2, qmin, qmax);
    limit_jumps(d, qmin, qmax, beta);
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = qk + d[i];
}

// Single interior neighbour (src/anuga_HMPP/shallow_water_ext.c:3058-3205).
__device__ __forceinline__ void one_nbr_jumps(double qk, double q1, double dx2, double dy2,
                                              const double (&dxv)[3], const double (&dyv)[3],
                                              double beta, double (&out)[3]) {
    const double dq1 = q1 - qk;
    const double a = dq1 * dx2, b = dq1 * dy2;
    double d[3];
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] = a * dxv[i] + b * dyv[i];
    double qmin, qmax;
    if (dq1 >= 0.0) {
        qmin = 0.0;
        qmax = dq1;
    } else {
        qmin = dq1;
        qmax = 0.0;
    }
    limit_jumps(d, qmin, qmax, beta);
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = qk + d[i];
}

// The 'tsunami' distribute (gpu_domain_advanced.py:1755-1812): the edge
// extrapolation of src/anuga_HMPP/shallow_water_ext.c:3328-3964
// (_extrapolate_second_order_edge_sw) after protect_swb2 (applied by the
// update kernel or prepare_fp64): limited auxiliary-triangle gradients
// evaluated at the edge midpoints, dry surrogate neighbours replaced by the
// triangle itself, beta fully wet or dry, vertex values from the edge values
// (v_i = e_j + e_k - e_i), momenta back from velocities with the edge and
// vertex depths; cells skipped as dry keep their previous edge values.  Edge
// values are always stored (the flux reads them), then the boundary values.
template <int BS>
__global__ void __launch_bounds__(BS) distribute_de_fp64(DevMesh M, DevState S, DevParams P,
                                                         const BcTag *tags, Ctrl *ctrl,
                                                         int flags) {
    const bool fused = flags & kFused;
    ctrl = block_ctrl(ctrl, M);
    if (fused && ctrl_halted(ctrl)) return;
    const int N = M.N;
    const double time = ctrl->time;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int bad_bc = 0, no_nbr = 0;
    if (k < N) {
        const bool vel = P.extrapolate_velocity_second_order == 1;
        const double *U = vel ? S.uvel : S.uh;  // extrapolated centroid values
        const double *V = vel ? S.vvel : S.vh;
        const double wk = S.w[k], uk = U[k], vk = V[k];
        const int nbk = M.nb[k];
        double ew[3], eu[3], ev[3];
        bool flat = false, keep = false;
        if (nbk == 3) {
            flat = true;
        } else {
            const double x = M.cxy[k], y = M.cxy[N + k];
            double vx[3], vy[3], dxv[3], dyv[3];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                vx[i] = M.vxy[(2 * i) * N + k];
                vy[i] = M.vxy[(2 * i + 1) * N + k];
            }
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const int a = (i + 1) % 3, b = (i + 2) % 3;
                dxv[i] = 0.5 * (vx[a] + vx[b]) - x;  // edge midpoint offsets
                dyv[i] = 0.5 * (vy[a] + vy[b]) - y;
            }
            if (nbk <= 1) {
                int k0 = M.surr[k], k1 = M.surr[N + k], k2 = M.surr[2 * N + k];
                if (S.w[k2] <= S.zc[k2]) k2 = k;
                if (S.w[k0] <= S.zc[k0]) k0 = k;
                if (S.w[k1] <= S.zc[k1]) k1 = k;
                const double x0 = M.cxy[k0], y0 = M.cxy[N + k0];
                const double dx1 = M.cxy[k1] - x0, dx2 = M.cxy[k2] - x0;
                const double dy1 = M.cxy[N + k1] - y0, dy2 = M.cxy[N + k2] - y0;
                const double area2 = dy2 * dx1 - dy1 * dx2;
                if (area2 <= 0) {
                    flat = true;
                } else {
                    const double hc = wk - S.zc[k];
                    const double h0 = S.w[k0] - S.zc[k0];
                    const double h1 = S.w[k1] - S.zc[k1];
                    const double h2 = S.w[k2] - S.zc[k2];
                    const double hmin = omin(omin(h0, omin(h1, h2)), hc);
                    const double hfactor = hmin > 0.0 ? 1.0 : 0.0;
                    if (P.optimise_dry_cells && omax(h0, omax(h1, h2)) < P.epsilon) {
                        keep = true;
                    } else {
                        const double inv_area2 = 1.0 / area2;
                        aux_jumps(wk, S.w[k0], S.w[k1], S.w[k2], dx1, dy1, dx2, dy2, inv_area2,
                                  dxv, dyv, P.beta_w_dry + (P.beta_w - P.beta_w_dry) * hfactor,
                                  ew);
                        aux_jumps(uk, U[k0], U[k1], U[k2], dx1, dy1, dx2, dy2, inv_area2, dxv,
                                  dyv, P.beta_uh_dry + (P.beta_uh - P.beta_uh_dry) * hfactor,
                                  eu);
                        aux_jumps(vk, V[k0], V[k1], V[k2], dx1, dy1, dx2, dy2, inv_area2, dxv,
                                  dyv, P.beta_vh_dry + (P.beta_vh - P.beta_vh_dry) * hfactor,
                                  ev);
                    }
                }
            } else {
                int k1 = -1;
#pragma unroll
                for (int i = 2; i >= 0; i--) {
                    const int sn = M.surr[i * N + k];
                    if (sn != k) k1 = sn;
                }
                if (k1 < 0) {
                    no_nbr = 1;
                    flat = true;
                } else {
                    const double dx1 = M.cxy[k1] - x, dy1 = M.cxy[N + k1] - y;
                    const double area2 = dx1 * dx1 + dy1 * dy1;
                    double dx2 = 1.0 / area2;
                    const double dy2 = dx2 * dy1;
                    dx2 *= dx1;
                    one_nbr_jumps(wk, S.w[k1], dx2, dy2, dxv, dyv, P.beta_w, ew);
                    one_nbr_jumps(uk, U[k1], dx2, dy2, dxv, dyv, P.beta_w, eu);
                    one_nbr_jumps(vk, V[k1], dx2, dy2, dxv, dyv, P.beta_w, ev);
                }
            }
        }
        if (flat) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                ew[i] = wk;
                eu[i] = uk;
                ev[i] = vk;
            }
        } else if (keep) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                ew[i] = S.we[i * N + k];
                eu[i] = S.uhe[i * N + k];
                ev[i] = S.vhe[i * N + k];
            }
        }
        double ow[3], ou[3], ov[3];
        ow[0] = ew[1] + ew[2] - ew[0];
        ow[1] = ew[0] + ew[2] - ew[1];
        ow[2] = ew[0] + ew[1] - ew[2];
        ou[0] = eu[1] + eu[2] - eu[0];
        ou[1] = eu[0] + eu[2] - eu[1];
        ou[2] = eu[0] + eu[1] - eu[2];
        ov[0] = ev[1] + ev[2] - ev[0];
        ov[1] = ev[0] + ev[2] - ev[1];
        ov[2] = ev[0] + ev[1] - ev[2];
        if (vel) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const double de = omax(ew[i] - S.ze[i * N + k], 0.0);
                eu[i] = eu[i] * de;
                ev[i] = ev[i] * de;
                const double dv = omax(ow[i] - S.zv[i * N + k], 0.0);
                ou[i] = ou[i] * dv;
                ov[i] = ov[i] * dv;
            }
        }
#pragma unroll
        for (int i = 0; i < 3; i++) {
            S.we[i * N + k] = ew[i];
            S.uhe[i * N + k] = eu[i];
            S.vhe[i * N + k] = ev[i];
            S.wv[i * N + k] = ow[i];
            S.uhv[i * N + k] = ou[i];
            S.vhv[i * N + k] = ov[i];
        }
        if ((flags & kWriteBoundary) && nbk > 0) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const int pk = M.nbr[i * N + k];
                if (pk < 0) {
                    const int mb = -pk - 1;
                    const double ze = S.ze[i * N + k];
                    double wb, uhb, vhb;
                    if (!eval_boundary(tags[M.btag[mb]], time, ew[i], eu[i], ev[i],
                                       M.normals[(2 * i) * N + k],
                                       M.normals[(2 * i + 1) * N + k], ze, P.g, wb, uhb, vhb)) {
                        bad_bc = 1;
                        wb = uhb = vhb = 0.0;
                    }
                    S.wb[mb] = wb;
                    S.uhb[mb] = uhb;
                    S.vhb[mb] = vhb;
                    S.zb[mb] = ze;
                }
            }
        }
    }
    if (bad_bc) set_status(ctrl, SWGPU_EBOUNDARY);
    if (no_nbr) set_status(ctrl, SWGPU_EMESH);
    if (fused) {
        __syncthreads();
        if (threadIdx.x == 0 && last_block_done(&ctrl->done_distribute, ctrl->blocks_distribute))
            apply_pending_halt(ctrl);
    }
}

// distribute_to_vertices_and_edges for triangle k: extrapolation of the
// current order (src/anuga_HMPP/shallow_water_ext.c:2717-3324 or
// extrapolate_first_order.cu:3-30), balance_deep_and_shallow
// (shallow_water_ext.c:1462-1636), vertex values stored; optionally the edge
// values (quantity.c:687-706) and the boundary values of k's boundary edges.
// Quantity.extrapolate_second_order_and_limit_by_vertex / _by_edge for one
// quantity q of triangle k, vertex values to out: the centroid gradient from
// the surrogate neighbours (src/anuga_HMPP/quantity.c:24-95 with the plane
// gradients of util_ext.h:66-162; no true neighbour leaves it zero),
// extrapolation to vertices and edge midpoints (quantity.c:130-172), then
// one limiter phi over the three vertices (:298-361) or the three edges
// (:363-447) against the min/max of the true neighbours' centroids.
// Returns false where the surrogate neighbours repeat (the reference's
// _compute_gradients gives up there).
__device__ __forceinline__ bool limit_by_neighbours(const DevMesh &M, const double *q, int k,
                                                    double beta, bool by_edge, double out[3]) {
    const int N = M.N;
    const int nbk = M.nb[k];
    const double qk = q[k];
    const double x = M.cxy[k], y = M.cxy[N + k];
    double a = 0.0, b = 0.0;
    bool ok = true;
    if (nbk < 2) {
        const int k0 = M.surr[k], k1 = M.surr[N + k], k2 = M.surr[2 * N + k];
        if (k0 == k1 || k1 == k2) {
            ok = false;
        } else {
            const double x0 = M.cxy[k0], y0 = M.cxy[N + k0];
            const double x1 = M.cxy[k1], y1 = M.cxy[N + k1];
            const double x2 = M.cxy[k2], y2 = M.cxy[N + k2];
            const double q0 = q[k0], q1 = q[k1], q2 = q[k2];
            const double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
            a = (y2 - y0) * (q1 - q0) - (y1 - y0) * (q2 - q0);
            a /= det;
            b = (x1 - x0) * (q2 - q0) - (x2 - x0) * (q1 - q0);
            b /= det;
        }
    } else if (nbk == 2) {
        int k0 = k;
        for (int i = 0; i < 3 && k0 == k; i++) k0 = M.surr[i * N + k];
        if (k0 == k) {
            ok = false;
        } else {
            const double xx = x - M.cxy[k0], yy = y - M.cxy[N + k0], qq = qk - q[k0];
            const double det = xx * xx + yy * yy;
            a = xx * qq / det;
            b = yy * qq / det;
        }
    }
    double v[3], e[3], dqa[3];
#pragma unroll
    for (int i = 0; i < 3; i++)
        v[i] = qk + a * (M.vxy[(2 * i) * N + k] - x) + b * (M.vxy[(2 * i + 1) * N + k] - y);
    e[0] = 0.5 * (v[1] + v[2]);
    e[1] = 0.5 * (v[2] + v[0]);
    e[2] = 0.5 * (v[0] + v[1]);
    double qmin = qk, qmax = qk;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int pk = M.nbr[i * N + k];
        if (pk >= 0) {
            const double qn = q[pk >> 2];
            qmin = omin(qmin, qn);
            qmax = omax(qmax, qn);
        }
    }
    double phi = 1.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        double r = 1.0;
        const double dq = (by_edge ? e[i] : v[i]) - qk;
        dqa[i] = dq;
        if (dq > 0.0) r = (qmax - qk) / dq;
        if (dq < 0.0) r = (qmin - qk) / dq;
        phi = omin(omin(r * beta, 1.0), phi);
    }
    if (by_edge) {
#pragma unroll
        for (int i = 0; i < 3; i++) e[i] = qk + phi * dqa[i];
        out[0] = e[1] + e[2] - e[0];
        out[1] = e[2] + e[0] - e[1];
        out[2] = e[0] + e[1] - e[2];
    } else {
#pragma unroll
        for (int i = 0; i < 3; i++) out[i] = qk + phi * dqa[i];
    }
    return ok;
}

// balance_deep_and_shallow (src/anuga_HMPP/shallow_water_ext.c:1462-1636)
// of one triangle: centroid stage wk, bed zk, momentum uk, vk; bed vertex
// values zvk; stage / momentum vertex values ow, ou, ov blended in place.
__device__ __forceinline__ void balance_one(const DevParams &P, double wk, double zk, double uk,
                                            double vk, const double (&zvk)[3], double (&ow)[3],
                                            double (&ou)[3], double (&ov)[3]) {
    const double eps = 1.0e-6;
    const double hc = wk - zk;
    double dz = 0.0, hv[3];
    if (P.tight_slope_limiters == 0) {
#pragma unroll
        for (int i = 0; i < 3; i++) dz = omax(dz, fabs(zvk[i] - zk));
    }
#pragma unroll
    for (int i = 0; i < 3; i++) hv[i] = ow[i] - zvk[i];
    const double hmin = omin(hv[0], omin(hv[1], hv[2]));
    double alpha;
    if (P.tight_slope_limiters == 0) {
        alpha = dz > 0.0 ? omax(omin(P.alpha_balance * hmin / dz, 1.0), 0.0) : 1.0;
    } else if (hmin < P.H0) {
        alpha = 1.0;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const double hd = hc - hv[i];
            if (!(hd <= 0)) alpha = omin(alpha, (hc - P.H0) / hd);
        }
        if (alpha > 1.0) alpha = 1.0;
        if (alpha < 0.0) alpha = 0.0;
    } else {
        alpha = 1.0;
    }
    if (alpha < 1) {
        double uc = 0.0, vc = 0.0;
        if (P.use_centroid_velocities == 1 && hc > eps) {
            uc = uk / hc;
            vc = vk / hc;
        }
#pragma unroll
        for (int i = 0; i < 3; i++) {
            ow[i] = zvk[i] + (1 - alpha) * hc + alpha * hv[i];
            if (P.use_centroid_velocities == 1) {
                const double h = ow[i] - zvk[i];
                ou[i] = uc * h;
                ov[i] = vc * h;
            } else {
                ou[i] = (1 - alpha) * uk + alpha * ou[i];
                ov[i] = (1 - alpha) * vk + alpha * ov[i];
            }
        }
    }
}

// balance_deep_and_shallow as the stand-alone method
// (gpu_domain_advanced.py:957-995): reads the stored vertex values.
__global__ void __launch_bounds__(kBlock) balance_fp64(DevMesh M, DevState S, DevParams P) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = M.N;
    if (k >= N) return;
    double zvk[3], ow[3], ou[3], ov[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        zvk[i] = S.zv[i * N + k];
        ow[i] = S.wv[i * N + k];
        ou[i] = S.uhv[i * N + k];
        ov[i] = S.vhv[i * N + k];
    }
    balance_one(P, S.w[k], S.zc[k], S.uh[k], S.vh[k], zvk, ow, ou, ov);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        S.wv[i * N + k] = ow[i];
        S.uhv[i * N + k] = ou[i];
        S.vhv[i * N + k] = ov[i];
    }
}

template <int BS>
__global__ void __launch_bounds__(BS) distribute_fp64(DevMesh M, DevState S, DevParams P,
                                                          const BcTag *tags, Ctrl *ctrl,
                                                          int flags) {
    const bool fused = flags & kFused;
    ctrl = block_ctrl(ctrl, M);
    if (fused && ctrl_halted(ctrl)) return;
    const int N = M.N;
    const int order = (int)ctrl->order;
    const double time = ctrl->time;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int bad_bc = 0, no_nbr = 0;
    if (k < N) {
        const double wk = S.w[k], zk = S.zc[k], uk = S.uh[k], vk = S.vh[k];
        double zvk[3];
#pragma unroll
        for (int i = 0; i < 3; i++) zvk[i] = S.zv[i * N + k];
        double ow[3], ou[3], ov[3];
        // the stand-alone extrapolate_second_order_sw is second order with
        // the optimised limiter whatever the domain's order and limiter
        const bool extrapolate_only = flags & kExtrapolateOnly;
        if (order == 1 && !extrapolate_only) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                ow[i] = wk;
                ou[i] = uk;
                ov[i] = vk;
            }
        } else if (P.limiter != kLimiterOptimised && !extrapolate_only) {
            const bool by_edge = P.limiter == kLimiterEdge;
            bool ok = limit_by_neighbours(M, S.w, k, P.beta_w, by_edge, ow);
            ok &= limit_by_neighbours(M, S.uh, k, P.beta_uh, by_edge, ou);
            ok &= limit_by_neighbours(M, S.vh, k, P.beta_vh, by_edge, ov);
            if (!ok) no_nbr = 1;
        } else {
            const bool vel = P.extrapolate_velocity_second_order == 1;
            // centroid values being extrapolated (velocity or momentum)
            const double qu = vel ? S.uvel[k] : uk;
            const double qv = vel ? S.vvel[k] : vk;
            const int nbk = M.nb[k];
            bool keep = false;  // dry: previous vertex values stay
            bool flat = false;  // zero gradient: centroid values at vertices
            if (nbk == 3) {
                flat = true;
            } else {
                const double x = M.cxy[k], y = M.cxy[N + k];
                double dxv[3], dyv[3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    dxv[i] = M.vxy[(2 * i) * N + k] - x;
                    dyv[i] = M.vxy[(2 * i + 1) * N + k] - y;
                }
                if (nbk <= 1) {
                    const int k0 = M.surr[k], k1 = M.surr[N + k], k2 = M.surr[2 * N + k];
                    const double x0 = M.cxy[k0], y0 = M.cxy[N + k0];
                    const double dx1 = M.cxy[k1] - x0, dx2 = M.cxy[k2] - x0;
                    const double dy1 = M.cxy[N + k1] - y0, dy2 = M.cxy[N + k2] - y0;
                    const double area2 = dy2 * dx1 - dy1 * dx2;
                    if (area2 <= 0) {
                        flat = true;
                    } else {
                        const double w0 = S.w[k0], w1 = S.w[k1], w2 = S.w[k2];
                        const double hc = wk - zk;
                        const double h0 = w0 - S.zc[k0];
                        const double h1 = w1 - S.zc[k1];
                        const double h2 = w2 - S.zc[k2];
                        const double hmin = omin(omin(h0, omin(h1, h2)), hc);
                        double hfactor = 0.0;
                        if (hmin > 0.001) hfactor = (hmin - 0.001) / (hmin + 0.004);
                        if (P.optimise_dry_cells && omax(h0, omax(h1, h2)) < P.epsilon) {
                            keep = true;
                        } else {
                            const double inv_area2 = 1.0 / area2;
                            aux_jumps(wk, w0, w1, w2, dx1, dy1, dx2, dy2, inv_area2, dxv, dyv,
                                      P.beta_w_dry + (P.beta_w - P.beta_w_dry) * hfactor, ow);
                            const double u0 = vel ? S.uvel[k0] : S.uh[k0];
                            const double u1 = vel ? S.uvel[k1] : S.uh[k1];
                            const double u2 = vel ? S.uvel[k2] : S.uh[k2];
                            aux_jumps(qu, u0, u1, u2, dx1, dy1, dx2, dy2, inv_area2, dxv, dyv,
                                      P.beta_uh_dry + (P.beta_uh - P.beta_uh_dry) * hfactor, ou);
                            const double v0 = vel ? S.vvel[k0] : S.vh[k0];
                            const double v1 = vel ? S.vvel[k1] : S.vh[k1];
                            const double v2 = vel ? S.vvel[k2] : S.vh[k2];
                            aux_jumps(qv, v0, v1, v2, dx1, dy1, dx2, dy2, inv_area2, dxv, dyv,
                                      P.beta_vh_dry + (P.beta_vh - P.beta_vh_dry) * hfactor, ov);
                        }
                    }
                } else {
                    // the one interior neighbour: first surrogate that is not k
                    int k1 = -1;
#pragma unroll
                    for (int i = 2; i >= 0; i--) {
                        const int s = M.surr[i * N + k];
                        if (s != k) k1 = s;
                    }
                    if (k1 < 0) {
                        no_nbr = 1;
                        flat = true;
                    } else {
                        const double dx1 = M.cxy[k1] - x, dy1 = M.cxy[N + k1] - y;
                        const double area2 = dx1 * dx1 + dy1 * dy1;
                        double dx2 = 1.0 / area2;
                        const double dy2 = dx2 * dy1;
                        dx2 *= dx1;
                        one_nbr_jumps(wk, S.w[k1], dx2, dy2, dxv, dyv, P.beta_w, ow);
                        one_nbr_jumps(qu, vel ? S.uvel[k1] : S.uh[k1], dx2, dy2, dxv, dyv,
                                      P.beta_w, ou);
                        one_nbr_jumps(qv, vel ? S.vvel[k1] : S.vh[k1], dx2, dy2, dxv, dyv,
                                      P.beta_w, ov);
                    }
                }
            }
            if (flat) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    ow[i] = wk;
                    ou[i] = qu;
                    ov[i] = qv;
                }
            } else if (keep) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    ow[i] = S.wv[i * N + k];
                    ou[i] = S.uhv[i * N + k];
                    ov[i] = S.vhv[i * N + k];
                }
            }
            if (vel) {
                // back from velocity to momentum with the vertex depth
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const double dv = omax(ow[i] - zvk[i], 0.);
                    ou[i] = ou[i] * dv;
                    ov[i] = ov[i] * dv;
                }
            }
        }

        if (!(flags & kExtrapolateOnly)) balance_one(P, wk, zk, uk, vk, zvk, ow, ou, ov);

#pragma unroll
        for (int i = 0; i < 3; i++) {
            S.wv[i * N + k] = ow[i];
            S.uhv[i * N + k] = ou[i];
            S.vhv[i * N + k] = ov[i];
        }
        if (flags & kWriteEdges) {
            S.we[k] = 0.5 * (ow[1] + ow[2]);
            S.we[N + k] = 0.5 * (ow[0] + ow[2]);
            S.we[2 * N + k] = 0.5 * (ow[0] + ow[1]);
            S.uhe[k] = 0.5 * (ou[1] + ou[2]);
            S.uhe[N + k] = 0.5 * (ou[0] + ou[2]);
            S.uhe[2 * N + k] = 0.5 * (ou[0] + ou[1]);
            S.vhe[k] = 0.5 * (ov[1] + ov[2]);
            S.vhe[N + k] = 0.5 * (ov[0] + ov[2]);
            S.vhe[2 * N + k] = 0.5 * (ov[0] + ov[1]);
        }
        if ((flags & kWriteBoundary) && M.nb[k] > 0) {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const int pk = M.nbr[i * N + k];
                if (pk < 0) {
                    const int mb = -pk - 1;
                    const int a = (i == 0) ? 1 : 0, b = (i == 2) ? 1 : 2;
                    const double we = 0.5 * (ow[a] + ow[b]);
                    const double uhe = 0.5 * (ou[a] + ou[b]);
                    const double vhe = 0.5 * (ov[a] + ov[b]);
                    double wb, uhb, vhb;
                    if (!eval_boundary(tags[M.btag[mb]], time, we, uhe, vhe,
                                       M.normals[(2 * i) * N + k],
                                       M.normals[(2 * i + 1) * N + k], S.ze[i * N + k], P.g,
                                       wb, uhb, vhb)) {
                        bad_bc = 1;
                        wb = uhb = vhb = 0.0;
                    }
                    S.wb[mb] = wb;
                    S.uhb[mb] = uhb;
                    S.vhb[mb] = vhb;
                    S.zb[mb] = S.ze[i * N + k];
                }
            }
        }
    }
    if (bad_bc) set_status(ctrl, SWGPU_EBOUNDARY);
    if (no_nbr) set_status(ctrl, SWGPU_EMESH);
    if (fused) {
        __syncthreads();
        if (threadIdx.x == 0 && last_block_done(&ctrl->done_distribute, ctrl->blocks_distribute)) apply_pending_halt(ctrl);
    }
}

// update_boundary as a stand-alone pass over boundary slots, from the
// stored vertex values (gpu_domain_advanced.py:2006-2108).
__global__ void __launch_bounds__(kBlock) boundary_fp64(DevMesh M, DevState S, DevParams P,
                                                        const BcTag *tags, Ctrl *ctrl) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.Nb) return;
    const int N = M.N;
    const int k = M.bcell[m], i = M.bedge[m];
    if (M.blk_scen) ctrl += M.blk_scen[k >> 8];  // the owning scenario's time
    const int a = (i == 0) ? 1 : 0, b = (i == 2) ? 1 : 2;
    // the 'tsunami' distribute stores its edge values; otherwise they are the
    // interpolation of the vertex values
    const double we = P.flow_algorithm ? S.we[i * N + k]
                                       : 0.5 * (S.wv[a * N + k] + S.wv[b * N + k]);
    const double uhe = P.flow_algorithm ? S.uhe[i * N + k]
                                        : 0.5 * (S.uhv[a * N + k] + S.uhv[b * N + k]);
    const double vhe = P.flow_algorithm ? S.vhe[i * N + k]
                                        : 0.5 * (S.vhv[a * N + k] + S.vhv[b * N + k]);
    double wb, uhb, vhb;
    if (!eval_boundary(tags[M.btag[m]], ctrl->time, we, uhe, vhe, M.normals[(2 * i) * N + k],
                       M.normals[(2 * i + 1) * N + k], S.ze[i * N + k], P.g, wb, uhb, vhb)) {
        set_status(ctrl, SWGPU_EBOUNDARY);
        wb = uhb = vhb = 0.0;
    }
    S.wb[m] = wb;
    S.uhb[m] = uhb;
    S.vhb[m] = vhb;
    S.zb[m] = S.ze[i * N + k];
}

// interpolate_from_vertices_to_edges for stage, xmom, ymom (quantity.c:687-706).
__global__ void __launch_bounds__(kBlock) interpolate_fp64(DevMesh M, DevState S) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = M.N;
    if (k >= N) return;
    const double *V[3] = {S.wv, S.uhv, S.vhv};
    double *E[3] = {S.we, S.uhe, S.vhe};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const double q0 = V[q][k], q1 = V[q][N + k], q2 = V[q][2 * N + k];
        E[q][k] = 0.5 * (q1 + q2);
        E[q][N + k] = 0.5 * (q0 + q2);
        E[q][2 * N + k] = 0.5 * (q0 + q1);
    }
}

// update_centroids_of_velocities_and_height
// (update_centroids_of_velocities_and_height.cu:1-52), centroids and
// boundary slots.
__global__ void __launch_bounds__(kBlock) other_quantities(DevMesh M, DevState S) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const double H0 = 1.0e-8;
    if (k < M.N) {
        double h = S.w[k] - S.zc[k];
        if (h < 0) h = 0;
        const double f = h / (h * h + H0);
        S.hc[k] = h;
        S.uc[k] = S.uh[k] * f;
        S.vc[k] = S.vh[k] * f;
    }
    if (k < M.Nb) {
        double h = S.wb[k] - S.zb[k];
        if (h < 0) h = 0;
        const double f = h / (h * h + H0);
        S.hb[k] = h;
        S.ub[k] = S.uhb[k] * f;
        S.vb[k] = S.vhb[k] * f;
    }
}

// Water volume: per-block partial sums in a fixed order, then one block adds
// the partials in index order (deterministic).
__global__ void __launch_bounds__(kBlock) mass_partials(DevMesh M, DevState S) {
    __shared__ double sh[kBlock];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    sh[threadIdx.x] = k < M.N ? M.areas[k] * (S.w[k] - S.zc[k]) : 0.0;
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) S.partials[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kBlock) mass_final(const double *partials, int n, double *out) {
    __shared__ double sh[kBlock];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partials[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int t = kBlock / 2; t > 0; t >>= 1) {
        if ((int)threadIdx.x < t) sh[threadIdx.x] += sh[threadIdx.x + t];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// ------------------------------------------------------------ launches ---

void launch_prepare_fp64(const DevMesh &M, const DevState &S, const DevParams &P, Ctrl *,
                         cudaStream_t st) {
    prepare_fp64<<<grid_for(M.N), kBlock, 0, st>>>(M, S, P);
}
// Block sizes of the fused-step kernels come from M.shape.
void launch_distribute_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                            const BcTag *tags, Ctrl *ctrl, int flags, cudaStream_t st) {
    const int bs = M.shape.distribute, g = (M.n_launch + bs - 1) / bs;
    if (P.flow_algorithm) {
        if (bs == 128)
            distribute_de_fp64<128><<<g, 128, 0, st>>>(M, S, P, tags, ctrl, flags);
        else if (bs == 512)
            distribute_de_fp64<512><<<g, 512, 0, st>>>(M, S, P, tags, ctrl, flags);
        else
            distribute_de_fp64<256><<<g, 256, 0, st>>>(M, S, P, tags, ctrl, flags);
    } else if (bs == 128)
        distribute_fp64<128><<<g, 128, 0, st>>>(M, S, P, tags, ctrl, flags);
    else if (bs == 512)
        distribute_fp64<512><<<g, 512, 0, st>>>(M, S, P, tags, ctrl, flags);
    else
        distribute_fp64<256><<<g, 256, 0, st>>>(M, S, P, tags, ctrl, flags);
}
void launch_boundary_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                          const BcTag *tags, Ctrl *ctrl,
                          cudaStream_t st) {
    if (M.Nb > 0) boundary_fp64<<<grid_for(M.Nb), kBlock, 0, st>>>(M, S, P, tags, ctrl);
}
void launch_flux_fp64(const DevMesh &M, const DevState &S, const DevParams &P, Ctrl *ctrl,
                      int flags, cudaStream_t st) {
    const int bs = M.shape.flux, g = (M.n_launch + bs - 1) / bs;
    if (bs == 64)
        flux_fp64<64><<<g, 64, 0, st>>>(M, S, P, ctrl, flags);
    else if (bs == 128)
        flux_fp64<128><<<g, 128, 0, st>>>(M, S, P, ctrl, flags);
    else
        flux_fp64<256><<<g, 256, 0, st>>>(M, S, P, ctrl, flags);
}
void launch_forcing_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                         bool explicit_target, cudaStream_t st) {
    forcing_fp64<<<grid_for(M.N), kBlock, 0, st>>>(M, S, P, explicit_target ? 1 : 0);
}
void launch_velocities_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                            cudaStream_t st) {
    velocities_fp64<<<grid_for(M.N), kBlock, 0, st>>>(M, S, P);
}
void launch_balance_fp64(const DevMesh &M, const DevState &S, const DevParams &P,
                         cudaStream_t st) {
    balance_fp64<<<grid_for(M.N), kBlock, 0, st>>>(M, S, P);
}
void launch_update_fp64(const DevMesh &M, const DevState &S, const DevParams &P, Ctrl *ctrl,
                        double dt, int flags, const Stage &stage, cudaStream_t st) {
    const int bs = M.shape.update, g = (M.n_launch + bs - 1) / bs;
    if (bs == 128)
        update_fp64<128><<<g, 128, 0, st>>>(M, S, P, ctrl, dt, flags, stage);
    else if (bs == 512)
        update_fp64<512><<<g, 512, 0, st>>>(M, S, P, ctrl, dt, flags, stage);
    else
        update_fp64<256><<<g, 256, 0, st>>>(M, S, P, ctrl, dt, flags, stage);
}
void launch_saxpy_fp64(const DevMesh &M, const DevState &S, double a, double b,
                       cudaStream_t st) {
    saxpy_fp64<<<grid_for(M.N), kBlock, 0, st>>>(M.N, a, b, S.w, S.uh, S.vh, S.bw, S.buh,
                                                 S.bvh);
}
void launch_interpolate_fp64(const DevMesh &M, const DevState &S, cudaStream_t st) {
    interpolate_fp64<<<grid_for(M.N), kBlock, 0, st>>>(M, S);
}
void launch_other_quantities(const DevMesh &M, const DevState &S, cudaStream_t st) {
    const int n = M.N > M.Nb ? M.N : M.Nb;
    other_quantities<<<grid_for(n), kBlock, 0, st>>>(M, S);
}
void launch_mass_partials(const DevMesh &M, const DevState &S, cudaStream_t st) {
    mass_partials<<<grid_for(M.N), kBlock, 0, st>>>(M, S);
}
void launch_mass(const DevMesh &M, const DevState &S, double *out, cudaStream_t st) {
    const int g = grid_for(M.N);
    mass_partials<<<g, kBlock, 0, st>>>(M, S);
    mass_final<<<1, kBlock, 0, st>>>(S.partials, g, out);
}

}  // namespace swgpu
