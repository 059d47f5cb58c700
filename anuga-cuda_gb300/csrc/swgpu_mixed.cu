// swgpu_mixed.cu -- mixed-precision evolve kernels.
//
// The same ANUGA algorithm as the FP64 path (limiter, central-upwind flux,
// gravity_wb, Manning friction, protect, balance), restructured for an
// HBM-bound GB300 kernel:
//   * conserved state is FP64 depth h (not stage) and FP64 momentum; the
//     update h += dt*E, uh += dt*E (then the friction factor) stays FP64;
//   * everything the limiter, extrapolation and flux read is FP32: centroid
//     depth and velocities, vertex depth and momentum, normals, lengths,
//     1/area, radii and per-triangle coefficients precomputed in FP64 on the
//     host relative to the triangle's own centroid (so no FP32 arithmetic
//     ever sees an absolute coordinate);
//   * stage differences for the limiter are depth differences plus
//     precomputed bed differences; the flux uses depths directly (the bed is
//     continuous across an edge, so w_r - w_l = h_r - h_l);
//   * the gravity term's stage gradient is the depth gradient (Green's
//     theorem over the edge midpoints, exact for the linear reconstruction)
//     plus the precomputed bed gradient.
// Bytes per triangle-step (own arrays; neighbour gathers hit L1/L2):
//   distribute ~109, flux ~116, update ~80.
#include <algorithm>
#include <cmath>
#include <vector>

#include "swgpu_device.cuh"
#include "swgpu_handle.cuh"

namespace swgpu {

// Read-only loads through the non-coherent path (the arrays a kernel reads
// are never written by the same kernel).
template <typename T>
__device__ __forceinline__ T ro(const T *p) {
    return __ldg(p);
}

// _compute_speed (shallow_water_ext.c:214-242) for both momentum components
// of one side of an edge with a single division: for h < lim the limited
// speed uh/(h + h0/h) is uh * h/(h*h + h0), and the momentum is reset to
// speed * h.
__device__ __forceinline__ void side_speed_f(float &h, float &uh, float &vh, float &u,
                                             float eps, float h0, float lim) {
    if (h < lim) {
        if (h < eps) {
            h = 0.0f;
            u = 0.0f;
            uh = 0.0f;
            vh = 0.0f;
        } else {
            const float f = __fdividef(h, h * h + h0);
            u = uh * f;
            uh = u * h;
            vh = (vh * f) * h;
        }
    } else {
        u = __fdividef(uh, h);
    }
}

// Central-upwind flux on depths (rotated frame inside), FP32.  The stage
// jump equals the depth jump (bed continuous across the edge).
__device__ __forceinline__ void central_flux_f(float hl_in, float uhl_in, float vhl_in,
                                               float hr_in, float uhr_in, float vhr_in, float n1,
                                               float n2, float g, float eps, float h0, float lim,
                                               float &f0, float &f1, float &f2, float &ms) {
    const float al = n1 * uhl_in + n2 * vhl_in;
    const float bl = -n2 * uhl_in + n1 * vhl_in;
    const float ar = n1 * uhr_in + n2 * vhr_in;
    const float br = -n2 * uhr_in + n1 * vhr_in;
    float hl = hl_in, uhl = al, vhl = bl, ul;
    float hr = hr_in, uhr = ar, vhr = br, ur;
    side_speed_f(hl, uhl, vhl, ul, eps, h0, lim);
    side_speed_f(hr, uhr, vhr, ur, eps, h0, lim);
    const float cl = sqrtf(g * hl), cr = sqrtf(g * hr);
    float smax = omaxf(ul + cl, ur + cr);
    if (smax < 0.0f) smax = 0.0f;
    float smin = ominf(ul - cl, ur - cr);
    if (smin > 0.0f) smin = 0.0f;
    const float denom = smax - smin;
    if (denom < eps) {
        f0 = f1 = f2 = 0.0f;
        ms = 0.0f;
        return;
    }
    const float inv = __fdividef(1.0f, denom);
    const float ss = smax * smin;
    const float fl0 = ul * hl, fl1 = ul * uhl + 0.5f * g * hl * hl, fl2 = ul * vhl;
    const float fr0 = ur * hr, fr1 = ur * uhr + 0.5f * g * hr * hr, fr2 = ur * vhr;
    const float e0 = (smax * fl0 - smin * fr0 + ss * (hr_in - hl_in)) * inv;
    const float e1 = (smax * fl1 - smin * fr1 + ss * (ar - al)) * inv;
    const float e2 = (smax * fl2 - smin * fr2 + ss * (br - bl)) * inv;
    ms = omaxf(fabsf(smax), fabsf(smin));
    f0 = e0;
    f1 = n1 * e1 - n2 * e2;
    f2 = n2 * e1 + n1 * e2;
}

// flux + gravity_wb, FP32, triangle centric.
__global__ void __launch_bounds__(kBlock) flux_mixed(DevMesh M, DevMixed X, DevParams P,
                                                     Ctrl *ctrl, int flags) {
    if ((flags & kFused) && ctrl_halted(ctrl)) return;
    const int N = M.N;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    float t = P.f_max_dt;
    if (k < N) {
        const float g = P.f_g, eps = P.f_eps;
        const float h0 = P.f_h0, lim = P.f_lim;
        float vh[3], vu[3], vv[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            vh[i] = ro(X.hv + i * N + k);
            vu[i] = ro(X.uhv + i * N + k);
            vv[i] = ro(X.vhv + i * N + k);
        }
        const float he[3] = {0.5f * (vh[1] + vh[2]), 0.5f * (vh[0] + vh[2]), 0.5f * (vh[0] + vh[1])};
        const float ue[3] = {0.5f * (vu[1] + vu[2]), 0.5f * (vu[0] + vu[2]), 0.5f * (vu[0] + vu[1])};
        const float ve[3] = {0.5f * (vv[1] + vv[2]), 0.5f * (vv[0] + vv[2]), 0.5f * (vv[0] + vv[1])};
        const float rk = ro(X.radius + k);
        const float inv_area = ro(X.inv_area + k);
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;            // flux sums
        float gx = 0.f, gy = 0.f, sx = 0.f, sy = 0.f;  // Green gradient, side term
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const int pk = ro(M.nbr + i * N + k);
            const float n1 = ro(X.nx + i * N + k), n2 = ro(X.ny + i * N + k);
            const float L = ro(X.len + i * N + k);
            float hr, uhr, vhr, rn = 3.0e38f;
            if (pk >= 0) {
                const int n = pk >> 2, m = pk & 3;
                const int a = (m == 0) ? 1 : 0, b = (m == 2) ? 1 : 2;
                hr = 0.5f * (ro(X.hv + a * N + n) + ro(X.hv + b * N + n));
                uhr = 0.5f * (ro(X.uhv + a * N + n) + ro(X.uhv + b * N + n));
                vhr = 0.5f * (ro(X.vhv + a * N + n) + ro(X.vhv + b * N + n));
                rn = ro(X.radius + n);
            } else {
                const int mb = -pk - 1;
                hr = ro(X.hbf + mb);
                uhr = ro(X.uhbf + mb);
                vhr = ro(X.vhbf + mb);
            }
            const float hl = he[i];
            const float hlL = hl * L;
            gx += hlL * n1;
            gy += hlL * n2;
            const float fact = -0.5f * g * hl * hlL;
            sx += fact * n1;
            sy += fact * n2;
            if (P.optimise_dry_cells && fabsf(hl) < eps && fabsf(hr) < eps) continue;
            float f0, f1, f2, ms;
            central_flux_f(hl, ue[i], ve[i], hr, uhr, vhr, n1, n2, g, eps, h0, lim, f0, f1, f2, ms);
            a0 -= f0 * L;
            a1 -= f1 * L;
            a2 -= f2 * L;
            if (ms > eps) {
                // min(rk/ms, rn/ms) = min(rk, rn)/ms: one division per edge
                t = ominf(t, __fdividef(fminf(rk, rn), ms));
            }
        }
        const float avg_h = ro(X.hf + k);
        const float wx = gx * inv_area + ro(X.zgrad + k);
        const float wy = gy * inv_area + ro(X.zgrad + N + k);
        X.ew[k] = a0 * inv_area;
        X.euh[k] = a1 * inv_area - g * wx * avg_h - sx * inv_area;
        X.evh[k] = a2 * inv_area - g * wy * avg_h - sy * inv_area;
    }
    block_min_timestep_f(t, ctrl);
    if ((flags & kFused) && threadIdx.x == 0 && last_block_done(&ctrl->done_flux))
        publish_step_clock(ctrl, P);
}

// Update: the conserved state stays FP64 and is advanced by increments
// computed in FP32 (each increment is small against the value it is added
// to, so its FP32 rounding is far below the FP32 resolution of the state;
// the additions themselves are FP64):
//   h  += dt*E_h
//   q  += q*(r - 1) + dt*E_q*r,   r = 1/(1 - dt*S)  (semi-implicit Manning)
// then protect and the FP32 centroid copies the next extrapolation reads.
__global__ void __launch_bounds__(kBlock) update_mixed(DevMesh M, DevState S, DevMixed X,
                                                       DevParams P, Ctrl *ctrl, int flags) {
    if ((flags & kFused) && ctrl_halted(ctrl)) return;
    const StepClock clk = published_step_clock(ctrl);
    const double dt = clk.dt;
    const float dtf = (float)dt;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int bad = 0, nonfinite = 0;
    if (k < M.N) {
        double h = X.hd[k], uh = S.uh[k], vh = S.vh[k];
        const float mah = P.f_mah;
        const float hf0 = ro(X.hf + k);  // FP32 copy of h written last step
        const float uf = ro(X.uvel + k) * omaxf(hf0, mah);
        const float vf = ro(X.vvel + k) * omaxf(hf0, mah);
        // Manning friction on the pre-update state
        float rm1 = 0.0f, r = 1.0f;  // r - 1 and r
        const float eta = ro(X.fric + k);
        if (eta > mah) {
            const float hm = hf0 - ro(X.zmoff + k);
            if (hm >= mah) {
                const float Sf = -P.f_g * eta * eta * sqrtf(uf * uf + vf * vf) *
                                 exp2f(-(7.0f / 3.0f) * __log2f(hm));
                const float dS = dtf * Sf;         // <= 0
                const float den = 1.0f - dS;
                if (!(den > 0.0f)) bad = 1;
                r = __fdividef(1.0f, den);
                rm1 = dS * r;                      // r - 1 without cancellation
            }
        }
        const float dh = dtf * ro(X.ew + k);
        const float du = uf * rm1 + dtf * ro(X.euh + k) * r;
        const float dv = vf * rm1 + dtf * ro(X.evh + k) * r;
        h += (double)dh;
        uh += (double)du;
        vh += (double)dv;
        // FP32 copies re-derived from the FP64 state (no drift between them)
        float hf = (float)h;
        float uhf = (float)uh, vhf = (float)vh;
        // protect (shallow_water_ext.c:1638-1705) on depth
        if (hf < mah) {
            if (P.f_mas < P.f_eps) {
                uh = vh = 0.0;
                uhf = vhf = 0.0f;
                if (h <= 0.0) {
                    h = 0.0;
                    hf = 0.0f;
                }
            } else if (h <= 0.0) {
                h = uh = vh = 0.0;
                hf = uhf = vhf = 0.0f;
            } else {
                const float u = uhf / hf, v = vhf / hf, ms = P.f_mas;
                if (fabsf(u) > ms) uhf = (u > 0 ? ms : -ms) * hf;
                if (fabsf(v) > ms) vhf = (v > 0 ? ms : -ms) * hf;
                uh = (double)uhf;
                vh = (double)vhf;
            }
        }
        // NaN / Inf anywhere in the new state stops the run (FP32 copies:
        // a non-finite FP64 value stays non-finite when narrowed)
        if (!(fabsf(hf) <= 3.0e38f) || !(fabsf(uhf) <= 3.0e38f) || !(fabsf(vhf) <= 3.0e38f))
            nonfinite = 1;
        X.hd[k] = h;
        S.uh[k] = uh;
        S.vh[k] = vh;
        X.hf[k] = hf;
        const float inv = __fdividef(1.0f, omaxf(hf, mah));
        X.uvel[k] = uhf * inv;
        X.vvel[k] = vhf * inv;
    }
    if (bad) set_status(ctrl, SWGPU_EDENOMINATOR);
    if (nonfinite) set_status(ctrl, SWGPU_ENONFINITE);
    if (flags & kFused) {
        __syncthreads();
        if (threadIdx.x == 0 && last_block_done(&ctrl->done_update)) commit_step(ctrl, clk, P);
    }
}

__device__ __forceinline__ void qminmax_f(float dq0, float dq1, float dq2, float &qmin,
                                          float &qmax) {
    if (dq0 >= 0.0f) {
        if (dq1 >= dq2) {
            qmax = (dq1 >= 0.0f) ? dq0 + dq1 : dq0;
            qmin = dq0 + dq2;
            if (qmin >= 0.0f) qmin = 0.0f;
        } else {
            qmax = (dq2 > 0.0f) ? dq0 + dq2 : dq0;
            qmin = dq0 + dq1;
            if (qmin >= 0.0f) qmin = 0.0f;
        }
    } else {
        if (dq1 <= dq2) {
            qmin = (dq1 < 0.0f) ? dq0 + dq1 : dq0;
            qmax = dq0 + dq2;
            if (qmax <= 0.0f) qmax = 0.0f;
        } else {
            qmin = (dq2 < 0.0f) ? dq0 + dq2 : dq0;
            qmax = dq0 + dq1;
            if (qmax <= 0.0f) qmax = 0.0f;
        }
    }
}

__device__ __forceinline__ void limit_f(float (&d)[3], float qmin, float qmax, float beta) {
    const float TINY = 1.0e-30f;
    float r = 1000.0f, r0 = 1.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (d[i] < -TINY) r0 = qmin / d[i];
        if (d[i] > TINY) r0 = qmax / d[i];
        r = ominf(r0, r);
    }
    const float phi = ominf(r * beta, 1.0f);
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] *= phi;
}

// jumps on the auxiliary triangle: d_i = c_i0*dq1 + c_i1*dq2, limited
__device__ __forceinline__ void aux_jumps_f(float dq0, float dq1, float dq2, const float (&c)[6],
                                            float beta, float (&d)[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] = c[2 * i] * dq1 + c[2 * i + 1] * dq2;
    float qmin, qmax;
    qminmax_f(dq0, dq1, dq2, qmin, qmax);
    limit_f(d, qmin, qmax, beta);
}

__device__ __forceinline__ void one_jumps_f(float dq1, const float (&c)[6], float beta,
                                            float (&d)[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] = c[2 * i] * dq1;
    const float qmin = dq1 >= 0.0f ? 0.0f : dq1, qmax = dq1 >= 0.0f ? dq1 : 0.0f;
    limit_f(d, qmin, qmax, beta);
}

// extrapolation + balance + boundary conditions, FP32 on depths.
__global__ void __launch_bounds__(kBlock) distribute_mixed(DevMesh M, DevState S, DevMixed X,
                                                           DevParams P, const BcTag *tags,
                                                           Ctrl *ctrl, int flags) {
    const bool fused = flags & kFused;
    if (fused && ctrl_halted(ctrl)) return;
    const int N = M.N;
    const int order = (int)ctrl->order;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int bad_bc = 0;
    if (k < N) {
        const float mah = P.f_mah;
        const float hc = ro(X.hf + (k));
        const float qu = ro(X.uvel + (k)), qv = ro(X.vvel + (k));
        const bool vel = P.extrapolate_velocity_second_order == 1;
        // centroid momentum (uvel = uh / max(h, mah))
        const float uk = qu * omaxf(hc, mah), vk = qv * omaxf(hc, mah);
        float dzv[3];
#pragma unroll
        for (int i = 0; i < 3; i++) dzv[i] = ro(X.dzv + (i * N + k));
        float oh[3], ou[3], ov[3];  // vertex depth, momentum (or velocity)
        bool flat = order == 1;
        if (order != 1) {
            const int kind = ro(X.kind + (k));
            const float cu = vel ? qu : uk, cv = vel ? qv : vk;
            if ((kind & 3) == 2) {
                flat = true;
            } else {
                float c[6];
#pragma unroll
                for (int j = 0; j < 6; j++) c[j] = ro(X.gc + (j * N + k));
                float dw[3] = {0.f, 0.f, 0.f}, du[3] = {0.f, 0.f, 0.f}, dv[3] = {0.f, 0.f, 0.f};
                bool keep = false;  // dry neighbourhood: previous vertex values stay
                if ((kind & 3) == 0) {
                    const int k0 = ro(M.surr + (k)), k1 = ro(M.surr + (N + k)), k2 = ro(M.surr + (2 * N + k));
                    const float h0 = ro(X.hf + (k0)), h1 = ro(X.hf + (k1)), h2 = ro(X.hf + (k2));
                    const float hmin = ominf(ominf(h0, ominf(h1, h2)), hc);
                    const float hmax = omaxf(h0, omaxf(h1, h2));
                    if (P.optimise_dry_cells && hmax < P.f_eps) {
                        keep = true;
                    } else {
                        float hfactor = 0.0f;
                        if (hmin > 0.001f) hfactor = (hmin - 0.001f) / (hmin + 0.004f);
                        const float z0 = ro(X.dzn + (k)), z1 = ro(X.dzn + (N + k)), z2 = ro(X.dzn + (2 * N + k));
                        // stage differences = depth differences + bed differences
                        const float dq0 = (h0 - hc) + z0;
                        const float dq1 = (h1 - h0) + (z1 - z0);
                        const float dq2 = (h2 - h0) + (z2 - z0);
                        aux_jumps_f(dq0, dq1, dq2, c,
                                    P.f_beta_w_dry + (P.f_beta_w - P.f_beta_w_dry) * hfactor,
                                    dw);
                        const float u0 = vel ? ro(X.uvel + (k0)) : ro(X.uvel + (k0)) * omaxf(h0, mah);
                        const float u1 = vel ? ro(X.uvel + (k1)) : ro(X.uvel + (k1)) * omaxf(h1, mah);
                        const float u2 = vel ? ro(X.uvel + (k2)) : ro(X.uvel + (k2)) * omaxf(h2, mah);
                        aux_jumps_f(u0 - cu, u1 - u0, u2 - u0, c,
                                    P.f_beta_uh_dry + (P.f_beta_uh - P.f_beta_uh_dry) * hfactor,
                                    du);
                        const float v0 = vel ? ro(X.vvel + (k0)) : ro(X.vvel + (k0)) * omaxf(h0, mah);
                        const float v1 = vel ? ro(X.vvel + (k1)) : ro(X.vvel + (k1)) * omaxf(h1, mah);
                        const float v2 = vel ? ro(X.vvel + (k2)) : ro(X.vvel + (k2)) * omaxf(h2, mah);
                        aux_jumps_f(v0 - cv, v1 - v0, v2 - v0, c,
                                    P.f_beta_vh_dry + (P.f_beta_vh - P.f_beta_vh_dry) * hfactor,
                                    dv);
                    }
                } else {
                    const int slot = (kind >> 2) & 3;
                    const int k1 = ro(M.surr + (slot * N + k));
                    const float h1 = ro(X.hf + (k1));
                    const float beta = P.f_beta_w;
                    one_jumps_f((h1 - hc) + ro(X.dzn + (slot * N + k)), c, beta, dw);
                    const float u1 = vel ? ro(X.uvel + (k1)) : ro(X.uvel + (k1)) * omaxf(h1, mah);
                    const float v1 = vel ? ro(X.vvel + (k1)) : ro(X.vvel + (k1)) * omaxf(h1, mah);
                    one_jumps_f(u1 - cu, c, beta, du);
                    one_jumps_f(v1 - cv, c, beta, dv);
                }
                if (keep) {
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        oh[i] = X.hv[i * N + k];
                        ou[i] = X.uhv[i * N + k];
                        ov[i] = X.vhv[i * N + k];
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        // vertex depth = centroid depth + stage jump - bed jump
                        oh[i] = (hc + dw[i]) - dzv[i];
                        ou[i] = cu + du[i];
                        ov[i] = cv + dv[i];
                    }
                }
            }
            if (flat) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    oh[i] = hc - dzv[i];
                    ou[i] = cu;
                    ov[i] = cv;
                }
            }
            if (vel) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float d = omaxf(oh[i], 0.0f);
                    ou[i] *= d;
                    ov[i] *= d;
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                oh[i] = hc - dzv[i];
                ou[i] = uk;
                ov[i] = vk;
            }
        }
        // balance_deep_and_shallow on depths (w_v - z_v = h_v)
        {
            const float H0 = P.f_H0;
            const float hmin = ominf(oh[0], ominf(oh[1], oh[2]));
            float alpha = 1.0f;
            if (P.tight_slope_limiters == 0) {
                float dz = 0.0f;
#pragma unroll
                for (int i = 0; i < 3; i++) dz = omaxf(dz, fabsf(dzv[i]));
                alpha = dz > 0.0f ? omaxf(ominf(P.f_alpha * hmin / dz, 1.0f), 0.0f)
                                  : 1.0f;
            } else if (hmin < H0) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float hd = hc - oh[i];
                    if (!(hd <= 0.0f)) alpha = ominf(alpha, (hc - H0) / hd);
                }
                alpha = fminf(fmaxf(alpha, 0.0f), 1.0f);
            }
            if (alpha < 1.0f) {
                const float uc = hc > 1.0e-6f ? uk / hc : 0.0f;
                const float vc = hc > 1.0e-6f ? vk / hc : 0.0f;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    oh[i] = (1.0f - alpha) * hc + alpha * oh[i];
                    if (P.use_centroid_velocities == 1) {
                        ou[i] = uc * oh[i];
                        ov[i] = vc * oh[i];
                    } else {
                        ou[i] = (1.0f - alpha) * uk + alpha * ou[i];
                        ov[i] = (1.0f - alpha) * vk + alpha * ov[i];
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 3; i++) {
            X.hv[i * N + k] = oh[i];
            X.uhv[i * N + k] = ou[i];
            X.vhv[i * N + k] = ov[i];
        }
        if ((flags & kWriteBoundary) && ro(M.nb + (k)) > 0) {
            const double time = ctrl->time;
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const int pk = ro(M.nbr + (i * N + k));
                if (pk < 0) {
                    const int mb = -pk - 1;
                    const int a = (i == 0) ? 1 : 0, b = (i == 2) ? 1 : 2;
                    const double ze = ro(S.ze + (i * N + k));
                    const float he = 0.5f * (oh[a] + oh[b]);
                    const double we = ze + (double)he;
                    const double uhe = 0.5 * ((double)ou[a] + (double)ou[b]);
                    const double vhe = 0.5 * ((double)ov[a] + (double)ov[b]);
                    double wb, uhb, vhb;
                    if (!eval_boundary(tags[ro(M.btag + (mb))], time, we, uhe, vhe,
                                       (double)ro(X.nx + (i * N + k)), (double)ro(X.ny + (i * N + k)), wb, uhb,
                                       vhb)) {
                        bad_bc = 1;
                        wb = we;
                        uhb = vhb = 0.0;
                    }
                    S.wb[mb] = wb;
                    S.uhb[mb] = uhb;
                    S.vhb[mb] = vhb;
                    S.zb[mb] = ze;
                    // reflective keeps the edge depth exactly; others from the stage
                    X.hbf[mb] = tags[ro(M.btag + (mb))].type == SWGPU_BC_REFLECTIVE ? he
                                                                               : (float)(wb - ze);
                    X.uhbf[mb] = (float)uhb;
                    X.vhbf[mb] = (float)vhb;
                }
            }
        }
    }
    if (bad_bc) set_status(ctrl, SWGPU_EBOUNDARY);
    if (fused) {
        __syncthreads();
        if (threadIdx.x == 0 && last_block_done(&ctrl->done_distribute)) apply_pending_halt(ctrl);
    }
}

// Depth from the FP64 stage (after an upload) or from the mixed state, then
// protect and the FP32 centroid copies.
__global__ void __launch_bounds__(kBlock) prepare_mixed(DevMesh M, DevState S, DevMixed X,
                                                        DevParams P, int from_stage) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M.N) return;
    double h = from_stage ? S.w[k] - S.zc[k] : X.hd[k];
    double uh = S.uh[k], vh = S.vh[k];
    if (h < P.minimum_allowed_height) {
        if (P.f_mas < P.f_eps) {
            uh = 0.0;
            vh = 0.0;
            if (h <= 0.0) h = 0.0;
        } else if (h <= 0.0) {
            h = 0.0;
            uh = 0.0;
            vh = 0.0;
        } else {
            const double u = uh / h, v = vh / h, ms = P.maximum_allowed_speed;
            if (fabs(u) > ms) uh = (u > 0 ? ms : -ms) * h;
            if (fabs(v) > ms) vh = (v > 0 ? ms : -ms) * h;
        }
    }
    X.hd[k] = h;
    S.uh[k] = uh;
    S.vh[k] = vh;
    const float hf = (float)h, mah = P.f_mah;
    X.hf[k] = hf;
    X.uvel[k] = (float)uh / omaxf(hf, mah);
    X.vvel[k] = (float)vh / omaxf(hf, mah);
}

// FP64 stage centroid / vertex values and momentum vertex values for
// downloads: w = h + z.
__global__ void __launch_bounds__(kBlock) vertices_from_mixed(DevMesh M, DevState S, DevMixed X) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = M.N;
    if (k >= N) return;
    S.w[k] = X.hd[k] + S.zc[k];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        S.wv[i * N + k] = (double)X.hv[i * N + k] + S.zv[i * N + k];
        S.uhv[i * N + k] = (double)X.uhv[i * N + k];
        S.vhv[i * N + k] = (double)X.vhv[i * N + k];
    }
}

__global__ void __launch_bounds__(kBlock) mass_partials_mixed(DevMesh M, DevState S, DevMixed X) {
    __shared__ double sh[kBlock];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    sh[threadIdx.x] = k < M.N ? M.areas[k] * X.hd[k] : 0.0;
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) S.partials[blockIdx.x] = sh[0];
}

__global__ void mass_final_mixed(const double *partials, int n, double *out) {
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

void launch_distribute_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                             const DevParams &P, const BcTag *tags, Ctrl *ctrl, int flags,
                             cudaStream_t st) {
    distribute_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, S, X, P, tags, ctrl, flags);
}
void launch_flux_mixed(const DevMesh &M, const DevState &, const DevMixed &X, const DevParams &P,
                       Ctrl *ctrl, int flags, cudaStream_t st) {
    flux_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, X, P, ctrl, flags);
}
void launch_update_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                         const DevParams &P, Ctrl *ctrl, int flags, cudaStream_t st) {
    update_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, S, X, P, ctrl, flags);
}
void launch_prepare_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                          const DevParams &P, int from_stage, cudaStream_t st) {
    prepare_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, S, X, P, from_stage);
}
void launch_vertices_from_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                                cudaStream_t st) {
    vertices_from_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, S, X);
}
void launch_mass_mixed(const DevMesh &M, const DevState &S, const DevMixed &X, double *out,
                       cudaStream_t st) {
    const int g = grid_for(M.N);
    mass_partials_mixed<<<g, kBlock, 0, st>>>(M, S, X);
    mass_final_mixed<<<1, kBlock, 0, st>>>(S.partials, g, out);
}

// ------------------------------------------------------ host geometry ---

// FP32 per-triangle coefficients of the mixed path, computed in FP64 from
// the host geometry and the current bed (downloaded) and friction.
int build_mixed_geometry(Handle *h) {
    const int N = h->M.N;
    const size_t n1 = N, n3 = 3 * (size_t)N;
    std::vector<double> zc(n1), zv(n3), ze(n3), fr(n1);
    cudaStreamSynchronize(h->stream);
    if (cudaMemcpy(zc.data(), h->S.zc, n1 * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(zv.data(), h->S.zv, n3 * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ze.data(), h->S.ze, n3 * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(fr.data(), h->S.fric, n1 * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return SWGPU_ECUDA;
    std::vector<float> nx(n3), ny(n3), len(n3), inv_area(n1), radius(n1), gc(6 * n1), dzn(n3),
        dzv(n3), zgrad(2 * n1), fric(n1), zmoff(n1);
    std::vector<uint8_t> kind(n1);
    const std::vector<double> &V = h->h_vxy, &C = h->h_cxy;
    for (int k = 0; k < N; k++) {
        for (int i = 0; i < 3; i++) {
            nx[i * n1 + k] = (float)h->h_normals[(2 * i) * n1 + k];
            ny[i * n1 + k] = (float)h->h_normals[(2 * i + 1) * n1 + k];
            len[i * n1 + k] = (float)h->h_len[i * n1 + k];
            dzv[i * n1 + k] = (float)(zv[i * n1 + k] - zc[k]);
            dzn[i * n1 + k] = (float)(zc[h->h_surr[i * n1 + k]] - zc[k]);
        }
        inv_area[k] = (float)(1.0 / h->h_areas[k]);
        radius[k] = (float)h->h_radii[k];
        fric[k] = (float)fr[k];
        zmoff[k] = (float)((zv[k] + zv[n1 + k] + zv[2 * n1 + k]) / 3.0 - zc[k]);
        const double x0 = V[0 * n1 + k], y0 = V[1 * n1 + k], x1 = V[2 * n1 + k],
                     y1 = V[3 * n1 + k], x2 = V[4 * n1 + k], y2 = V[5 * n1 + k];
        const double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
        const double z0 = zv[k], z1 = zv[n1 + k], z2 = zv[2 * n1 + k];
        zgrad[k] = (float)(((y2 - y0) * (z1 - z0) - (y1 - y0) * (z2 - z0)) / det);
        zgrad[n1 + k] = (float)(((x1 - x0) * (z2 - z0) - (x2 - x0) * (z1 - z0)) / det);
        const double x = C[k], y = C[n1 + k];
        double dxv[3], dyv[3];
        for (int i = 0; i < 3; i++) {
            dxv[i] = V[(2 * i) * n1 + k] - x;
            dyv[i] = V[(2 * i + 1) * n1 + k] - y;
        }
        const int nbk = h->h_nb[k];
        uint8_t kd = 2;
        double c[6] = {0, 0, 0, 0, 0, 0};
        if (nbk <= 1) {
            const int k0 = h->h_surr[k], k1 = h->h_surr[n1 + k], k2 = h->h_surr[2 * n1 + k];
            const double X0 = C[k0], Y0 = C[n1 + k0];
            const double dx1 = C[k1] - X0, dx2 = C[k2] - X0;
            const double dy1 = C[n1 + k1] - Y0, dy2 = C[n1 + k2] - Y0;
            const double area2 = dy2 * dx1 - dy1 * dx2;
            if (area2 > 0) {
                kd = 0;
                for (int i = 0; i < 3; i++) {
                    c[2 * i] = (dy2 * dxv[i] - dx2 * dyv[i]) / area2;
                    c[2 * i + 1] = (dx1 * dyv[i] - dy1 * dxv[i]) / area2;
                }
            }
        } else if (nbk == 2) {
            int slot = -1;
            for (int i = 0; i < 3 && slot < 0; i++)
                if (h->h_surr[i * n1 + k] != k) slot = i;
            if (slot >= 0) {
                const int k1 = h->h_surr[slot * n1 + k];
                const double dx1 = C[k1] - x, dy1 = C[n1 + k1] - y;
                const double area2 = dx1 * dx1 + dy1 * dy1;
                kd = (uint8_t)(1 | (slot << 2));
                for (int i = 0; i < 3; i++) c[2 * i] = (dx1 * dxv[i] + dy1 * dyv[i]) / area2;
            }
        }
        kind[k] = kd;
        for (int j = 0; j < 6; j++) gc[j * n1 + k] = (float)c[j];
    }
    const DevMixed &X = h->X;
    cudaError_t e = cudaSuccess;
    auto put = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    put(X.nx, nx.data(), n3 * 4);
    put(X.ny, ny.data(), n3 * 4);
    put(X.len, len.data(), n3 * 4);
    put(X.inv_area, inv_area.data(), n1 * 4);
    put(X.radius, radius.data(), n1 * 4);
    put(X.gc, gc.data(), 6 * n1 * 4);
    put(X.dzn, dzn.data(), n3 * 4);
    put(X.dzv, dzv.data(), n3 * 4);
    put(X.zgrad, zgrad.data(), 2 * n1 * 4);
    put(X.fric, fric.data(), n1 * 4);
    put(X.zmoff, zmoff.data(), n1 * 4);
    put(X.kind, kind.data(), n1);
    return e == cudaSuccess ? SWGPU_OK : SWGPU_ECUDA;
}

}  // namespace swgpu
