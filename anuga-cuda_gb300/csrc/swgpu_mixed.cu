// swgpu_mixed.cu -- mixed-precision evolve kernels.
//
// The same ANUGA algorithm as the FP64 path (gradient limiter on the
// auxiliary triangle, balance_deep_and_shallow, central-upwind flux,
// gravity_wb, semi-implicit Manning friction, protect), restructured for a
// GB300, whose FP64 pipe runs at 1/64 of the FP32 rate:
//
//  * The conserved state is FP64 depth h and FP64 momentum.  The update adds
//    FP32 increments (dt*E and the friction term) to it with FP64 adds, so
//    the state itself never loses precision to FP32.
//  * Everything the limiter, extrapolation and flux read is FP32 and stored
//    in deviation form: centroid stage and depth; per-vertex STAGE JUMPS from
//    the centroid; bed offsets of vertices and edges from the centroid bed;
//    geometry as normals, lengths, 1/area, radii and per-triangle jump
//    coefficients computed in FP64 on the host.  No FP32 expression adds or
//    subtracts absolute coordinates or two large depths.
//  * Hydrostatic pressure enters as a difference: the edge flux minus the
//    owner's edge pressure (gravity_wb's side term, folded into the flux),
//    0.5 g (h_r - h_l)(h_r + h_l) with h_r - h_l taken from the stage jump.
//    The stage gradient of the gravity term is the Green sum of the edge
//    stage jumps.  In deep water both would otherwise be differences of
//    O(g h^2) numbers, which is where FP32 loses the answer.
//  * The mass flux is computed with unfused, correctly rounded products so
//    that it is exactly antisymmetric: both triangles of an edge build the
//    same edge depths from the same data, and water volume is conserved to
//    the FP64 rounding of the reduction.
//  * FP32 <-> FP64 conversions of the state run on the integer pipe.
//
// Bytes per triangle-step (own arrays; neighbour gathers hit L1/L2):
//   distribute ~114, flux ~128, update ~104.
#include <algorithm>
#include <cstring>
#include <cmath>
#include <vector>

#include "swgpu_device.cuh"
#include "swgpu_handle.cuh"

namespace swgpu {

// Read-only loads through the non-coherent path (no kernel writes an array
// it reads this way).
template <typename T>
__device__ __forceinline__ T ro(const T *p) {
    return __ldg(p);
}

// Exact FP32 -> FP64 widening on the integer pipe (inputs are flushed to
// zero when denormal, as this unit compiles with -ftz).
__device__ __forceinline__ double widen(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned long long mant = (unsigned long long)(u & 0x7fffffu) << 29;
    const unsigned long long ex =
        e == 0 ? 0ull : (e == 0xffu ? 0x7ffull : (unsigned long long)(e + 896u));
    const unsigned long long bits = e == 0 ? sign : (sign | (ex << 52) | mant);
    return __longlong_as_double((long long)bits);
}

// FP64 -> FP32 narrowing, round to nearest even, on the integer pipe
// (results below the FP32 normal range flush to zero, overflow gives
// infinity, NaN stays NaN).
__device__ __forceinline__ float narrow(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const unsigned ed = (unsigned)((b >> 52) & 0x7ffu);
    const int e = (int)ed - 896;
    const unsigned long long frac = b & 0xfffffffffffffull;
    unsigned r;
    if (ed == 0x7ffu) {
        r = sign | 0x7f800000u | (frac ? 0x400000u : 0u);
    } else if (e <= 0) {
        r = sign;
    } else if (e >= 255) {
        r = sign | 0x7f800000u;
    } else {
        const unsigned m = (unsigned)(frac >> 29);
        const unsigned long long rest = frac & 0x1fffffffull;  // the 29 dropped bits
        r = ((unsigned)e << 23) | m;
        // round half to even; a carry out of the mantissa bumps the exponent
        // (up to infinity) as it should
        if (rest > 0x10000000ull || (rest == 0x10000000ull && (m & 1u))) r += 1u;
        r |= sign;
    }
    return __uint_as_float(r);
}

// x as an FP32 pair on the integer pipe: hi = x rounded to nearest (as
// narrow), lo = the exact remainder x - hi rounded to nearest.  lo is zero
// where x lies outside FP32's normal range or the remainder falls below it.
__device__ __forceinline__ void split_double(double x, float &hi, float &lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const unsigned ed = (unsigned)((b >> 52) & 0x7ffu);
    const int e = (int)ed - 896;
    if (ed == 0x7ffu || e <= 0 || e >= 255) {
        hi = narrow(x);
        lo = 0.0f;
        return;
    }
    const unsigned long long frac = b & 0xfffffffffffffull;
    const unsigned m = (unsigned)(frac >> 29);
    int rest = (int)(frac & 0x1fffffffull);  // the 29 dropped bits
    unsigned r = ((unsigned)e << 23) | m;
    if (rest > 0x10000000 || (rest == 0x10000000 && (m & 1u))) {
        r += 1u;  // rounded up: the remainder is negative
        rest -= 0x20000000;
    }
    hi = __uint_as_float(r | sign);
    // remainder = rest * 2^(ed - 1075): one rounding (int -> float), then an
    // exact scaling by a power of two (flushed to zero below FP32's range)
    const int se = (int)ed - 1075 + 127;
    const float scale = se > 0 ? __uint_as_float((unsigned)se << 23) : 0.0f;
    lo = __uint_as_float(__float_as_uint(__fmul_rn(__int2float_rn(rest), scale)) ^ sign);
}

// (ah + al) + (bh + bl) as an FP32 pair hi + lo (TwoSum of the high parts,
// the low parts added to its error, TwoSum again): about 46 bits.
__device__ __forceinline__ void add_pairs(float ah, float al, float bh, float bl, float &hi,
                                          float &lo) {
    const float s = __fadd_rn(ah, bh);
    const float bs = __fsub_rn(s, ah);
    const float es = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bs)), __fsub_rn(bh, bs));
    const float t = __fadd_rn(es, __fadd_rn(al, bl));
    hi = __fadd_rn(s, t);
    const float bt = __fsub_rn(hi, s);
    lo = __fadd_rn(__fsub_rn(s, __fsub_rn(hi, bt)), __fsub_rn(t, bt));
}

// h <= 0 for an h that is not NaN, on the integer pipe (-0 included).
__device__ __forceinline__ bool not_positive(double h) { return __double_as_longlong(h) <= 0; }

// Edge depth of edge i of a triangle from its centroid depth, the stage
// jumps of the two vertices of the edge and the bed offset of the edge.
// Both triangles of an edge evaluate it with the same operations.
__device__ __forceinline__ float edge_depth(float hc, float dwa, float dwb, float dze) {
    return (hc + 0.5f * (dwa + dwb)) - dze;
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
            u = __fmul_rn(uh, f);
            uh = __fmul_rn(u, h);
            vh = __fmul_rn(__fmul_rn(vh, f), h);
        }
    } else {
        u = __fdividef(uh, h);
    }
}

// Central-upwind flux (shallow_water_ext.c:302-441) of one edge seen from
// its owner, with the owner's hydrostatic edge pressure 0.5 g hl^2 removed
// from the normal momentum flux (that term is gravity_wb's side term,
// shallow_water_ext.c:1990-2028).  jump = w_r - w_l.  Returns the xy fluxes.
__device__ __forceinline__ void edge_flux_dev(float hl_in, float uhl_in, float vhl_in, float hr_in,
                                              float uhr_in, float vhr_in, float jump, float n1,
                                              float n2, const DevParams &P, float &f0, float &f1,
                                              float &f2, float &ms) {
    const float g = P.f_g, eps = P.f_eps;
    // rotation into the edge frame with unfused products, so that the two
    // triangles of an edge get exactly negated normal momenta
    const float al = __fadd_rn(__fmul_rn(n1, uhl_in), __fmul_rn(n2, vhl_in));
    const float bl = __fsub_rn(__fmul_rn(n1, vhl_in), __fmul_rn(n2, uhl_in));
    const float ar = __fadd_rn(__fmul_rn(n1, uhr_in), __fmul_rn(n2, vhr_in));
    const float br = __fsub_rn(__fmul_rn(n1, vhr_in), __fmul_rn(n2, uhr_in));
    float hl = hl_in, uhl = al, vhl = bl, ul;
    float hr = hr_in, uhr = ar, vhr = br, ur;
    side_speed_f(hl, uhl, vhl, ul, eps, P.f_h0, P.f_lim);
    side_speed_f(hr, uhr, vhr, ur, eps, P.f_h0, P.f_lim);
    const float cl = sqrtf(g * hl), cr = sqrtf(g * hr);
    float smax = omaxf(ul + cl, ur + cr);
    if (smax < 0.0f) smax = 0.0f;
    float smin = ominf(ul - cl, ur - cr);
    if (smin > 0.0f) smin = 0.0f;
    const float denom = smax - smin;
    if (denom < eps) {
        f0 = 0.0f;
        const float p = -0.5f * g * hl * hl;  // only the side term remains
        f1 = n1 * p;
        f2 = n2 * p;
        ms = 0.0f;
        return;
    }
    const float inv = __fdividef(1.0f, denom);
    const float ss = __fmul_rn(smax, smin);
    // mass: unfused products, exactly antisymmetric under swapping sides
    const float fl0 = __fmul_rn(ul, hl), fr0 = __fmul_rn(ur, hr);
    f0 = __fmul_rn(__fadd_rn(__fsub_rn(__fmul_rn(smax, fl0), __fmul_rn(smin, fr0)),
                             __fmul_rn(ss, jump)),
                   inv);
    // depth difference across the edge: the stage jump unless a side was
    // zeroed by the eps limit
    const float dH = (hl == hl_in && hr == hr_in) ? jump : hr - hl;
    const float dP = 0.5f * g * dH * (hr + hl);  // p_r - p_l
    const float e1 = (smax * ul * uhl - smin * ur * uhr + ss * (ar - al) - smin * dP) * inv;
    const float e2 = (smax * ul * vhl - smin * ur * vhr + ss * (br - bl)) * inv;
    ms = omaxf(fabsf(smax), fabsf(smin));
    f1 = n1 * e1 - n2 * e2;
    f2 = n2 * e1 + n1 * e2;
}

// ---- one-dimensional TMA (cp.async.bulk) staging of a block's tile ------

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// Raises the bytes the current phase waits for, without arriving.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// Arrives without adding bytes.
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    unsigned long long state;
    asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];"
                 : "=l"(state)
                 : "r"(smem_u32(bar))
                 : "memory");
    (void)state;
}
// Global -> shared bulk copy completing on the mbarrier.  dst, src 16-byte
// aligned, bytes a multiple of 16 (planes are padded to 64 elements and
// tiles start at multiples of 128 elements).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes,
                                          unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
    return ok != 0;
}
// Bounded wait for phase 0: every thread gives up after kWaitLimit polls
// (each poll may suspend in hardware), reports SWGPU_ETIMEOUT, and polls once
// more as long again so that copies still in flight land before the block
// leaves.  Returns true when the data arrived; on false the caller skips
// every later use of the tile.  Should the second wait run out as well, the
// block leaves with copies possibly still in flight into shared memory that
// a later block may be given: the host then marks the handle unusable on
// reading the status (every later call fails; only destroy remains).
constexpr int kWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, Ctrl *ctrl,
                                                  unsigned parity = 0) {
    for (int it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    set_status(ctrl, SWGPU_ETIMEOUT);
    for (int it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) break;
    return false;
}
// Programmatic dependent launch: let the next kernel of the stream start
// its blocks as this one's finish, and wait (in the next kernel) until the
// previous kernel has completed and its writes are visible.  Both are no-ops
// for kernels launched without the programmatic attribute.
__device__ __forceinline__ void pdl_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Orders this thread's earlier generic-proxy accesses to shared memory
// before later async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The flux kernel's own data for one tile of TILE triangles (= threads per
// block: 64, 128 or 256), filled by 12 bulk copies (7 static, 5 of state)
// that together move 29 four-byte values per triangle.
template <int TILE>
struct __align__(128) FluxTile {
    float2 ws[TILE];  // stage pair
    float hf[TILE];
    float2 rad[TILE];  // radius, 1/area
    float4 es[3][TILE];  // edge state (depth, stage jump, momenta) per edge
    float2 nrm[3][TILE];  // unit normals
    int2 lnb[3][TILE];  // edge length (float bits), packed neighbour (read where used)
};

// The bulk copies of a flux tile starting at triangle k0 (span elements of
// each padded plane), completing on bar, in two halves: the static geometry
// (issued before the previous kernel has finished) and the state.
template <int TILE>
__device__ __forceinline__ void flux_tile_issue_static(const DevMixed &X, FluxTile<TILE> &T,
                                                       int k0, int span,
                                                       unsigned long long *bar) {
    const int SP = X.S;
    const unsigned bytes = (unsigned)span * 4u;
    mbar_expect_tx(bar, 14u * bytes);  // 14 four-byte static values per triangle
    bulk_load(T.rad, X.rad + k0, 2u * bytes, bar);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        bulk_load(T.nrm[i], X.nrm + i * SP + k0, 2u * bytes, bar);
        bulk_load(T.lnb[i], X.lnb + i * SP + k0, 2u * bytes, bar);
    }
}
template <int TILE>
__device__ __forceinline__ void flux_tile_issue_dynamic(const DevMixed &X, FluxTile<TILE> &T,
                                                        int k0, int span,
                                                        unsigned long long *bar) {
    const int SP = X.S;
    const unsigned bytes = (unsigned)span * 4u;
    mbar_arrive_expect_tx(bar, 15u * bytes);  // 15 dynamic values; the tile's one arrival
    bulk_load(T.ws, X.ws + k0, 2u * bytes, bar);
    bulk_load(T.hf, X.hf + k0, bytes, bar);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        bulk_load(T.es[i], X.es + i * SP + k0, 4u * bytes, bar);
    }
}
// All 12 bulk copies of a flux tile starting at triangle k0 (span elements
// of each padded plane), completing on bar.  Called by one thread.
template <int TILE>
__device__ __forceinline__ void flux_tile_issue(const DevMixed &X, FluxTile<TILE> &T, int k0,
                                                int span, unsigned long long *bar) {
    flux_tile_issue_static<TILE>(X, T, k0, span, bar);
    flux_tile_issue_dynamic<TILE>(X, T, k0, span, bar);
}

// Fluxes + gravity_wb of triangle k0 + tid of a staged tile (cnt valid
// triangles); stores the explicit updates and returns the triangle's CFL
// timestep bound.
template <int TILE>
__device__ __forceinline__ float flux_tile_triangle(const DevMixed &X, const DevParams &P,
                                                    const FluxTile<TILE> &T, int k0, int cnt) {
    const int SP = X.S;
    const int tid = threadIdx.x;
    const int k = k0 + tid;
    float t = P.f_max_dt;
    const float eps = P.f_eps;
    const float2 wsk = T.ws[tid];
    const float wk = wsk.x, lk = wsk.y;
    const float rk = T.rad[tid].x;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;  // flux sums
    float gx = 0.f, gy = 0.f;            // Green sum of edge stage jumps
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float2 nr = T.nrm[i][tid];
        const int2 lq = T.lnb[i][tid];
        const float n1 = nr.x, n2 = nr.y, L = __int_as_float(lq.x);
        const float4 el = T.es[i][tid];
        const float hl = el.x, dwl = el.y, uhl = el.z, vhl = el.w;
        float hr, uhr, vhr, jump;
        const int pki = lq.y;
        if (pki >= 0) {
            // the neighbour's stored edge state: the very numbers it uses
            // itself, so both sides see the same two states
            const int n = pki >> 2, m = pki & 3;
            const int ln = n - k0;
            float wn, lnn, dwn;
            float4 en;
            float2 wsn;
            if ((unsigned)ln < (unsigned)cnt) {
                en = T.es[m][ln];
                wsn = T.ws[ln];
            } else {
                en = ro(X.es + m * SP + n);
                wsn = ro(X.ws + n);
            }
            wn = wsn.x;
            lnn = wsn.y;
            hr = en.x;
            dwn = en.y;
            uhr = en.z;
            vhr = en.w;
            jump = ((wn - wk) + (lnn - lk)) + (dwn - dwl);
        } else {
            const int mb = -pki - 1;
            hr = ro(X.hbf + mb);
            jump = ro(X.wjb + mb);
            uhr = ro(X.uhbf + mb);
            vhr = ro(X.vhbf + mb);
        }
        gx += dwl * L * n1;
        gy += dwl * L * n2;
        if (P.optimise_dry_cells && fabsf(hl) < eps && fabsf(hr) < eps) continue;
        float f0, f1, f2, ms;
        edge_flux_dev(hl, uhl, vhl, hr, uhr, vhr, jump, n1, n2, P, f0, f1, f2, ms);
        a0 -= f0 * L;
        a1 -= f1 * L;
        a2 -= f2 * L;
        // ANUGA lowers the timestep by radii[k]/ms and radii[n]/ms at each
        // edge (shallow_water_ext.c:4653-4664).  The neighbour n evaluates
        // the same edge with the same two states and gets the same ms (the
        // flux is exactly antisymmetric), so it contributes radii[n]/ms
        // itself: over the mesh, each triangle's own radius gives the same
        // minimum without the neighbour's radius being read.
        if (ms > eps) t = ominf(t, __fdividef(rk, ms));
    }
    const float ghc = P.f_g * T.hf[tid];
    const float inv_area = T.rad[tid].y;
    X.ewu[k] = make_float2(a0 * inv_area, (a1 - ghc * gx) * inv_area);
    X.evh[k] = (a2 - ghc * gy) * inv_area;
    return t;
}

// Fluxes + gravity_wb, FP32, triangle centric (no atomics).  Each block
// stages its tile of TILE triangles with one-dimensional TMA bulk copies into
// shared memory; neighbours inside the tile (most of them, in Morton order)
// are read from shared memory, the others from global memory.
template <int TILE>
__global__ void __launch_bounds__(TILE, 1536 / TILE) flux_mixed(DevMesh M, DevMixed X, DevParams P,
                                                        Ctrl *ctrl, int flags) {
    pdl_launch_dependents();
    ctrl = block_ctrl(ctrl, M);
    __shared__ FluxTile<TILE> T;
    __shared__ __align__(8) unsigned long long bar;
    const int N = M.N;
    const int tid = threadIdx.x;
    const int k0 = blockIdx.x * TILE;
    const int cnt = min(TILE, N - k0);
    const int span = min(TILE, X.S - k0);  // tile length in the padded planes (x64)
    // A scenario that has stopped stays stopped for the rest of the run (only
    // the host clears the flag, between runs), so a flag already raised
    // before the previous kernel has finished means a block with nothing to
    // do and nothing to fetch.  Thread 0 reads it for the whole block.
    __shared__ int stopped_early;
    if (tid == 0) {
        mbar_init(&bar, 1);
        stopped_early = (flags & kFused) ? ctrl_halted(ctrl) : 0;
        // geometry and neighbour indices do not change between steps:
        // fetched while the previous kernel may still run
        if (!stopped_early) flux_tile_issue_static<TILE>(X, T, k0, span, &bar);
    }
    __syncthreads();
    pdl_wait();
    if (stopped_early) return;  // no copy was issued
    // the flag as the previous kernels left it (no kernel of this step
    // changes it before this grid completes): the same for every thread
    const bool halted = (flags & kFused) && ctrl_halt_settled(ctrl);
    if (tid == 0) {
        if (halted)
            mbar_arrive(&bar);  // the static copies only
        else
            flux_tile_issue_dynamic<TILE>(X, T, k0, span, &bar);
    }
    // the running timestep minimum, read (by the thread that will reduce)
    // while the copies fly: the block's atomic is skipped when it cannot
    // lower it, without a read at the end
    __shared__ unsigned long long ft_seen;
    if (tid == 0) ft_seen = *(volatile unsigned long long *)&ctrl->ftmin_bits;
    const bool arrived = mbar_wait_bounded(&bar, ctrl);
    if (halted) return;
    float t = P.f_max_dt;
    if (arrived && tid < cnt) t = flux_tile_triangle<TILE>(X, P, T, k0, cnt);
    if (flags & kNoTimestep) return;  // later Runge-Kutta stage: the step's dt is set
    // the step's clock is evaluated from the minimum by step_clock_mixed once
    // this grid has completed: no block waits on a count of finished blocks
    block_min_timestep_f<TILE>(t, ctrl, &ft_seen);
}

// The same fluxes with persistent blocks: each block walks tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... and double-buffers them, the bulk
// copies of the next tile in flight while the current one is computed.
template <int TILE>
__global__ void __launch_bounds__(TILE) flux_mixed_pipelined(DevMesh M, DevMixed X, DevParams P,
                                                             Ctrl *ctrl_base, int flags,
                                                             int ntiles) {
    __shared__ FluxTile<TILE> T[2];
    __shared__ __align__(8) unsigned long long bar[2];
    const int N = M.N;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    __syncthreads();
    int tile = blockIdx.x, buf = 0;
    unsigned parity = 0u;  // bit b: phase parity of bar[b]
    if (tid == 0 && tile < ntiles)
        flux_tile_issue_static<TILE>(X, T[0], tile * TILE, min(TILE, X.S - tile * TILE), &bar[0]);
    pdl_wait();
    if (tid == 0 && tile < ntiles)
        flux_tile_issue_dynamic<TILE>(X, T[0], tile * TILE, min(TILE, X.S - tile * TILE), &bar[0]);
    if (tile + (int)gridDim.x >= ntiles) pdl_launch_dependents();
    // the block's timestep minimum is taken over all its tiles of one
    // scenario and reduced once (at the end, or when the scenario changes):
    // no per-tile barrier waits for the atomic
    Ctrl *acc_ctrl = nullptr;
    float tacc = P.f_max_dt;
    const bool take_dt = !(flags & kNoTimestep);
    while (tile < ntiles) {
        const int next = tile + gridDim.x;
        // the next kernel's blocks may start once every block is on its last tile
        if (next < ntiles && next + (int)gridDim.x >= ntiles) pdl_launch_dependents();
        if (tid == 0 && next < ntiles) {
            fence_proxy_async();  // the buffer's reads (previous tile) come first
            flux_tile_issue<TILE>(X, T[buf ^ 1], next * TILE, min(TILE, X.S - next * TILE),
                                  &bar[buf ^ 1]);
        }
        const int k0 = tile * TILE;
        const int cnt = min(TILE, N - k0);
        Ctrl *ctrl = M.blk_scen ? ctrl_base + M.blk_scen[k0 >> 8] : ctrl_base;
        const bool skip = (flags & kFused) && ctrl_halted(ctrl);
        if (take_dt && acc_ctrl && ctrl != acc_ctrl) {  // uniform over the block
            block_min_timestep_f<TILE>(tacc, acc_ctrl);
            tacc = P.f_max_dt;
        }
        acc_ctrl = ctrl;
        const bool arrived = mbar_wait_bounded(&bar[buf], ctrl, (parity >> buf) & 1u);
        parity ^= 1u << buf;
        if (!skip && arrived && tid < cnt)
            tacc = ominf(tacc, flux_tile_triangle<TILE>(X, P, T[buf], k0, cnt));
        __syncthreads();  // everyone is done with T[buf] before it is refilled
        tile = next;
        buf ^= 1;
    }
    if (take_dt && acc_ctrl) block_min_timestep_f<TILE>(tacc, acc_ctrl);
}

// FP32 copies of the updated state and protect (shallow_water_ext.c:
// 1638-1705) on depth; shared by the update and the stand-alone prepare.
// No FP64 arithmetic: the stage pair comes from depth and bed as FP32 pairs
// (zhi + zlo: the bed centroid).
__device__ __forceinline__ void finish_state(const DevParams &P, double &h, double &uh, double &vh,
                                             float zhi, float zlo, float &hf, float &wf,
                                             float &wlo, float &uvel, float &vvel,
                                             int &nonfinite) {
    float hl;
    split_double(h, hf, hl);
    float uhf = narrow(uh), vhf = narrow(vh);
    if (hf < P.f_mah) {  // false for NaN: h is a number below
        if (P.f_mas < P.f_eps) {
            uh = vh = 0.0;
            uhf = vhf = 0.0f;
            if (not_positive(h)) {
                h = 0.0;
                hf = hl = 0.0f;
            }
        } else if (not_positive(h)) {
            h = uh = vh = 0.0;
            hf = hl = uhf = vhf = 0.0f;
        } else {
            const float u = uhf / hf, v = vhf / hf, ms = P.f_mas;
            if (fabsf(u) > ms) uhf = (u > 0 ? ms : -ms) * hf;
            if (fabsf(v) > ms) vhf = (v > 0 ? ms : -ms) * hf;
            uh = widen(uhf);
            vh = widen(vhf);
        }
    }
    // stage as an unevaluated FP32 sum hi + lo (~46 bits): the limiter and
    // the flux take stage differences between neighbours from it
    add_pairs(hf, hl, zhi, zlo, wf, wlo);
    if (!(fabsf(hf) <= 3.0e38f) || !(fabsf(uhf) <= 3.0e38f) || !(fabsf(vhf) <= 3.0e38f))
        nonfinite = 1;
    const float inv = __fdividef(1.0f, omaxf(hf, P.f_mah));
    uvel = uhf * inv;
    vvel = vhf * inv;
}

// Update: h += dt*E_h;  q += q*(r - 1) + dt*E_q*r  with r = 1/(1 - dt*S) the
// semi-implicit Manning factor.  Increments in FP32, additions in FP64.
template <int BS>
__global__ void __launch_bounds__(BS, 2048 / BS) update_mixed(DevMesh M, DevState S, DevMixed X,
                                                       DevParams P, Ctrl *ctrl, int flags,
                                                       Stage stg) {
    pdl_launch_dependents();
    ctrl = block_ctrl(ctrl, M);
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = k < M.N;
    // static per-triangle data before the previous kernel has finished
    const float4 us = in ? ro(X.ust + k) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float eta = us.x, zmoff = us.y, zhi = us.z, zlo = us.w;
    pdl_wait();
    // a stopped scenario's threads load nothing more (the flag is settled:
    // only the step clock kernel and the distribute change it)
    if ((flags & kFused) && ctrl_halt_settled(ctrl)) return;
    // every load first, the control block's with them (this thread is the
    // only writer of element k)
    const StepClock clk = published_step_clock(ctrl);
    const int kk = in ? k : 0;
    const double h0 = ro(X.hd + kk), uh0 = ro(S.uh + kk), vh0 = ro(S.vh + kk);
    const bool combine = stg.kind == kStageMid || stg.kind == kStageLast;
    double bh = 0.0, bu = 0.0, bv = 0.0;
    if (combine) {
        bh = ro(S.bw + kk);
        bu = ro(S.buh + kk);
        bv = ro(S.bvh + kk);
    }
    const float hf0 = ro(X.hf + kk);  // FP32 copies of the pre-update state
    const float2 vel0 = ro(X.vel + kk);
    const float uv0 = vel0.x, vv0 = vel0.y;
    const float2 ewu = ro(X.ewu + kk);
    const float ew = ewu.x, euh = ewu.y, evh = ro(X.evh + kk);
    const float dtf = (float)clk.dt;
    int bad = 0, nonfinite = 0;
    if (in) {
        double h = h0, uh = uh0, vh = vh0;
        const float mah = P.f_mah;
        const float uf = uv0 * omaxf(hf0, mah);
        const float vf = vv0 * omaxf(hf0, mah);
        float rm1 = 0.0f, r = 1.0f;  // r - 1 and r
        if (eta > mah) {
            const float hm = hf0 - zmoff;
            if (hm >= mah) {
                const float Sf = -P.f_g * eta * eta * sqrtf(uf * uf + vf * vf) *
                                 exp2f(-(7.0f / 3.0f) * __log2f(hm));
                const float dS = dtf * Sf;  // <= 0
                const float den = 1.0f - dS;
                if (!(den > 0.0f)) bad = 1;
                r = __fdividef(1.0f, den);
                rm1 = dS * r;  // r - 1 without cancellation
            }
        }
        h += widen(dtf * ew);
        uh += widen(uf * rm1 + dtf * euh * r);
        vh += widen(vf * rm1 + dtf * evh * r);
        if (combine) {
            // saxpy_conserved_quantities in FP64 on depth: with a + b = 1 it
            // is the stage saxpy minus the (unchanged) bed
            h = stg.a * h + stg.b * bh;
            uh = stg.a * uh + stg.b * bu;
            vh = stg.a * vh + stg.b * bv;
        }
        float hf, wf, wl, uv, vv;
        finish_state(P, h, uh, vh, zhi, zlo, hf, wf, wl, uv, vv, nonfinite);
        if (stg.kind == kStageFirst) {  // backup_conserved_quantities (depth, momenta)
            S.bw[k] = h0;
            S.buh[k] = uh0;
            S.bvh[k] = vh0;
        }
        X.hd[k] = h;
        S.uh[k] = uh;
        S.vh[k] = vh;
        X.hf[k] = hf;
        X.ws[k] = make_float2(wf, wl);
        X.vel[k] = make_float2(uv, vv);
        if ((flags & kTrack) && (stg.kind == kStageEuler || stg.kind == kStageLast))
            track_depth(S, k, h, step_end_time(ctrl, clk, stg), P.track_threshold);
    }
    // the stage is committed by the distribute (its scenario's first block)
    if (bad) set_status(ctrl, SWGPU_EDENOMINATOR);
    if (nonfinite) set_status(ctrl, SWGPU_ENONFINITE);
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

// a / b from the approximate reciprocal and one Newton correction of the
// quotient (Markstein's method: q = a r, q += r (a - b q)), within about an
// ulp; for the |b| > 1e-30 of the limiter, under FTZ.
__device__ __forceinline__ float div_refined(float a, float b) {
    const float r = __fdividef(1.0f, b);
    const float q = a * r;
    return fmaf(fmaf(-b, q, a), r, q);
}

// limit_gradient (shallow_water_ext.c:151-181); refined divisions (the
// limiter is where FP32 error grows most: an approximate quotient here
// raised the 1000-step stage error by 14%, the refined one by 0.04%)
__device__ __forceinline__ void limit_f(float (&d)[3], float qmin, float qmax, float beta) {
    const float TINY = 1.0e-30f;
    float r = 1000.0f, r0 = 1.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (d[i] < -TINY) r0 = div_refined(qmin, d[i]);
        if (d[i] > TINY) r0 = div_refined(qmax, d[i]);
        r = ominf(r0, r);
    }
    const float phi = ominf(r * beta, 1.0f);
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] *= phi;
}

// jumps on the auxiliary triangle: d_i = c_i0*dq1 + c_i1*dq2, limited
template <typename C>
__device__ __forceinline__ void aux_jumps_f(float dq0, float dq1, float dq2, const C &c,
                                            float beta, float (&d)[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] = c(2 * i) * dq1 + c(2 * i + 1) * dq2;
    float qmin, qmax;
    qminmax_f(dq0, dq1, dq2, qmin, qmax);
    limit_f(d, qmin, qmax, beta);
}

template <typename C>
__device__ __forceinline__ void one_jumps_f(float dq1, const C &c, float beta,
                                            float (&d)[3]) {
#pragma unroll
    for (int i = 0; i < 3; i++) d[i] = c(2 * i) * dq1;
    const float qmin = dq1 >= 0.0f ? 0.0f : dq1, qmax = dq1 >= 0.0f ? dq1 : 0.0f;
    limit_f(d, qmin, qmax, beta);
}

// Boundary values (evaluate_segment, per boundary type) of triangle k's
// boundary edges from the edge values this thread has just stored.  Out of
// line: boundary triangles are rare, and the FP64 evaluation inlined would
// raise the register pressure of every thread of the distribute.  Returns 1
// when an edge's boundary could not be evaluated.
__device__ __noinline__ int boundary_edges_mixed(int k, int N, int SP, double time, double g,
                                                 const int *nbr, const int *btag,
                                                 const BcTag *tags, const double *ze_,
                                                 const float4 *es, const float2 *nrm,
                                                 double *wb_, double *uhb_,
                                                 double *vhb_, double *zb_, float *hbf,
                                                 float *wjb, float *uhbf, float *vhbf) {
    int bad = 0;
    for (int i = 0; i < 3; i++) {
        const int pk = ro(nbr + i * N + k);
        if (pk >= 0) continue;
        const int mb = -pk - 1;
        const float4 e = es[i * SP + k];  // this thread's own stores: a plain load
        const float hle = e.x;
        const double ze = ro(ze_ + i * N + k);
        const double we = ze + widen(hle);
        const BcTag &T = tags[ro(btag + mb)];
        double wb, uhb, vhb;
        if (!eval_boundary(T, time, we, widen(e.z), widen(e.w),
                           widen(ro(nrm + i * SP + k).x), widen(ro(nrm + i * SP + k).y), ze, g,
                           wb, uhb,
                           vhb)) {
            bad = 1;
            wb = we;
            uhb = vhb = 0.0;
        }
        wb_[mb] = wb;
        uhb_[mb] = uhb;
        vhb_[mb] = vhb;
        zb_[mb] = ze;
        if (boundary_keeps_edge_stage(T.type)) {
            // same depth and stage as the edge: exactly no jump
            hbf[mb] = hle;
            wjb[mb] = 0.0f;
        } else {
            hbf[mb] = (float)(wb - ze);
            wjb[mb] = (float)(wb - we);
        }
        uhbf[mb] = (float)uhb;
        vhbf[mb] = (float)vhb;
    }
    return bad;
}

// The distribute kernel's own data for one tile of BS triangles, filled by
// 16 bulk copies (20 four-byte values and one byte per triangle).
template <int BS>
struct __align__(128) DistTile {
    float2 ws[BS];   // stage pair
    float hf[BS];
    float2 vel[BS];  // velocities
    float2 gc[3][BS];  // per vertex: the coefficients of dq1 and dq2
    float dzv[3][BS];
    float dze[3][BS];
    int sur[3][BS];      // surrogate neighbours
    uint8_t kind[BS];    // DevMixed::kind
};

// Centroid value of neighbour n: from the tile when n is one of the block's
// triangles (most, in Morton order), else from global memory.
template <typename V>
__device__ __forceinline__ V tile_or_global(const V *tile, const V *plane, int n, int kb,
                                            int cnt) {
    const int ln = n - kb;
    return (unsigned)ln < (unsigned)cnt ? tile[ln] : ro(plane + n);
}

// Extrapolation + balance + boundary conditions, FP32, in stage jumps.  Each
// block stages its tile's own planes with one-dimensional TMA bulk copies
// into shared memory and reads in-tile neighbours from there.
//
// In the fused step the stage `stg` is committed here (commit_stage: time,
// counters, the stop decision, announce_halt) by the first block of each
// scenario, once the update grid has completed; every block takes the
// stage's order and end time from the step's clock (clk_*), which the commit
// does not write, so no block depends on when the commit runs.
template <int BS>
__global__ void __launch_bounds__(BS, 2048 / BS) distribute_mixed(DevMesh M, DevState S, DevMixed X,
                                                           DevParams P, const BcTag *tags,
                                                           Ctrl *ctrls, int flags, Stage stg) {
    const bool fused = flags & kFused;
    pdl_launch_dependents();
    Ctrl *ctrl = block_ctrl(ctrls, M);
    __shared__ DistTile<BS> T;
    __shared__ __align__(8) unsigned long long bar;
    const int N = M.N, SP = X.S;
    const int tid = threadIdx.x;
    const int kb = blockIdx.x * BS;
    const int cnt = min(BS, N - kb);
    const int span = min(BS, SP - kb);  // a multiple of 64 elements
    const int k = kb + tid;
    const unsigned bytes = (unsigned)span * 4u;
    // a scenario stopped before the previous kernel finished (halt == 1: its
    // last distribute has run) stays stopped for the rest of the run: its
    // blocks fetch nothing.  Thread 0 reads the flag for the whole block.
    __shared__ int stopped_early;
    if (tid == 0) {
        mbar_init(&bar, 1);
        stopped_early = fused && ctrl_halted(ctrl) == 1;
    }
    __syncthreads();
    // static planes (reconstruction coefficients, bed offsets) and index
    // planes before the previous kernel has finished
    if (tid == 0 && !stopped_early) {
        mbar_expect_tx(&bar, 15u * bytes + (unsigned)span);
#pragma unroll
        for (int i = 0; i < 3; i++) bulk_load(T.gc[i], X.gc + i * SP + kb, 2u * bytes, &bar);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            bulk_load(T.dzv[i], X.dzv + i * SP + kb, bytes, &bar);
            bulk_load(T.dze[i], X.dze + i * SP + kb, bytes, &bar);
            bulk_load(T.sur[i], X.surrp + i * SP + kb, bytes, &bar);
        }
        bulk_load(T.kind, X.kind + kb, (unsigned)span, &bar);  // span: a multiple of 64 bytes
    }
    pdl_wait();
    if (stopped_early) return;  // no copy was issued
    // halt == 1 only from a step clock kernel, which has completed: the same
    // for every thread (halt == 2: the scenario stops after this distribute)
    const bool halted = fused && ctrl_halt_settled(ctrl) == 1;
    if (tid == 0) {
        if (halted) {
            mbar_arrive(&bar);  // the static copies only
        } else {
            mbar_arrive_expect_tx(&bar, 5u * bytes);
            bulk_load(T.ws, X.ws + kb, 2u * bytes, &bar);
            bulk_load(T.hf, X.hf + kb, bytes, &bar);
            bulk_load(T.vel, X.vel + kb, 2u * bytes, &bar);
        }
    }
    int order;
    if (fused) {
        order = (int)ctrl->clk_order;
        // the first block of each scenario (thread 0 alone reads the map)
        if (tid == 0 && !halted &&
            (blockIdx.x == 0 ||
             (M.blk_scen && M.blk_scen[(kb - 1) >> 8] != M.blk_scen[kb >> 8]))) {
            commit_stage(ctrl, published_step_clock(ctrl), P, stg);
            announce_halt(ctrl);
        }
    } else {
        order = (int)ctrl->order;
    }
    const bool arrived = mbar_wait_bounded(&bar, ctrl);
    if (halted) return;
    int bad_bc = 0;
    if (arrived && tid < cnt) {
        const int kind = T.kind[tid];
        const float mah = P.f_mah;
        const float2 wsk = T.ws[tid], velk = T.vel[tid];
        const float wk = wsk.x, lk = wsk.y, hc = T.hf[tid];
        const float qu = velk.x, qv = velk.y;
        const bool vel = P.extrapolate_velocity_second_order == 1;
        const float hk = omaxf(hc, mah);
        const float uk = qu * hk, vk = qv * hk;  // centroid momentum
        float dw[3] = {0.f, 0.f, 0.f};  // vertex stage jumps
        float ou[3], ov[3];             // vertex momentum (or velocity)
        if (order != 1) {
            const float cu = vel ? qu : uk, cv = vel ? qv : vk;
            float du[3] = {0.f, 0.f, 0.f}, dv[3] = {0.f, 0.f, 0.f};
            bool keep = false;  // dry neighbourhood: previous vertex values stay
            if ((kind & 3) != 2) {
                // reconstruction coefficients, read from the tile at each use
                const auto c = [&](int j) {
                    const float2 g = T.gc[j >> 1][tid];
                    return (j & 1) ? g.y : g.x;
                };
                if ((kind & 3) == 0) {
                    const int k0 = T.sur[0][tid], k1 = T.sur[1][tid], k2 = T.sur[2][tid];
                    const float h0 = tile_or_global(T.hf, X.hf, k0, kb, cnt);
                    const float h1 = tile_or_global(T.hf, X.hf, k1, kb, cnt);
                    const float h2 = tile_or_global(T.hf, X.hf, k2, kb, cnt);
                    const float hmin = ominf(ominf(h0, ominf(h1, h2)), hc);
                    const float hmax = omaxf(h0, omaxf(h1, h2));
                    if (P.optimise_dry_cells && hmax < P.f_eps) {
                        keep = true;
                    } else {
                        float hfactor = 0.0f;
                        if (hmin > 0.001f) hfactor = (hmin - 0.001f) / (hmin + 0.004f);
                        const float2 s0 = tile_or_global(T.ws, X.ws, k0, kb, cnt);
                        const float2 s1 = tile_or_global(T.ws, X.ws, k1, kb, cnt);
                        const float2 s2 = tile_or_global(T.ws, X.ws, k2, kb, cnt);
                        const float w0 = s0.x, w1 = s1.x, w2 = s2.x;
                        const float l0 = s0.y, l1 = s1.y, l2 = s2.y;
                        aux_jumps_f((w0 - wk) + (l0 - lk), (w1 - w0) + (l1 - l0), (w2 - w0) + (l2 - l0), c,
                                    P.f_beta_w_dry + (P.f_beta_w - P.f_beta_w_dry) * hfactor, dw);
                        const float2 q0 = tile_or_global(T.vel, X.vel, k0, kb, cnt);
                        const float2 q1 = tile_or_global(T.vel, X.vel, k1, kb, cnt);
                        const float2 q2 = tile_or_global(T.vel, X.vel, k2, kb, cnt);
                        float u0 = q0.x, u1 = q1.x, u2 = q2.x;
                        float v0 = q0.y, v1 = q1.y, v2 = q2.y;
                        if (!vel) {
                            u0 *= omaxf(h0, mah);
                            v0 *= omaxf(h0, mah);
                            u1 *= omaxf(h1, mah);
                            v1 *= omaxf(h1, mah);
                            u2 *= omaxf(h2, mah);
                            v2 *= omaxf(h2, mah);
                        }
                        aux_jumps_f(u0 - cu, u1 - u0, u2 - u0, c,
                                    P.f_beta_uh_dry + (P.f_beta_uh - P.f_beta_uh_dry) * hfactor, du);
                        aux_jumps_f(v0 - cv, v1 - v0, v2 - v0, c,
                                    P.f_beta_vh_dry + (P.f_beta_vh - P.f_beta_vh_dry) * hfactor, dv);
                    }
                } else {
                    const int slot = (kind >> 2) & 3;
                    const int k1 = T.sur[slot][tid];
                    const float h1 = tile_or_global(T.hf, X.hf, k1, kb, cnt);
                    const float beta = P.f_beta_w;
                    const float2 s1 = tile_or_global(T.ws, X.ws, k1, kb, cnt);
                    one_jumps_f((s1.x - wk) + (s1.y - lk),
                                c, beta, dw);
                    const float2 q1 = tile_or_global(T.vel, X.vel, k1, kb, cnt);
                    float u1 = q1.x, v1 = q1.y;
                    if (!vel) {
                        u1 *= omaxf(h1, mah);
                        v1 *= omaxf(h1, mah);
                    }
                    one_jumps_f(u1 - cu, c, beta, du);
                    one_jumps_f(v1 - cv, c, beta, dv);
                }
            }
            if (keep) {
                // previous vertex values, from the stored edge values of the
                // (linear) reconstruction: v_i = e_a + e_b - e_i
                float e0[3], e1[3], e2[3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float4 e = X.es[i * SP + k];  // this thread's own, before it stores
                    e0[i] = e.y;
                    e1[i] = e.z;
                    e2[i] = e.w;
                }
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const int a = (i == 0) ? 1 : 0, b = (i == 2) ? 1 : 2;
                    dw[i] = (e0[a] + e0[b]) - e0[i];
                    ou[i] = (e1[a] + e1[b]) - e1[i];
                    ov[i] = (e2[a] + e2[b]) - e2[i];
                }
            } else {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    ou[i] = cu + du[i];
                    ov[i] = cv + dv[i];
                }
            }
            if (vel) {
                // velocity -> momentum with the vertex depth hc + dw - dzv
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float d = omaxf((hc + dw[i]) - T.dzv[i][tid], 0.0f);
                    ou[i] *= d;
                    ov[i] *= d;
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < 3; i++) {
                ou[i] = uk;
                ov[i] = vk;
            }
        }
        // balance_deep_and_shallow (shallow_water_ext.c:1462-1636) with vertex
        // depth h_i = hc + (dw_i - dzv_i); the blend keeps the form
        // dw_i <- alpha*(dw_i - dzv_i) + dzv_i
        {
            // the bed offsets at the vertices, read from the tile here rather
            // than held in registers through the reconstruction
            float dzv[3];
#pragma unroll
            for (int i = 0; i < 3; i++) dzv[i] = T.dzv[i][tid];
            float rel[3];  // h_i - hc
#pragma unroll
            for (int i = 0; i < 3; i++) rel[i] = dw[i] - dzv[i];
            const float hmin = hc + ominf(rel[0], ominf(rel[1], rel[2]));
            float alpha = 1.0f;
            if (P.tight_slope_limiters == 0) {
                float dz = 0.0f;
#pragma unroll
                for (int i = 0; i < 3; i++) dz = omaxf(dz, fabsf(dzv[i]));
                alpha = dz > 0.0f ? omaxf(ominf(P.f_alpha * hmin / dz, 1.0f), 0.0f) : 1.0f;
            } else if (hmin < P.f_H0) {
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float hd = -rel[i];
                    if (!(hd <= 0.0f)) alpha = ominf(alpha, (hc - P.f_H0) / hd);
                }
                alpha = fminf(fmaxf(alpha, 0.0f), 1.0f);
            }
            if (alpha < 1.0f) {
                const float uc = hc > 1.0e-6f ? uk / hc : 0.0f;
                const float vc = hc > 1.0e-6f ? vk / hc : 0.0f;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float r = alpha * rel[i];
                    dw[i] = r + dzv[i];
                    if (P.use_centroid_velocities == 1) {
                        ou[i] = uc * (hc + r);
                        ov[i] = vc * (hc + r);
                    } else {
                        ou[i] = (1.0f - alpha) * uk + alpha * ou[i];
                        ov[i] = (1.0f - alpha) * vk + alpha * ov[i];
                    }
                }
            }
        }
        // edge values (quantity.c:687-706 interpolation) stored for the flux:
        // depth, stage jump from the centroid, momentum
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const int a = (i == 0) ? 1 : 0, b = (i == 2) ? 1 : 2;
            X.es[i * SP + k] = make_float4(edge_depth(hc, dw[a], dw[b], T.dze[i][tid]),
                                           0.5f * (dw[a] + dw[b]), 0.5f * (ou[a] + ou[b]),
                                           0.5f * (ov[a] + ov[b]));
        }
        if ((flags & kWriteBoundary) && (kind & 16)) {  // a boundary edge
            // the control block and the boundary's time are looked up again
            // here rather than held in registers through the reconstruction
            // (neither changes during the kernel)
            const Ctrl *c = block_ctrl(ctrls, M);
            const double time =
                fused ? c->clk_t0 + c->clk_dt * (stg.kind == kStageMid ? stg.tfrac : 1.0)
                      : c->time;
            bad_bc = boundary_edges_mixed(k, N, SP, time, P.g, M.nbr, M.btag, tags, S.ze,
                                          X.es, X.nrm, S.wb, S.uhb, S.vhb,
                                          S.zb, X.hbf, X.wjb, X.uhbf, X.vhbf);
        }
    }
    if (bad_bc) set_status(block_ctrl(ctrls, M), SWGPU_EBOUNDARY);
}

// update_timestep (the step's clock) of each running scenario, evaluated
// once from the flux kernel's minimum after that grid has completed and
// published for the update kernel.  One thread per scenario.
__global__ void __launch_bounds__(128) step_clock_mixed(Ctrl *ctrl, int nscen, DevParams P) {
    pdl_launch_dependents();
    pdl_wait();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nscen) return;
    Ctrl *c = ctrl + s;
    const int halt = c->halt;
    if (halt == 2) c->halt = 1;  // the last step's distribute has run
    if (halt) return;
    publish_step_clock(c, P);
}

// Depth from the FP64 stage (after an upload) or from the mixed state, then
// protect and the FP32 centroid copies.
__global__ void __launch_bounds__(kBlock) prepare_mixed(DevMesh M, DevState S, DevMixed X,
                                                        DevParams P, int from_stage) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M.N) return;
    double h = from_stage ? S.w[k] - S.zc[k] : X.hd[k];
    double uh = S.uh[k], vh = S.vh[k];
    float hf, wf, wl, uv, vv;
    int nonfinite = 0;
    const float4 us = X.ust[k];
    finish_state(P, h, uh, vh, us.z, us.w, hf, wf, wl, uv, vv, nonfinite);
    X.hd[k] = h;
    S.uh[k] = uh;
    S.vh[k] = vh;
    X.hf[k] = hf;
    X.ws[k] = make_float2(wf, wl);
    X.vel[k] = make_float2(uv, vv);
}

// FP64 stage centroid / vertex values and momentum vertex values for
// downloads: w = h + z, vertex values from the stored edge values of the
// linear reconstruction (v_i = e_a + e_b - e_i).
__global__ void __launch_bounds__(kBlock) vertices_from_mixed(DevMesh M, DevState S, DevMixed X) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = M.N, SP = X.S;
    if (k >= N) return;
    const double w = X.hd[k] + S.zc[k];
    S.w[k] = w;
    float e0[3], e1[3], e2[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float4 e = X.es[i * SP + k];
        e0[i] = e.y;
        e1[i] = e.z;
        e2[i] = e.w;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int a = (i == 0) ? 1 : 0, b = (i == 2) ? 1 : 2;
        S.wv[i * N + k] = w + (double)((e0[a] + e0[b]) - e0[i]);
        S.uhv[i * N + k] = (double)((e1[a] + e1[b]) - e1[i]);
        S.vhv[i * N + k] = (double)((e2[a] + e2[b]) - e2[i]);
    }
}

// FP64 centroid stage w = h + z from the mixed state (downloads of the
// centroid values, update_other_quantities).
__global__ void __launch_bounds__(kBlock) stage_from_mixed(int N, const double *__restrict__ hd,
                                                           const double *__restrict__ zc,
                                                           double *__restrict__ w) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < N) w[k] = hd[k] + zc[k];
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

// Block sizes come from M.shape (the autotuner's choice; results do not
// depend on it).
// A launch of kernel k; with pdl, as a programmatic dependent of the stream's
// previous kernel (it may start during that kernel's last wave and waits for
// it with griddepcontrol.wait before reading what that kernel writes).
template <typename... KArgs, typename... Args>
static void launch_k(void (*k)(KArgs...), int grid, int block, cudaStream_t st, bool pdl,
                     Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k, args...);
}

void launch_distribute_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                             const DevParams &P, const BcTag *tags, Ctrl *ctrl, int flags,
                             const Stage &stage, cudaStream_t st) {
    const int bs = M.shape.distribute, g = (M.n_launch + bs - 1) / bs;
    const bool pdl = M.shape.pdl;
    if (bs == 128)
        launch_k(distribute_mixed<128>, g, 128, st, pdl, M, S, X, P, tags, ctrl, flags, stage);
    else if (bs == 512)
        launch_k(distribute_mixed<512>, g, 512, st, pdl, M, S, X, P, tags, ctrl, flags, stage);
    else
        launch_k(distribute_mixed<256>, g, 256, st, pdl, M, S, X, P, tags, ctrl, flags, stage);
}
void launch_flux_mixed(const DevMesh &M, const DevState &, const DevMixed &X, const DevParams &P,
                       Ctrl *ctrl, int flags, cudaStream_t st) {
    const int t = M.shape.flux, g = (M.n_launch + t - 1) / t;
    const bool pdl = M.shape.pdl;
    if (M.shape.pipelined && t <= 128) {
        // one wave of persistent blocks: as many as are resident per SM
        static int resident[2] = {0, 0};
        int &r = resident[t == 64 ? 0 : 1];
        if (r == 0) {
            if (t == 64)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, flux_mixed_pipelined<64>, 64, 0);
            else
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, flux_mixed_pipelined<128>, 128, 0);
            r = std::max(r, 1);
        }
        const int grid = std::min(g, r * std::max(M.shape.sms, 1));
        if (t == 64)
            launch_k(flux_mixed_pipelined<64>, grid, 64, st, pdl, M, X, P, ctrl, flags, g);
        else
            launch_k(flux_mixed_pipelined<128>, grid, 128, st, pdl, M, X, P, ctrl, flags, g);
        return;
    }
    if (t == 64)
        launch_k(flux_mixed<64>, g, 64, st, pdl, M, X, P, ctrl, flags);
    else if (t == 256)
        launch_k(flux_mixed<256>, g, 256, st, pdl, M, X, P, ctrl, flags);
    else
        launch_k(flux_mixed<128>, g, 128, st, pdl, M, X, P, ctrl, flags);
}
void launch_step_clock_mixed(const DevParams &P, Ctrl *ctrl, int nscen, bool pdl,
                             cudaStream_t st) {
    launch_k(step_clock_mixed, (nscen + 127) / 128, 128, st, pdl, ctrl, nscen, P);
}
void launch_update_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                         const DevParams &P, Ctrl *ctrl, int flags, const Stage &stage,
                         cudaStream_t st) {
    const int bs = M.shape.update, g = (M.n_launch + bs - 1) / bs;
    const bool pdl = M.shape.pdl;
    if (bs == 128)
        launch_k(update_mixed<128>, g, 128, st, pdl, M, S, X, P, ctrl, flags, stage);
    else if (bs == 512)
        launch_k(update_mixed<512>, g, 512, st, pdl, M, S, X, P, ctrl, flags, stage);
    else
        launch_k(update_mixed<256>, g, 256, st, pdl, M, S, X, P, ctrl, flags, stage);
}
void launch_prepare_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                          const DevParams &P, int from_stage, cudaStream_t st) {
    prepare_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, S, X, P, from_stage);
}
void launch_vertices_from_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                                cudaStream_t st) {
    vertices_from_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, S, X);
}
void launch_stage_from_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                             cudaStream_t st) {
    stage_from_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M.N, X.hd, S.zc, S.w);
}
void launch_mass_partials_mixed(const DevMesh &M, const DevState &S, const DevMixed &X,
                                cudaStream_t st) {
    mass_partials_mixed<<<grid_for(M.N), kBlock, 0, st>>>(M, S, X);
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
    const size_t n1 = N, n3 = 3 * (size_t)N, sp = h->X.S;
    std::vector<double> zc(n1), zv(n3), ze(n3), fr(n1);
    cudaStreamSynchronize(h->stream);
    if (cudaMemcpy(zc.data(), h->S.zc, n1 * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(zv.data(), h->S.zv, n3 * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ze.data(), h->S.ze, n3 * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(fr.data(), h->S.fric, n1 * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return SWGPU_ECUDA;
    // FP32 planes use the padded stride sp (see DevMixed::S)
    std::vector<float2> nrm(3 * sp), gc(3 * sp);
    std::vector<float2> rad(n1);
    std::vector<int2> lnb(3 * sp, make_int2(0, 0));
    std::vector<float> dzv(3 * sp), dze(3 * sp);
    std::vector<float4> ust(n1);
    std::vector<uint8_t> kind(n1);
    const std::vector<double> &V = h->h_vxy, &C = h->h_cxy;
    for (int k = 0; k < N; k++) {
        for (int i = 0; i < 3; i++) {
            nrm[i * sp + k] = make_float2((float)h->h_normals[(2 * i) * n1 + k],
                                          (float)h->h_normals[(2 * i + 1) * n1 + k]);
            const float L = (float)h->h_len[i * n1 + k];
            int lbits;
            std::memcpy(&lbits, &L, sizeof lbits);
            lnb[i * sp + k] = make_int2(lbits, h->h_nbr[i * n1 + k]);
            dzv[i * sp + k] = (float)(zv[i * n1 + k] - zc[k]);
            dze[i * sp + k] = (float)(ze[i * n1 + k] - zc[k]);
        }
        rad[k] = make_float2((float)h->h_radii[k], (float)(1.0 / h->h_areas[k]));
        {
            const float zhi = (float)zc[k];
            ust[k] = make_float4((float)fr[k],
                                 (float)((zv[k] + zv[n1 + k] + zv[2 * n1 + k]) / 3.0 - zc[k]), zhi,
                                 (float)(zc[k] - (double)zhi));
        }
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
        if (h->h_nb[k] > 0) kd |= 16;  // has a boundary edge
        kind[k] = kd;
        for (int i = 0; i < 3; i++) gc[i * sp + k] = make_float2((float)c[2 * i], (float)c[2 * i + 1]);
    }
    const DevMixed &X = h->X;
    cudaError_t e = cudaSuccess;
    auto put = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    put(X.nrm, nrm.data(), 3 * sp * 8);
    put(X.lnb, lnb.data(), 3 * sp * 8);
    put(X.rad, rad.data(), n1 * 8);
    put(X.gc, gc.data(), 3 * sp * 8);
    put(X.dzv, dzv.data(), 3 * sp * 4);
    put(X.dze, dze.data(), 3 * sp * 4);
    put(X.ust, ust.data(), n1 * 16);
    put(X.kind, kind.data(), n1);
    return e == cudaSuccess ? SWGPU_OK : SWGPU_ECUDA;
}

}  // namespace swgpu
