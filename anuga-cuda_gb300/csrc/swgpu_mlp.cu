// swgpu_mlp.cu -- BF16 tensor-core MLP surrogate of the solver's maximum
// depth and arrival time.
//
// Rows are (scenario s, triangle k) pairs.  Each row's 16 input features
// are assembled on the fly: the scenario's 9 parameters, the triangle's bed
// elevation, centroid x and y, its distance to the scenario's source
// (parameters 1 and 2), and 3 zeros; each is normalised by a per-feature
// affine map.  The network is 16 -> 128 -> 128 -> 2 with ReLU, weights and
// activations in BF16, every product accumulated in FP32 by
// mma.sync.m16n8k16 (one warp = 16 rows; a layer's FP32 accumulator
// fragments are re-packed in registers as the next layer's BF16 A
// fragments, so activations never leave the register file in inference).
// Training keeps FP32 master weights (Adam); a step is one fused
// forward/backward kernel over a random batch, an FP32 weight-gradient
// reduction over the batch and the Adam update.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdarg>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "swgpu_internal.cuh"

namespace {

constexpr int kF = 16;      // input features (13 used)
constexpr int kH = 128;     // hidden units per layer
constexpr int kOut = 2;     // outputs: max depth, arrival time (normalised)
constexpr int kParams = 9;  // scenario parameters
constexpr int kS1 = 24;     // smem row strides (elements) with padding against bank conflicts
constexpr int kS2 = 136;
constexpr int kWarps = 8;   // warps per block, 16 rows each
constexpr int kRowsPerBlock = 16 * kWarps;

// flat FP32 parameter vector: W1 [16][128] (in-major), b1, W2 [128][128],
// b2, W3 [128][2], b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kF * kH;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH * kOut;
constexpr int kNumParams = kOffB3 + kOut;

// BF16 weight images in the layouts the mma B fragments read
struct BfWeights {
    __nv_bfloat16 w1t[kH * kS1];  // [out][in]
    __nv_bfloat16 w2t[kH * kS2];  // [out][in]
    __nv_bfloat16 w2[kH * kS2];   // [in][out] (backward)
    __nv_bfloat16 w3t[8 * kS2];   // [out (2 used)][in]
    __nv_bfloat16 w3[kH * 8];     // [in][out] (backward, 2 used)
    float b1[kH], b2[kH], b3[8];
};

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ float2 unpack2(uint32_t u) {
    __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162 *>(&u);
    return __bfloat1622float2(v);
}
__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16 *p) {
    return *reinterpret_cast<const uint32_t *>(p);
}
// D += A(16x16, row) * B(16x8, col), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct FeatureTables {
    const float *scen;   // [S][9]
    const float *tri;    // [N][3]: x, y, z
    const float *mu;     // [16]
    const float *isd;    // [16]
    long long N;
};

__device__ __forceinline__ float raw_feature(int c, const float *th, float x, float y, float z) {
    if (c < kParams) return th[c];
    if (c == 9) return z;
    if (c == 10) return x;
    if (c == 11) return y;
    if (c == 12) {
        const float dx = x - th[1], dy = y - th[2];
        return sqrtf(dx * dx + dy * dy);
    }
    return 0.0f;
}

// The A fragment of one warp's 16 rows: row g and g+8 of the tile (rows
// r0 + g, r0 + g + 8), columns 2t, 2t+1, 2t+8, 2t+9 (g = lane/4, t = lane%4).
__device__ __forceinline__ void load_features(const FeatureTables &F, long long row_a,
                                              long long row_b, bool va, bool vb,
                                              uint32_t (&a)[4]) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    float v[2][4];
    const long long rows[2] = {row_a, row_b};
    const bool valid[2] = {va, vb};
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int cols[4] = {2 * t, 2 * t + 1, 2 * t + 8, 2 * t + 9};
        if (!valid[h]) {
#pragma unroll
            for (int j = 0; j < 4; j++) v[h][j] = 0.0f;
            continue;
        }
        const long long s = rows[h] / F.N, k = rows[h] - s * F.N;
        const float *th = F.scen + s * kParams;
        const float x = F.tri[3 * k], y = F.tri[3 * k + 1], z = F.tri[3 * k + 2];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = cols[j];
            v[h][j] = (raw_feature(c, th, x, y, z) - F.mu[c]) * F.isd[c];
        }
    }
    a[0] = pack2(v[0][0], v[0][1]);
    a[1] = pack2(v[1][0], v[1][1]);
    a[2] = pack2(v[0][2], v[0][3]);
    a[3] = pack2(v[1][2], v[1][3]);
}

// One hidden layer over a warp's 16 rows: acc[j] = bias + A x W^T for the
// 16 n-tiles of 8 units; then ReLU and re-pack as 8 A fragments (k-steps).
template <int KSTEPS, int STRIDE>
__device__ __forceinline__ void hidden_layer(const uint32_t (*a)[4], const __nv_bfloat16 *wt,
                                             const float *bias, uint32_t (&out)[8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int jj = 0; jj < 8; jj++) {  // pairs of n-tiles -> one k-step of the next layer
        float acc[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int j = 2 * jj + h;
            const float bl = bias[8 * j + 2 * t], bh = bias[8 * j + 2 * t + 1];
            acc[h][0] = bl;
            acc[h][1] = bh;
            acc[h][2] = bl;
            acc[h][3] = bh;
            const __nv_bfloat16 *col = wt + (8 * j + g) * STRIDE;
#pragma unroll
            for (int kk = 0; kk < KSTEPS; kk++)
                mma16816(acc[h], a[kk], lds32(col + 16 * kk + 2 * t),
                         lds32(col + 16 * kk + 8 + 2 * t));
        }
        out[jj][0] = pack2(fmaxf(acc[0][0], 0.f), fmaxf(acc[0][1], 0.f));
        out[jj][1] = pack2(fmaxf(acc[0][2], 0.f), fmaxf(acc[0][3], 0.f));
        out[jj][2] = pack2(fmaxf(acc[1][0], 0.f), fmaxf(acc[1][1], 0.f));
        out[jj][3] = pack2(fmaxf(acc[1][2], 0.f), fmaxf(acc[1][3], 0.f));
    }
}

// Output layer: the one n-tile whose columns 0 and 1 are the outputs.
__device__ __forceinline__ void output_layer(const uint32_t (&a)[8][4], const BfWeights &W,
                                             float (&y)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    y[0] = y[2] = W.b3[2 * t];
    y[1] = y[3] = W.b3[2 * t + 1];
    const __nv_bfloat16 *col = W.w3t + g * kS2;
#pragma unroll
    for (int kk = 0; kk < 8; kk++)
        mma16816(y, a[kk], lds32(col + 16 * kk + 2 * t), lds32(col + 16 * kk + 8 + 2 * t));
}

__device__ void load_weights(BfWeights &dst, const BfWeights *src) {
    const int n = (int)(sizeof(BfWeights) / 16);
    const int4 *s = reinterpret_cast<const int4 *>(src);
    int4 *d = reinterpret_cast<int4 *>(&dst);
    for (int i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    __syncthreads();
}

// ---- inference -----------------------------------------------------------
__global__ void __launch_bounds__(32 * kWarps) mlp_predict(FeatureTables F, const BfWeights *gw,
                                                           long long row0, long long nrows,
                                                           float *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem[];
    BfWeights &W = *reinterpret_cast<BfWeights *>(smem);
    load_weights(W, gw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (long long base = (long long)blockIdx.x * kRowsPerBlock; base < nrows;
         base += (long long)gridDim.x * kRowsPerBlock) {
        const long long ra = base + 16 * warp + g, rb = ra + 8;
        uint32_t x[1][4];
        load_features(F, row0 + ra, row0 + rb, ra < nrows, rb < nrows, x[0]);
        uint32_t a1[8][4], a2[8][4];
        hidden_layer<1, kS1>(x, W.w1t, W.b1, a1);
        hidden_layer<8, kS2>(a1, W.w2t, W.b2, a2);
        float y[4];
        output_layer(a2, W, y);
        if (t == 0) {
            if (ra < nrows) {
                out[2 * ra] = y[0];
                out[2 * ra + 1] = y[1];
            }
            if (rb < nrows) {
                out[2 * rb] = y[2];
                out[2 * rb + 1] = y[3];
            }
        }
    }
}

// ---- inference on the 5th-generation tensor cores (tcgen05, TMEM) --------
//
// A CTA of 4 warps takes tiles of 128 rows.  Layer 1 (K = 16) and layer 2
// (K = 128) are each one 128 x 128 tcgen05.mma chain issued by one thread:
// A (activations) and B (weights, N x K) in shared memory in the canonical
// K-major layout without swizzle (8-row x 16-byte core matrices, adjacent
// along K 128 bytes apart, along M/N (K/8)*128 bytes apart), the FP32
// accumulators in tensor memory (256 columns: layer 1 in 0..127, layer 2 in
// 128..255).  Completion is signalled through tcgen05.commit on an
// mbarrier; warp w then reads TMEM lanes 32w..32w+31 (its rows) with
// tcgen05.ld, applies bias and ReLU, and writes the next layer's A tile, or
// for layer 2 evaluates the 128 -> 2 output layer on the CUDA cores.

constexpr int kTcRows = 128;

struct __align__(1024) TcSmem {
    __nv_bfloat16 a1[kTcRows * kF];   // layer-1 A: 128 x 16
    __nv_bfloat16 b1[kH * kF];        // W1 as N x K: 128 x 16
    __nv_bfloat16 a2[kTcRows * kH];   // layer-2 A: 128 x 128
    __nv_bfloat16 b2[kH * kH];        // W2 as N x K: 128 x 128
    float w3[kH * 2], bias1[kH], bias2[kH], bias3[2];
    unsigned long long bar;
    unsigned tmem_base;
};

// Byte offset of element (r, k) of an R x K K-major tile in the canonical
// no-swizzle layout.
__host__ __device__ __forceinline__ unsigned canon_offset(int r, int k, int K) {
    return (unsigned)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ unsigned long long smem_desc(const void *p, unsigned lbo,
                                                        unsigned sbo) {
    const unsigned addr = (unsigned)__cvta_generic_to_shared(p);
    return (unsigned long long)((addr >> 4) & 0x3FFFu) |
           ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both
// K-major, N = 128, M = 128.
constexpr unsigned kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) |
                              ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(unsigned d_tmem, unsigned long long a,
                                       unsigned long long b, bool accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(kTcIdesc), "r"((unsigned)accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            (unsigned)__cvta_generic_to_shared(bar))
        : "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void proxy_fence() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld32(unsigned taddr, float (&v)[32]) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init_tc(unsigned long long *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                     (unsigned)__cvta_generic_to_shared(bar))
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"((unsigned)__cvta_generic_to_shared(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
constexpr int kTcWaitLimit = 1 << 22;
// bounded wait for the MMA chain; false after kTcWaitLimit polls
__device__ __forceinline__ bool tc_wait(unsigned long long *bar, unsigned parity) {
    for (int i = 0; i < kTcWaitLimit; i++)
        if (mbar_test(bar, parity)) return true;
    return false;
}

__global__ void __launch_bounds__(128, 1) mlp_predict_tc(FeatureTables F, const float *params,
                                                         long long row0, long long nrows,
                                                         float *__restrict__ out,
                                                         int *__restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned view of the dynamic shared memory
    TcSmem &T = *reinterpret_cast<TcSmem *>(
        smem_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(smem_raw) & 1023u)) & 1023u));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // weights into the canonical layouts (BF16) and FP32 biases
    for (int e = tid; e < kH * kF; e += 128) {
        const int n = e / kF, k = e % kF;  // W1 [in k][out n]
        *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<unsigned char *>(T.b1) +
                                           canon_offset(n, k, kF)) =
            __float2bfloat16(params[kOffW1 + k * kH + n]);
    }
    for (int e = tid; e < kH * kH; e += 128) {
        const int n = e / kH, k = e % kH;  // W2 [in k][out n]
        *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<unsigned char *>(T.b2) +
                                           canon_offset(n, k, kH)) =
            __float2bfloat16(params[kOffW2 + k * kH + n]);
    }
    for (int e = tid; e < kH * 2; e += 128)  // W3 rounded like the other weights
        T.w3[e] = __bfloat162float(__float2bfloat16(params[kOffW3 + e]));
    for (int e = tid; e < kH; e += 128) {
        T.bias1[e] = params[kOffB1 + e];
        T.bias2[e] = params[kOffB2 + e];
    }
    if (tid < 2) T.bias3[tid] = params[kOffB3 + tid];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
                         (unsigned)__cvta_generic_to_shared(&T.tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) mbar_init_tc(&T.bar);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = T.tmem_base;
    const unsigned d1 = tmem, d2 = tmem + 128u;              // column offsets
    const unsigned lane_base = (unsigned)(32 * warp) << 16;  // this warp's TMEM lanes
    unsigned parity = 0u;
    bool ok = true;
    for (long long base = (long long)blockIdx.x * kTcRows; base < nrows && ok;
         base += (long long)gridDim.x * kTcRows) {
        const long long r = base + tid;  // this thread's row
        const bool valid = r < nrows;
        // ---- layer-1 A: the row's 16 normalised features
        {
            float v[kF];
            if (valid) {
                const long long q = row0 + r;
                const long long sidx = q / F.N, k = q - sidx * F.N;
                const float *th = F.scen + sidx * kParams;
                const float x = F.tri[3 * k], y = F.tri[3 * k + 1], z = F.tri[3 * k + 2];
#pragma unroll
                for (int c = 0; c < kF; c++)
                    v[c] = (raw_feature(c, th, x, y, z) - F.mu[c]) * F.isd[c];
            } else {
#pragma unroll
                for (int c = 0; c < kF; c++) v[c] = 0.f;
            }
#pragma unroll
            for (int c = 0; c < kF; c += 2)
                *reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(T.a1) +
                                              canon_offset(tid, c, kF)) = pack2(v[c], v[c + 1]);
        }
        proxy_fence();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            // K = 16: one MMA
            tc_mma(d1, smem_desc(T.a1, 128, (kF / 8) * 128), smem_desc(T.b1, 128, (kF / 8) * 128),
                   false);
            tc_commit(&T.bar);
        }
        // every thread votes, so that the whole block leaves together on a timeout
        if (!__syncthreads_and(tc_wait(&T.bar, parity))) {
            ok = false;
            if (tid == 0) atomicExch(status, SWGPU_ETIMEOUT);
            break;
        }
        parity ^= 1u;
        tc_fence_after();
        // ---- layer-1 epilogue: bias, ReLU, BF16 into layer-2 A
#pragma unroll
        for (int ch = 0; ch < 4; ch++) {
            float v[32];
            tc_ld32(d1 + lane_base + 32u * ch, v);
#pragma unroll
            for (int c = 0; c < 32; c += 2) {
                const int col = 32 * ch + c;
                const float a = fmaxf(v[c] + T.bias1[col], 0.f);
                const float b = fmaxf(v[c + 1] + T.bias1[col + 1], 0.f);
                *reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(T.a2) +
                                              canon_offset(tid, col, kH)) = pack2(a, b);
            }
        }
        proxy_fence();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
#pragma unroll
            for (int kk = 0; kk < kH / 16; kk++)  // K = 128 in 8 steps of 16
                tc_mma(d2,
                       smem_desc(reinterpret_cast<unsigned char *>(T.a2) + kk * 256, 128,
                                 (kH / 8) * 128),
                       smem_desc(reinterpret_cast<unsigned char *>(T.b2) + kk * 256, 128,
                                 (kH / 8) * 128),
                       kk > 0);
            tc_commit(&T.bar);
        }
        if (!__syncthreads_and(tc_wait(&T.bar, parity))) {
            ok = false;
            if (tid == 0) atomicExch(status, SWGPU_ETIMEOUT);
            break;
        }
        parity ^= 1u;
        tc_fence_after();
        // ---- layer-2 epilogue and the output layer on the CUDA cores
        float y0 = T.bias3[0], y1 = T.bias3[1];
#pragma unroll
        for (int ch = 0; ch < 4; ch++) {
            float v[32];
            tc_ld32(d2 + lane_base + 32u * ch, v);
#pragma unroll
            for (int c = 0; c < 32; c++) {
                const int col = 32 * ch + c;
                // the activation is rounded to BF16 like the mma.sync path's
                const float a = __bfloat162float(__float2bfloat16(fmaxf(v[c] + T.bias2[col], 0.f)));
                y0 += a * T.w3[2 * col];
                y1 += a * T.w3[2 * col + 1];
            }
        }
        if (valid) {
            out[2 * r] = y0;
            out[2 * r + 1] = y1;
        }
        tc_fence_before();
        __syncthreads();  // TMEM and the A tiles are reused by the next tile
        tc_fence_after();
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem)
                     : "memory");
}

// ---- training ------------------------------------------------------------
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Row of batch position r: either given, or drawn uniformly from all
// (scenario, triangle) pairs of the training set.
__device__ __forceinline__ long long batch_row(const long long *rows, unsigned long long seed,
                                               long long r, long long total) {
    if (rows) return rows[r];
    return (long long)(mix64(seed ^ (unsigned long long)r * 0xD1B54A32D192ED03ull) %
                       (unsigned long long)total);
}

struct BatchScratch {
    __nv_bfloat16 *x;   // [B][16]
    __nv_bfloat16 *a1;  // [B][128]
    __nv_bfloat16 *a2;  // [B][128]
    float *dz1;         // [B][128]
    float *dz2;         // [B][128]
    float *dy;          // [B][2]
    float *y;           // [B][2] outputs
};

// Forward and backward of a batch: loss = mean over rows and outputs of
// wt_o (y_o - target_o)^2.  Stores the inputs, activations and the
// gradients with respect to each layer's pre-activations for the weight
// gradient kernel; accumulates the loss.
__global__ void __launch_bounds__(32 * kWarps)
    mlp_forward_backward(FeatureTables F, const BfWeights *gw, const float *__restrict__ targets,
                         const long long *rows, unsigned long long seed, long long batch,
                         long long total, float w_depth, float w_arrival, BatchScratch B,
                         float *loss) {
    extern __shared__ __align__(16) unsigned char smem[];
    BfWeights &W = *reinterpret_cast<BfWeights *>(smem);
    load_weights(W, gw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float my_loss = 0.0f;
    const float inv_b = 1.0f / (float)batch;
    for (long long base = (long long)blockIdx.x * kRowsPerBlock; base < batch;
         base += (long long)gridDim.x * kRowsPerBlock) {
        const long long ra = base + 16 * warp + g, rb = ra + 8;
        const bool va = ra < batch, vb = rb < batch;
        const long long qa = va ? batch_row(rows, seed, ra, total) : 0;
        const long long qb = vb ? batch_row(rows, seed, rb, total) : 0;
        uint32_t x[1][4];
        load_features(F, qa, qb, va, vb, x[0]);
        uint32_t a1[8][4], a2[8][4];
        hidden_layer<1, kS1>(x, W.w1t, W.b1, a1);
        hidden_layer<8, kS2>(a1, W.w2t, W.b2, a2);
        float y[4];
        output_layer(a2, W, y);
        // dL/dy for outputs 0 and 1 of rows a and b (held by t == 0)
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        if (t == 0) {
            const float wts[2] = {w_depth, w_arrival};
            if (va) {
#pragma unroll
                for (int o = 0; o < 2; o++) {
                    const float e = y[o] - targets[2 * qa + o];
                    d[o] = 2.0f * wts[o] * e * inv_b;
                    my_loss += wts[o] * e * e * inv_b;
                    B.dy[2 * ra + o] = d[o];
                    B.y[2 * ra + o] = y[o];
                }
            }
            if (vb) {
#pragma unroll
                for (int o = 0; o < 2; o++) {
                    const float e = y[2 + o] - targets[2 * qb + o];
                    d[2 + o] = 2.0f * wts[o] * e * inv_b;
                    my_loss += wts[o] * e * e * inv_b;
                    B.dy[2 * rb + o] = d[2 + o];
                    B.y[2 * rb + o] = y[2 + o];
                }
            }
        }
        // broadcast the group's dy to its 4 threads
        const int src = lane & ~3;
#pragma unroll
        for (int i = 0; i < 4; i++) d[i] = __shfl_sync(0xffffffffu, d[i], src);
        // dz2 = (dy W3^T) * relu'(z2), in the C layout of layer 2; re-packed
        // as A fragments for dz2 W2^T
        uint32_t g2[8][4];
#pragma unroll
        for (int jj = 0; jj < 8; jj++) {
            float dz[2][4];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = 2 * jj + h;
                const int u0 = 8 * j + 2 * t, u1 = u0 + 1;
                const float2 w30 = __bfloat1622float2(
                    *reinterpret_cast<const __nv_bfloat162 *>(&W.w3[u0 * 8]));
                const float2 w31 = __bfloat1622float2(
                    *reinterpret_cast<const __nv_bfloat162 *>(&W.w3[u1 * 8]));
                const float2 pa = unpack2(a2[jj][h == 0 ? 0 : 2]);  // row a, units u0,u1
                const float2 pb = unpack2(a2[jj][h == 0 ? 1 : 3]);  // row b
                dz[h][0] = pa.x > 0.f ? d[0] * w30.x + d[1] * w30.y : 0.f;
                dz[h][1] = pa.y > 0.f ? d[0] * w31.x + d[1] * w31.y : 0.f;
                dz[h][2] = pb.x > 0.f ? d[2] * w30.x + d[3] * w30.y : 0.f;
                dz[h][3] = pb.y > 0.f ? d[2] * w31.x + d[3] * w31.y : 0.f;
                if (va) {
                    B.dz2[ra * kH + u0] = dz[h][0];
                    B.dz2[ra * kH + u1] = dz[h][1];
                }
                if (vb) {
                    B.dz2[rb * kH + u0] = dz[h][2];
                    B.dz2[rb * kH + u1] = dz[h][3];
                }
            }
            g2[jj][0] = pack2(dz[0][0], dz[0][1]);
            g2[jj][1] = pack2(dz[0][2], dz[0][3]);
            g2[jj][2] = pack2(dz[1][0], dz[1][1]);
            g2[jj][3] = pack2(dz[1][2], dz[1][3]);
        }
        // dz1 = (dz2 W2^T) * relu'(z1)
#pragma unroll
        for (int jj = 0; jj < 8; jj++) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = 2 * jj + h;
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
                const __nv_bfloat16 *col = W.w2 + (8 * j + g) * kS2;
#pragma unroll
                for (int kk = 0; kk < 8; kk++)
                    mma16816(acc, g2[kk], lds32(col + 16 * kk + 2 * t),
                             lds32(col + 16 * kk + 8 + 2 * t));
                const int u0 = 8 * j + 2 * t, u1 = u0 + 1;
                const float2 pa = unpack2(a1[jj][h == 0 ? 0 : 2]);
                const float2 pb = unpack2(a1[jj][h == 0 ? 1 : 3]);
                if (va) {
                    B.dz1[ra * kH + u0] = pa.x > 0.f ? acc[0] : 0.f;
                    B.dz1[ra * kH + u1] = pa.y > 0.f ? acc[1] : 0.f;
                }
                if (vb) {
                    B.dz1[rb * kH + u0] = pb.x > 0.f ? acc[2] : 0.f;
                    B.dz1[rb * kH + u1] = pb.y > 0.f ? acc[3] : 0.f;
                }
            }
        }
        // inputs and activations of the rows for the weight gradients
#pragma unroll
        for (int jj = 0; jj < 8; jj++) {
            const int u0 = 16 * jj + 2 * t;
            if (va) {
                *reinterpret_cast<uint32_t *>(&B.a1[ra * kH + u0]) = a1[jj][0];
                *reinterpret_cast<uint32_t *>(&B.a1[ra * kH + u0 + 8]) = a1[jj][2];
                *reinterpret_cast<uint32_t *>(&B.a2[ra * kH + u0]) = a2[jj][0];
                *reinterpret_cast<uint32_t *>(&B.a2[ra * kH + u0 + 8]) = a2[jj][2];
            }
            if (vb) {
                *reinterpret_cast<uint32_t *>(&B.a1[rb * kH + u0]) = a1[jj][1];
                *reinterpret_cast<uint32_t *>(&B.a1[rb * kH + u0 + 8]) = a1[jj][3];
                *reinterpret_cast<uint32_t *>(&B.a2[rb * kH + u0]) = a2[jj][1];
                *reinterpret_cast<uint32_t *>(&B.a2[rb * kH + u0 + 8]) = a2[jj][3];
            }
        }
        if (va) {
            *reinterpret_cast<uint32_t *>(&B.x[ra * kF + 2 * t]) = x[0][0];
            *reinterpret_cast<uint32_t *>(&B.x[ra * kF + 2 * t + 8]) = x[0][2];
        }
        if (vb) {
            *reinterpret_cast<uint32_t *>(&B.x[rb * kF + 2 * t]) = x[0][1];
            *reinterpret_cast<uint32_t *>(&B.x[rb * kF + 2 * t + 8]) = x[0][3];
        }
    }
    for (int o = 16; o > 0; o >>= 1) my_loss += __shfl_xor_sync(0xffffffffu, my_loss, o);
    if (lane == 0) atomicAdd(loss, my_loss);
}

// Weight gradients: grad[i][o] += sum over a chunk of rows of
// in[r][i] * dz[r][o] (FP32), one block per (layer tile, row chunk).
constexpr int kChunk = 256;
__global__ void __launch_bounds__(256) mlp_weight_grads(BatchScratch B, long long batch,
                                                        float *__restrict__ grad) {
    __shared__ float sin_[32][kH + 1];
    __shared__ float sdz[32][kH + 1];
    // blockIdx.y: 0 -> W2 (128 x 128), 1 -> W1 (16 x 128), 2 -> W3 (128 x 2),
    // 3 -> biases b1, b2, b3
    const int layer = blockIdx.y;
    const long long r0 = (long long)blockIdx.x * kChunk;
    const long long r1 = r0 + kChunk < batch ? r0 + kChunk : batch;
    const int tid = threadIdx.x;
    // each thread owns 64 (i, o) entries of a 128 x 128 tile: i = tid / 2,
    // o = (tid % 2) * 64 + c
    float acc[64];
#pragma unroll
    for (int c = 0; c < 64; c++) acc[c] = 0.f;
    const int ni = layer == 1 ? kF : kH;
    const int no = layer == 2 ? kOut : kH;
    for (long long rb = r0; rb < r1; rb += 32) {
        const int nr = (int)(r1 - rb < 32 ? r1 - rb : 32);
        for (int e = tid; e < 32 * kH; e += 256) {
            const int rr = e / kH, c = e % kH;
            float vin = 0.f, vdz = 0.f;
            if (rr < nr) {
                const long long r = rb + rr;
                if (layer == 0) {
                    vin = __bfloat162float(B.a1[r * kH + c]);
                    vdz = B.dz2[r * kH + c];
                } else if (layer == 1) {
                    vin = c < kF ? __bfloat162float(B.x[r * kF + c]) : 0.f;
                    vdz = B.dz1[r * kH + c];
                } else if (layer == 2) {
                    vin = __bfloat162float(B.a2[r * kH + c]);
                    vdz = c < kOut ? B.dy[r * kOut + c] : 0.f;
                } else {
                    vin = B.dz1[r * kH + c];   // bias rows: b1 from dz1, b2 from dz2,
                    vdz = B.dz2[r * kH + c];   // b3 from dy
                }
            }
            sin_[rr][c] = vin;
            sdz[rr][c] = vdz;
        }
        __syncthreads();
        if (layer < 3) {
            const int i = tid >> 1, ob = (tid & 1) * 64;
            if (i < ni) {
                for (int rr = 0; rr < nr; rr++) {
                    const float a = sin_[rr][i];
#pragma unroll
                    for (int c = 0; c < 64; c++) acc[c] += a * sdz[rr][ob + c];
                }
            }
        } else if (tid < kH) {
            for (int rr = 0; rr < nr; rr++) {
                acc[0] += sin_[rr][tid];
                acc[1] += sdz[rr][tid];
            }
            if (tid < kOut)
                for (int rr = 0; rr < nr; rr++) acc[2] += B.dy[(rb + rr) * kOut + tid];
        }
        __syncthreads();
    }
    if (layer < 3) {
        const int i = tid >> 1, ob = (tid & 1) * 64;
        if (i >= ni) return;
        float *gw = grad + (layer == 0 ? kOffW2 : layer == 1 ? kOffW1 : kOffW3);
        for (int c = 0; c < 64; c++) {
            const int o = ob + c;
            if (o < no) atomicAdd(&gw[i * no + o], acc[c]);
        }
    } else if (tid < kH) {
        atomicAdd(&grad[kOffB1 + tid], acc[0]);
        atomicAdd(&grad[kOffB2 + tid], acc[1]);
        if (tid < kOut) atomicAdd(&grad[kOffB3 + tid], acc[2]);
    }
}

// BF16 images of the FP32 parameters.
__global__ void mlp_pack_weights(const float *__restrict__ p, BfWeights *W) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    if (tid < kH * kS1) {
        const int o = tid / kS1, i = tid % kS1;
        W->w1t[tid] = i < kF ? __float2bfloat16(p[kOffW1 + i * kH + o]) : zero;
    }
    if (tid < kH * kS2) {
        const int r = tid / kS2, c = tid % kS2;
        W->w2t[tid] = c < kH ? __float2bfloat16(p[kOffW2 + c * kH + r]) : zero;
        W->w2[tid] = c < kH ? __float2bfloat16(p[kOffW2 + r * kH + c]) : zero;
    }
    if (tid < 8 * kS2) {
        const int o = tid / kS2, i = tid % kS2;
        W->w3t[tid] = (o < kOut && i < kH) ? __float2bfloat16(p[kOffW3 + i * kOut + o]) : zero;
    }
    if (tid < kH * 8) {
        const int i = tid / 8, o = tid % 8;
        W->w3[tid] = o < kOut ? __float2bfloat16(p[kOffW3 + i * kOut + o]) : zero;
    }
    if (tid < kH) {
        W->b1[tid] = p[kOffB1 + tid];
        W->b2[tid] = p[kOffB2 + tid];
    }
    if (tid < 8) W->b3[tid] = tid < kOut ? p[kOffB3 + tid] : 0.f;
}

// Adam on the FP32 master parameters.
__global__ void mlp_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                         float *__restrict__ v, int n, float lr, float b1, float b2, float eps,
                         float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

struct Mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    float *params = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    BfWeights *w = nullptr;
    float *mu = nullptr, *isd = nullptr;
    float *scen = nullptr, *tri = nullptr, *targets = nullptr;
    long long S = 0, N = 0;
    BatchScratch scratch{};
    long long scratch_rows = 0;
    long long *rows = nullptr;
    long long rows_cap = 0;
    float *loss = nullptr;
    int *status = nullptr;   // device-side failure of the tensor-core kernel
    int tensor_path = 0;     // 0: mma.sync, 1: tcgen05 (inference)
    long long adam_t = 0;
    std::vector<void *> allocs;
    std::string err;
};

thread_local std::string g_mlp_error;

int mfail(Mlp *m, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (m) m->err = buf;
    g_mlp_error = buf;
    return code;
}

#define MCK(x)                                                                         \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess)                                                         \
            return mfail(m, SWGPU_ECUDA, "%s: %s", #x, cudaGetErrorString(e_));       \
    } while (0)

template <typename T>
int malloc_dev(Mlp *m, T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
    if (e != cudaSuccess)
        return mfail(m, SWGPU_ENOMEM, "cudaMalloc %zu bytes: %s", count * sizeof(T),
                     cudaGetErrorString(e));
    m->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return SWGPU_OK;
}

int ensure_scratch(Mlp *m, long long batch) {
    if (batch <= m->scratch_rows) return SWGPU_OK;
    int rc;
    BatchScratch &B = m->scratch;
    if ((rc = malloc_dev(m, &B.x, (size_t)batch * kF))) return rc;
    if ((rc = malloc_dev(m, &B.a1, (size_t)batch * kH))) return rc;
    if ((rc = malloc_dev(m, &B.a2, (size_t)batch * kH))) return rc;
    if ((rc = malloc_dev(m, &B.dz1, (size_t)batch * kH))) return rc;
    if ((rc = malloc_dev(m, &B.dz2, (size_t)batch * kH))) return rc;
    if ((rc = malloc_dev(m, &B.dy, (size_t)batch * kOut))) return rc;
    if ((rc = malloc_dev(m, &B.y, (size_t)batch * kOut))) return rc;
    m->scratch_rows = batch;
    return SWGPU_OK;
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

FeatureTables tables(const Mlp *m) {
    return FeatureTables{m->scen, m->tri, m->mu, m->isd, m->N};
}

// forward + backward + weight gradients of one batch into m->grad
int batch_gradients(Mlp *m, const long long *d_rows, unsigned long long seed, long long batch,
                    long long total, float w_depth, float w_arrival) {
    int rc = ensure_scratch(m, batch);
    if (rc) return rc;
    MCK(cudaMemsetAsync(m->grad, 0, sizeof(float) * kNumParams, m->stream));
    MCK(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
    const long long tiles = (batch + kRowsPerBlock - 1) / kRowsPerBlock;
    const int grid = (int)std::min<long long>(tiles, 4LL * sm_count());
    mlp_forward_backward<<<grid, 32 * kWarps, sizeof(BfWeights), m->stream>>>(
        tables(m), m->w, m->targets, d_rows, seed, batch, total, w_depth, w_arrival, m->scratch,
        m->loss);
    const dim3 g2((unsigned)((batch + kChunk - 1) / kChunk), 4);
    mlp_weight_grads<<<g2, 256, 0, m->stream>>>(m->scratch, batch, m->grad);
    MCK(cudaGetLastError());
    return SWGPU_OK;
}

}  // namespace

extern "C" {

int swgpu_mlp_create(const float *params, const float *feature_mean,
                     const float *feature_inv_std, void **handle_out) {
    if (!params || !feature_mean || !feature_inv_std || !handle_out)
        return mfail(nullptr, SWGPU_EINVAL, "swgpu_mlp_create: null argument");
    *handle_out = nullptr;
    Mlp *m = new Mlp();
    int rc = SWGPU_OK;
    cudaError_t e = cudaGetDevice(&m->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(BfWeights));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_predict_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(TcSmem) + 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_forward_backward,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(BfWeights));
    if (e != cudaSuccess) {
        rc = mfail(m, SWGPU_ECUDA, "swgpu_mlp_create: %s", cudaGetErrorString(e));
        delete m;
        return rc;
    }
    if ((rc = malloc_dev(m, &m->params, kNumParams)) || (rc = malloc_dev(m, &m->grad, kNumParams)) ||
        (rc = malloc_dev(m, &m->adam_m, kNumParams)) ||
        (rc = malloc_dev(m, &m->adam_v, kNumParams)) || (rc = malloc_dev(m, &m->w, 1)) ||
        (rc = malloc_dev(m, &m->mu, kF)) || (rc = malloc_dev(m, &m->isd, kF)) ||
        (rc = malloc_dev(m, &m->loss, 1)) || (rc = malloc_dev(m, &m->status, 1))) {
        for (void *p : m->allocs) cudaFree(p);
        delete m;
        return rc;
    }
    cudaMemcpy(m->params, params, sizeof(float) * kNumParams, cudaMemcpyHostToDevice);
    cudaMemcpy(m->mu, feature_mean, sizeof(float) * kF, cudaMemcpyHostToDevice);
    cudaMemcpy(m->isd, feature_inv_std, sizeof(float) * kF, cudaMemcpyHostToDevice);
    cudaMemset(m->adam_m, 0, sizeof(float) * kNumParams);
    cudaMemset(m->adam_v, 0, sizeof(float) * kNumParams);
    cudaMemset(m->status, 0, sizeof(int));
    mlp_pack_weights<<<(kH * kS2 + 255) / 256, 256, 0, m->stream>>>(m->params, m->w);
    e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        rc = mfail(m, SWGPU_ECUDA, "swgpu_mlp_create: %s", cudaGetErrorString(e));
        for (void *p : m->allocs) cudaFree(p);
        delete m;
        return rc;
    }
    *handle_out = m;
    return SWGPU_OK;
}

int swgpu_mlp_destroy(void *handle) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m) return SWGPU_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    for (void *p : m->allocs) cudaFree(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return SWGPU_OK;
}

const char *swgpu_mlp_last_error(void *handle) {
    Mlp *m = static_cast<Mlp *>(handle);
    return m ? m->err.c_str() : g_mlp_error.c_str();
}

int swgpu_mlp_set_data(void *handle, const float *tri_xyz, int64_t ntri, const float *scen,
                       int64_t nscen, const float *targets) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || !tri_xyz || !scen || ntri <= 0 || nscen <= 0)
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_set_data: bad argument");
    if ((long long)ntri * nscen >= (1LL << 40))
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_set_data: too many rows");
    int rc;
    if ((rc = malloc_dev(m, &m->tri, (size_t)ntri * 3)) ||
        (rc = malloc_dev(m, &m->scen, (size_t)nscen * kParams)))
        return rc;
    MCK(cudaMemcpy(m->tri, tri_xyz, sizeof(float) * 3 * ntri, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->scen, scen, sizeof(float) * kParams * nscen, cudaMemcpyHostToDevice));
    m->targets = nullptr;
    if (targets) {
        if ((rc = malloc_dev(m, &m->targets, (size_t)ntri * nscen * kOut))) return rc;
        MCK(cudaMemcpy(m->targets, targets, sizeof(float) * kOut * ntri * nscen,
                       cudaMemcpyHostToDevice));
    }
    m->N = ntri;
    m->S = nscen;
    return SWGPU_OK;
}

int swgpu_mlp_predict(void *handle, int64_t row0, int64_t nrows, float *out_device,
                      float *elapsed_ms) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || !out_device || nrows <= 0 || row0 < 0 || row0 + nrows > m->S * m->N)
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_predict: bad rows");
    cudaEvent_t a, b;
    MCK(cudaEventCreate(&a));
    MCK(cudaEventCreate(&b));
    MCK(cudaEventRecord(a, m->stream));
    if (m->tensor_path == 1) {
        // two CTAs per SM: each holds 256 TMEM columns of the SM's 512
        const long long tiles = (nrows + kTcRows - 1) / kTcRows;
        const int grid = (int)std::min<long long>(tiles, 2LL * sm_count());
        mlp_predict_tc<<<grid, 128, sizeof(TcSmem) + 1024, m->stream>>>(
            tables(m), m->params, row0, nrows, out_device, m->status);
    } else {
        const long long tiles = (nrows + kRowsPerBlock - 1) / kRowsPerBlock;
        const int grid = (int)std::min<long long>(tiles, 4LL * sm_count());
        mlp_predict<<<grid, 32 * kWarps, sizeof(BfWeights), m->stream>>>(tables(m), m->w, row0,
                                                                          nrows, out_device);
    }
    MCK(cudaGetLastError());
    MCK(cudaEventRecord(b, m->stream));
    MCK(cudaEventSynchronize(b));
    if (m->tensor_path == 1) {
        int st = 0;
        MCK(cudaMemcpy(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost));
        if (st) return mfail(m, st, "swgpu_mlp_predict: tensor-core wait timed out");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (elapsed_ms) *elapsed_ms = ms;
    return SWGPU_OK;
}

int swgpu_mlp_gradients(void *handle, const int64_t *rows, int64_t nrows, float w_depth,
                        float w_arrival, float *outputs, float *grad, float *loss) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || !rows || nrows <= 0 || !m->targets)
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_gradients: bad argument or no targets");
    int rc;
    if (nrows > m->rows_cap) {
        if ((rc = malloc_dev(m, &m->rows, (size_t)nrows))) return rc;
        m->rows_cap = nrows;
    }
    MCK(cudaMemcpyAsync(m->rows, rows, sizeof(long long) * nrows, cudaMemcpyHostToDevice,
                        m->stream));
    if ((rc = batch_gradients(m, m->rows, 0, nrows, m->S * m->N, w_depth, w_arrival))) return rc;
    if (outputs)
        MCK(cudaMemcpyAsync(outputs, m->scratch.y, sizeof(float) * kOut * nrows,
                            cudaMemcpyDeviceToHost, m->stream));
    if (grad)
        MCK(cudaMemcpyAsync(grad, m->grad, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost,
                            m->stream));
    if (loss)
        MCK(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return SWGPU_OK;
}

int swgpu_mlp_train(void *handle, int steps, int64_t batch, uint64_t seed, float lr,
                    float w_depth, float w_arrival, float *last_loss, float *elapsed_ms) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || steps <= 0 || batch <= 0 || !m->targets)
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_train: bad argument or no targets");
    cudaEvent_t a, b;
    MCK(cudaEventCreate(&a));
    MCK(cudaEventCreate(&b));
    MCK(cudaEventRecord(a, m->stream));
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < steps; s++) {
        const unsigned long long step_seed = seed * 0x9E3779B97F4A7C15ull + (unsigned)s;
        int rc = batch_gradients(m, nullptr, step_seed, batch, m->S * m->N, w_depth, w_arrival);
        if (rc) return rc;
        m->adam_t++;
        const float c1 = 1.f / (1.f - powf(b1, (float)m->adam_t));
        const float c2 = 1.f / (1.f - powf(b2, (float)m->adam_t));
        mlp_adam<<<(kNumParams + 255) / 256, 256, 0, m->stream>>>(
            m->params, m->grad, m->adam_m, m->adam_v, kNumParams, lr, b1, b2, 1e-8f, c1, c2);
        mlp_pack_weights<<<(kH * kS2 + 255) / 256, 256, 0, m->stream>>>(m->params, m->w);
    }
    MCK(cudaGetLastError());
    MCK(cudaEventRecord(b, m->stream));
    MCK(cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (elapsed_ms) *elapsed_ms = ms;
    if (last_loss) MCK(cudaMemcpy(last_loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    return SWGPU_OK;
}

int swgpu_mlp_get_params(void *handle, float *params) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || !params) return mfail(m, SWGPU_EINVAL, "swgpu_mlp_get_params: null argument");
    MCK(cudaStreamSynchronize(m->stream));
    MCK(cudaMemcpy(params, m->params, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost));
    return SWGPU_OK;
}

int swgpu_mlp_num_params(void) { return kNumParams; }

int swgpu_mlp_set_tensor_path(void *handle, int path) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || (path != 0 && path != 1))
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_set_tensor_path: 0 (mma.sync) or 1 (tcgen05)");
    m->tensor_path = path;
    return SWGPU_OK;
}

}  // extern "C"
