// swgpu_mlp.cu -- BF16 surrogate network of the solver's maximum depth and
// arrival time, on the 5th-generation tensor cores (tcgen05, TMEM).
//
// Rows are (scenario s, triangle k) pairs.  Each row's 16 input features
// are assembled on the fly: the scenario's 9 parameters, the triangle's
// centroid x and y, bed elevation and distance to the inflow, and 3 zeros,
// each normalised by a per-feature affine map.  The network is
//   16 -> 256 -> 256 -> 256 -> 3  (ReLU after each hidden layer)
// with weights and activations in BF16 and every product accumulated in
// FP32; its outputs are the normalised maximum depth, the normalised
// arrival time and the 90% quantile of the first output's absolute error.
//
// Every GEMM of the forward and backward passes is the one kernel
// tc_gemm: a CTA of 4 warps computes a 128 x N tile (N = 256 or 16) of
// A (M x K) times B (N x K)^T, both operands K-major in global memory.
// Chunks of 64 along K are staged by cp.async into shared memory in the
// canonical K-major no-swizzle layout (8-row x 16-byte core matrices, 128
// bytes apart along K, (K/8)*128 bytes apart along M/N), double-buffered;
// one thread issues the chunk's tcgen05.mma (kind::f16, M = 128) into an
// FP32 accumulator in tensor memory and commits it to the stage's
// mbarrier, which frees the stage for the chunk after next.  The epilogue
// reads each warp's 32 TMEM lanes (its 32 rows) with tcgen05.ld and either
//  * adds the bias, applies ReLU and stores BF16 activations (a hidden
//    layer of the forward pass),
//  * multiplies by the ReLU mask of the previous activations and stores
//    BF16 gradients (the backward pass through a layer), or
//  * adds the FP32 partial weight gradient of its slice of the batch into
//    the gradient vector (split over the batch, K = rows).
// Activations and gradients are stored row-major (rows x features) for the
// next layer's A operand and, in training, also feature-major (features x
// rows) for the weight gradients, whose K is the batch.  The 256 -> 3
// output layer and its gradient run on the CUDA cores (head kernels).
// Training keeps FP32 master weights updated by Adam.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "swgpu_internal.cuh"

namespace {

constexpr int kF = 16;       // input features (13 used)
constexpr int kH = 256;      // hidden units per layer
constexpr int kOut = 3;      // outputs: depth, arrival time, depth-error estimate
constexpr int kTargets = 2;  // targets per row: depth, arrival time
constexpr int kParams = 9;   // scenario parameters
constexpr int kTri = 4;      // per-triangle table: x, y, z, distance to the inflow
constexpr float kQuantile = 0.9f;  // quantile of the depth error the third output learns

// flat FP32 parameter vector, weights in-major ([in][out]):
// W1 [16][256], b1, W2 [256][256], b2, W3 [256][256], b3, W4 [256][3], b4
constexpr long kOffW1 = 0;
constexpr long kOffB1 = kOffW1 + kF * kH;
constexpr long kOffW2 = kOffB1 + kH;
constexpr long kOffB2 = kOffW2 + kH * kH;
constexpr long kOffW3 = kOffB2 + kH;
constexpr long kOffB3 = kOffW3 + kH * kH;
constexpr long kOffW4 = kOffB3 + kH;
constexpr long kOffB4 = kOffW4 + kH * kOut;
constexpr long kNumParams = kOffB4 + kOut;

// BF16 weight images in the layouts the GEMMs read as their B operand
// (N x K, K contiguous): forward layers need W^T ([out][in]), the backward
// pass through a layer needs W itself ([in][out]).
struct BfWeights {
    __nv_bfloat16 wt1[kH * kF];   // [out][in]
    __nv_bfloat16 wt2[kH * kH];
    __nv_bfloat16 wt3[kH * kH];
    __nv_bfloat16 w2[kH * kH];    // [in][out]
    __nv_bfloat16 w3[kH * kH];
    __nv_bfloat16 w4[kH * kOut];  // [in][out] (head, CUDA cores)
};

// ---- features --------------------------------------------------------------

struct FeatureTables {
    const float *scen;   // [S][9]
    const float *tri;    // [N][4]: x, y, z, distance to the inflow
    const float *mu;     // [16]
    const float *isd;    // [16]
    long long N;
};

__device__ __forceinline__ float raw_feature(int c, const float *th, const float *tr) {
    if (c < kParams) return th[c];
    if (c == 9) return tr[2];   // bed
    if (c == 10) return tr[0];  // x
    if (c == 11) return tr[1];  // y
    if (c == 12) return tr[3];  // distance to the inflow
    return 0.0f;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Row of batch position r: given (rows), drawn uniformly from all (scenario,
// triangle) pairs (seeded), or row0 + r (inference).
__device__ __forceinline__ long long batch_row(const long long *rows, unsigned long long seed,
                                               long long r, long long total, long long row0) {
    if (rows) return rows[r];
    if (total > 0)
        return (long long)(mix64(seed ^ (unsigned long long)r * 0xD1B54A32D192ED03ull) %
                           (unsigned long long)total);
    return row0 + r;
}

// Normalised BF16 features of batch rows [0, nrows): row-major xr [Bp][16]
// and (training) feature-major xc [16][Bp]; rows nrows..Bp-1 are zero.
// Also records each batch row's data row (training targets).
__global__ void __launch_bounds__(256) mlp_features(FeatureTables F, const long long *rows,
                                                    unsigned long long seed, long long total,
                                                    long long row0, long long nrows, long long Bp,
                                                    __nv_bfloat16 *__restrict__ xr,
                                                    __nv_bfloat16 *__restrict__ xc,
                                                    long long *__restrict__ row_of) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= Bp) return;
    float v[kF];
    if (r < nrows) {
        const long long q = batch_row(rows, seed, r, total, row0);
        if (row_of) row_of[r] = q;
        const long long s = q / F.N, k = q - s * F.N;
        const float *th = F.scen + s * kParams;
        const float *tr = F.tri + k * kTri;
#pragma unroll
        for (int c = 0; c < kF; c++) v[c] = (raw_feature(c, th, tr) - F.mu[c]) * F.isd[c];
    } else {
#pragma unroll
        for (int c = 0; c < kF; c++) v[c] = 0.0f;
    }
    __align__(16) __nv_bfloat16 b[kF];
#pragma unroll
    for (int c = 0; c < kF; c++) b[c] = __float2bfloat16(v[c]);
    int4 *dst = reinterpret_cast<int4 *>(xr + r * kF);
    dst[0] = reinterpret_cast<const int4 *>(b)[0];
    dst[1] = reinterpret_cast<const int4 *>(b)[1];
    if (xc) {
#pragma unroll
        for (int c = 0; c < kF; c++) xc[c * Bp + r] = b[c];
    }
}

// ---- tcgen05 GEMM ----------------------------------------------------------

constexpr int kTileM = 128;  // rows per CTA (TMEM lanes)
constexpr int kChunkK = 64;  // K per stage
constexpr int kGemmThreads = 256;  // 8 warps: the epilogue splits the columns in two

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start, leading-dimension byte offset
// (between core matrices along K), stride byte offset (between 8-row groups
// along M/N), descriptor version 1 (bit 46), no swizzle.
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo,
                                                        unsigned sbo) {
    return (unsigned long long)((addr >> 4) & 0x3FFFu) |
           ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N given.
__host__ __device__ constexpr unsigned tc_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) |
           ((unsigned)(kTileM >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(unsigned d_tmem, unsigned long long a,
                                       unsigned long long b, unsigned idesc, bool accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"((unsigned)accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
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
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
constexpr int kTcWaitLimit = 1 << 22;
// Bounded wait of the whole CTA for an MMA commit: every thread polls at
// most kTcWaitLimit times; true when all saw the phase complete.
__device__ __forceinline__ bool cta_wait(unsigned long long *bar, unsigned parity) {
    bool ok = false;
    for (int i = 0; i < kTcWaitLimit && !ok; i++) ok = mbar_test(bar, parity);
    return __syncthreads_and(ok) != 0;
}

// 16-byte asynchronous copy global -> shared; src_bytes 0 fills zeros.
__device__ __forceinline__ void cp_async16(unsigned dst, const void *src, unsigned src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Stages rows [r0, r0 + R) x k-range [k0, k0 + kc) of a K-major matrix
// (row stride ld elements, nvalid valid rows) into the canonical layout at
// smem address dst.  Vector v (8 elements) goes to byte 16 v: the 8 lanes
// of a group take 8 consecutive rows at one k (a 128-byte core matrix),
// consecutive groups the next k, so a warp stores 512 contiguous bytes and
// reads 64 contiguous bytes of each of 8 rows.
__device__ __forceinline__ void stage_operand(unsigned dst, const __nv_bfloat16 *src, long ld,
                                              long long r0, long long nvalid, int R, long k0,
                                              int kc) {
    const int lg = kc == kChunkK ? 3 : 1;  // log2 of the 16-byte vectors per row (kc 64 or 16)
    const int nvec = R << lg;
    for (int v = threadIdx.x; v < nvec; v += kGemmThreads) {
        const int r = (v & 7) + ((v >> (3 + lg)) << 3);
        const int kv = (v >> 3) & ((1 << lg) - 1);
        const long long row = r0 + r;
        const bool in = row < nvalid;
        const __nv_bfloat16 *p = in ? src + row * ld + k0 + 8 * kv : src;
        cp_async16(dst + 16u * (unsigned)v, p, in ? 16u : 0u);
    }
}

enum { kEpiHidden = 0, kEpiDgrad = 1, kEpiWgrad = 2, kEpiWgradT = 3 };

struct GemmArgs {
    const __nv_bfloat16 *A;  // M x K, K contiguous, row stride lda
    long lda;
    const __nv_bfloat16 *B;  // N x K, K contiguous, row stride ldb
    long ldb;
    long long M;             // valid rows of A (and of the output)
    long K;                  // K of the whole product (a multiple of 16)
    long k_per_split;        // K range of one blockIdx.y (a multiple of 64, or K)
    // epilogue
    const float *bias;               // hidden: [N]
    const __nv_bfloat16 *mask;       // dgrad: previous activations [M][N] row-major
    __nv_bfloat16 *out_row;          // hidden/dgrad: [M][N]
    __nv_bfloat16 *out_col;          // hidden/dgrad: [N][ldc] (may be null)
    long ldc;
    float *grad;                     // wgrad: partials [splits][M][N] (or [splits][N][M]
                                     // transposed), one slice per blockIdx.y
    int *status;
};

template <int N>
struct __align__(1024) GemmSmem {
    __nv_bfloat16 a[2][kTileM * kChunkK];
    __nv_bfloat16 b[2][N * kChunkK];
    unsigned long long bar[2];
    unsigned tmem_base;
};

template <int N>
__host__ __device__ constexpr int tmem_cols() {
    return N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
}

// The epilogue of one 32-column slice c0 .. c0+31 (or 16 for N = 16) of
// this thread's row.
// Row stride (elements) of the BF16 output tile staged in shared memory:
// 129 words, so that a warp writing one row per lane, or reading 32
// consecutive words of one row, touches 32 different banks.
template <int N>
constexpr int kStageStride = N + 2;

// The epilogue of one 32-column slice c0 .. c0+31 (or 16 for N = 16) of
// this thread's row (trow within the tile).  Weight gradients go straight to
// their partial; activations and gradients of activations are written as
// BF16 pairs into the shared-memory tile, stored to global memory by
// gemm_store_tile.
template <int N, int EPI, int W>
__device__ __forceinline__ void gemm_epilogue(const GemmArgs &g, long long row, int trow, int c0,
                                              const float (&v)[W], __nv_bfloat16 *stile) {
    if (row >= g.M) return;
    if (EPI == kEpiWgrad) {
        float4 *dst = reinterpret_cast<float4 *>(g.grad + (long long)blockIdx.y * g.M * N +
                                                 row * N + c0);
#pragma unroll
        for (int q = 0; q < W / 4; q++)
            dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        return;
    }
    if (EPI == kEpiWgradT) {
        float *dst = g.grad + (long long)blockIdx.y * g.M * N;
#pragma unroll
        for (int j = 0; j < W; j++) dst[(long long)(c0 + j) * g.M + row] = v[j];
        return;
    }
    __align__(16) __nv_bfloat16 o[W];
    if (EPI == kEpiHidden) {
        const float4 *bp = reinterpret_cast<const float4 *>(g.bias + c0);
#pragma unroll
        for (int q = 0; q < W / 4; q++) {
            const float4 b = __ldg(bp + q);
            o[4 * q] = __float2bfloat16(fmaxf(v[4 * q] + b.x, 0.0f));
            o[4 * q + 1] = __float2bfloat16(fmaxf(v[4 * q + 1] + b.y, 0.0f));
            o[4 * q + 2] = __float2bfloat16(fmaxf(v[4 * q + 2] + b.z, 0.0f));
            o[4 * q + 3] = __float2bfloat16(fmaxf(v[4 * q + 3] + b.w, 0.0f));
        }
    } else {  // dgrad: the ReLU mask of the activations this layer read
        __align__(16) __nv_bfloat16 pm[W];
        const int4 *src = reinterpret_cast<const int4 *>(g.mask + row * N + c0);
#pragma unroll
        for (int q = 0; q < W / 8; q++) reinterpret_cast<int4 *>(pm)[q] = src[q];
#pragma unroll
        for (int j = 0; j < W; j++)
            o[j] = __float2bfloat16(__bfloat162float(pm[j]) > 0.0f ? v[j] : 0.0f);
    }
    unsigned *t32 = reinterpret_cast<unsigned *>(stile + trow * kStageStride<N> + c0);
#pragma unroll
    for (int j = 0; j < W / 2; j++) t32[j] = reinterpret_cast<const unsigned *>(o)[j];
}

// Stores the staged 128 x N BF16 tile: row-major (each warp writes whole
// rows, 32 consecutive words per instruction) and, when asked,
// feature-major (each warp writes one feature's 128 rows as 4-byte pairs,
// 128 bytes per instruction).
template <int N>
__device__ __forceinline__ void gemm_store_tile(const GemmArgs &g, long long m0,
                                                const __nv_bfloat16 *stile) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int TW = kStageStride<N> / 2;  // words per staged row
    const unsigned *t32 = reinterpret_cast<const unsigned *>(stile);
    for (int r = warp; r < kTileM; r += kGemmThreads / 32) {
        const long long grow = m0 + r;
        if (grow >= g.M) break;
        unsigned *dst = reinterpret_cast<unsigned *>(g.out_row + grow * N);
#pragma unroll
        for (int j = lane; j < N / 2; j += 32) dst[j] = t32[r * TW + j];
    }
    if (!g.out_col) return;
    for (int c = warp; c < N; c += kGemmThreads / 32) {
#pragma unroll
        for (int p = 0; p < kTileM / 64; p++) {
            const int r = 64 * p + 2 * lane;
            const long long grow = m0 + r;
            __nv_bfloat16 *dst = g.out_col + (long long)c * g.ldc + grow;
            const __nv_bfloat16 a = stile[r * kStageStride<N> + c];
            const __nv_bfloat16 b = stile[(r + 1) * kStageStride<N> + c];
            if (grow + 1 < g.M) {
                __nv_bfloat162 pair;
                pair.x = a;
                pair.y = b;
                *reinterpret_cast<__nv_bfloat162 *>(dst) = pair;
            } else if (grow < g.M) {
                *dst = a;
            }
        }
    }
}

// C (128 x N tile) = A (tile rows) x B^T over this CTA's K range, then the
// epilogue.  blockIdx.x: row tile; blockIdx.y: K split (weight gradients).
template <int N, int EPI>
__global__ void __launch_bounds__(kGemmThreads, 2) tc_gemm(GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    GemmSmem<N> &S = *reinterpret_cast<GemmSmem<N> *>(
        smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long m0 = (long long)blockIdx.x * kTileM;
    const long kb = (long)blockIdx.y * g.k_per_split;
    const long ke = g.K < kb + g.k_per_split ? g.K : kb + g.k_per_split;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&S.tmem_base)),
                     "n"(tmem_cols<N>())
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&S.bar[0]);
        mbar_init(&S.bar[1]);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = S.tmem_base;
    const int kc = g.K < kChunkK ? (int)g.K : kChunkK;  // 64, or 16 for K = 16
    // every K range is non-empty: the host launches ceil(K / k_per_split)
    // splits
    const int nk = (int)((ke - kb + kc - 1) / kc);
    constexpr unsigned idesc = tc_idesc(N);
    auto issue = [&](int c) {
        const int s = c & 1;
        const long k0 = kb + (long)c * kc;
        stage_operand(smem_u32(S.a[s]), g.A, g.lda, m0, g.M, kTileM, k0, kc);
        stage_operand(smem_u32(S.b[s]), g.B, g.ldb, 0, N, N, k0, kc);
        cp_async_commit();
    };
    bool ok = true;
    int last = -1;  // the last chunk whose MMAs were committed
    if (nk > 0) issue(0);
    for (int c = 0; c < nk && ok; c++) {
        if (c + 1 < nk) {
            // stage (c+1)&1 was read by the MMAs of chunk c-1
            if (c >= 1) ok = cta_wait(&S.bar[(c - 1) & 1], ((c - 1) >> 1) & 1);
            if (!ok) break;
            issue(c + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        proxy_fence();  // the copies into shared memory, before the tensor core reads
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const int s = c & 1;
            const unsigned sbo = (unsigned)(kc / 8) * 128u;
            const unsigned a0 = smem_u32(S.a[s]), b0 = smem_u32(S.b[s]);
            for (int kk = 0; kk < kc / 16; kk++)
                tc_mma(tmem, smem_desc(a0 + 256u * kk, 128, sbo),
                       smem_desc(b0 + 256u * kk, 128, sbo), idesc, c > 0 || kk > 0);
            tc_commit(&S.bar[s]);
        }
        last = c;
    }
    if (ok && last >= 0) ok = cta_wait(&S.bar[last & 1], (last >> 1) & 1);
    if (!ok) {
        // status first; then let copies land (cp.async completes on its own)
        // and give the MMAs in flight (up to the last committed chunk's) one
        // more bounded wait before the columns are freed
        if (tid == 0) atomicExch(g.status, SWGPU_ETIMEOUT);
        cp_async_wait<0>();
        if (last >= 0) cta_wait(&S.bar[last & 1], (last >> 1) & 1);
    } else {
        // warp w reads TMEM lanes 32 (w % 4) .. +31 (its rows; a warp may only
        // reach its own quarter of the lanes) and half w / 4 of the columns
        tc_fence_after();
        const int quarter = warp & 3, half = warp >> 2;
        const int trow = 32 * quarter + lane;
        const long long row = m0 + trow;
        const unsigned lane_addr = tmem + ((unsigned)(32 * quarter) << 16);
        // the operand stages are free (every MMA has completed): the output
        // tile is staged there
        __nv_bfloat16 *stile = &S.a[0][0];
        static_assert(EPI == kEpiWgrad || EPI == kEpiWgradT ||
                          kTileM * kStageStride<N> * 2 <= sizeof(S.a) + sizeof(S.b),
                      "staged tile fits in the operand stages");
        if (N >= 64) {
#pragma unroll 1
            for (int c0 = half * (N / 2); c0 < (half + 1) * (N / 2); c0 += 32) {
                float v[32];
                tc_ld32(lane_addr + c0, v);
                gemm_epilogue<N, EPI, 32>(g, row, trow, c0, v, stile);
            }
        } else if (half == 0) {
            float v[16];
            tc_ld16(lane_addr, v);
            gemm_epilogue<N, EPI, 16>(g, row, trow, 0, v, stile);
        }
        if constexpr (EPI == kEpiHidden || EPI == kEpiDgrad) {
            __syncthreads();
            gemm_store_tile<N>(g, m0, stile);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "n"(tmem_cols<N>())
                     : "memory");
}

// ---- output layer (CUDA cores) --------------------------------------------

constexpr int kHeadRows = 32;  // rows per block: one warp per row, 8 warps

// y = H3 W4 + b4 for each row; the 8 columns of lane l are 8l .. 8l+7;
// w4 is the block's shared copy of W4 ([in][out], BF16).
__device__ __forceinline__ void head_forward(const __nv_bfloat16 *h, const __nv_bfloat16 *w4,
                                             const float *b4, float (&hv)[8], float (&y)[kOut]) {
    const int lane = threadIdx.x & 31;
    __align__(16) __nv_bfloat16 hb[8];
    *reinterpret_cast<int4 *>(hb) = *reinterpret_cast<const int4 *>(h + 8 * lane);
    float acc[kOut] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int j = 0; j < 8; j++) {
        hv[j] = __bfloat162float(hb[j]);
#pragma unroll
        for (int o = 0; o < kOut; o++)
            acc[o] = fmaf(hv[j], __bfloat162float(w4[(8 * lane + j) * kOut + o]), acc[o]);
    }
#pragma unroll
    for (int o = 0; o < kOut; o++) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) acc[o] += __shfl_xor_sync(0xffffffffu, acc[o], d);
        y[o] = acc[o] + b4[o];
    }
}

constexpr int kPredictRows = 64;  // rows per block of the inference head: 8 per warp

__global__ void __launch_bounds__(256) mlp_head_predict(const __nv_bfloat16 *__restrict__ h3,
                                                        const BfWeights *W, const float *params,
                                                        long long nrows, float *__restrict__ out) {
    __shared__ __nv_bfloat16 w4[kH * kOut];
    for (int i = threadIdx.x; i < kH * kOut; i += blockDim.x) w4[i] = W->w4[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = warp; i < kPredictRows; i += 8) {
        const long long r = (long long)blockIdx.x * kPredictRows + i;
        if (r >= nrows) break;
        float hv[8], y[kOut];
        head_forward(h3 + r * kH, w4, params + kOffB4, hv, y);
        if (lane < kOut) out[r * kOut + lane] = y[lane];
    }
}

// Training head: outputs, loss, dL/dy and the gradient into layer 3,
// dz3 = (dy W4^T) * relu'(h3), stored row-major and feature-major; the
// output layer's own gradients (W4, b4) are summed per block.  loss =
// mean over rows of w_d (y0 - t0)^2 + w_a (y1 - t1)^2 + w_e rho(|y0 - t0| - y2),
// rho the pinball loss of the kQuantile quantile, so that y2 learns that
// quantile of the depth output's absolute error (taken as a constant).
__global__ void __launch_bounds__(256) mlp_head_train(
    const __nv_bfloat16 *__restrict__ h3, const BfWeights *W, const float *params,
    const float *__restrict__ targets, const long long *__restrict__ row_of, long long nrows,
    long long Bp, float w_d, float w_a, float w_e, float *__restrict__ y_out,
    __nv_bfloat16 *__restrict__ dz_row, __nv_bfloat16 *__restrict__ dz_col,
    float *__restrict__ grad, float *__restrict__ loss) {
    // rows padded by 16 bytes: the feature-major pass reads down a column
    __shared__ __align__(16) __nv_bfloat16 tile[kHeadRows][kH + 8];
    __shared__ float gw4[kH * kOut];
    __shared__ __nv_bfloat16 w4[kH * kOut];
    __shared__ float gb4[kOut];
    __shared__ float lsum;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kH * kOut; i += blockDim.x) {
        gw4[i] = 0.f;
        w4[i] = W->w4[i];
    }
    if (threadIdx.x < kOut) gb4[threadIdx.x] = 0.f;
    if (threadIdx.x == 0) lsum = 0.f;
    __syncthreads();
    const float inv_b = 1.0f / (float)nrows;
    const long long rb = (long long)blockIdx.x * kHeadRows;
    // this lane's share of the output layer's gradients over the warp's rows
    float gw[8][kOut], gb[kOut] = {0.f, 0.f, 0.f}, ls = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
        for (int o = 0; o < kOut; o++) gw[j][o] = 0.f;
    for (int i = warp; i < kHeadRows; i += 8) {
        const long long r = rb + i;
        __align__(16) __nv_bfloat16 dz[8];
        if (r < nrows) {
            float hv[8], y[kOut];
            head_forward(h3 + r * kH, w4, params + kOffB4, hv, y);
            const float *t = targets + row_of[r] * kTargets;
            const float e0 = y[0] - t[0], e1 = y[1] - t[1];
            const float u = fabsf(e0) - y[2];
            const float pin = u >= 0.f ? kQuantile * u : (kQuantile - 1.f) * u;
            const float d0 = 2.f * w_d * e0 * inv_b, d1 = 2.f * w_a * e1 * inv_b,
                        d2 = w_e * (u < 0.f ? 1.f - kQuantile : -kQuantile) * inv_b;
            if (lane == 0) {
                y_out[r * kOut] = y[0];
                y_out[r * kOut + 1] = y[1];
                y_out[r * kOut + 2] = y[2];
                ls += (w_d * e0 * e0 + w_a * e1 * e1 + w_e * pin) * inv_b;
                gb[0] += d0;
                gb[1] += d1;
                gb[2] += d2;
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int c = 8 * lane + j;
                const float w0 = __bfloat162float(w4[c * kOut]);
                const float w1 = __bfloat162float(w4[c * kOut + 1]);
                const float w2 = __bfloat162float(w4[c * kOut + 2]);
                const float g = fmaf(d0, w0, fmaf(d1, w1, d2 * w2));
                dz[j] = __float2bfloat16(hv[j] > 0.f ? g : 0.f);
                gw[j][0] += hv[j] * d0;
                gw[j][1] += hv[j] * d1;
                gw[j][2] += hv[j] * d2;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) dz[j] = __float2bfloat16(0.f);
        }
        *reinterpret_cast<int4 *>(&tile[i][8 * lane]) = *reinterpret_cast<const int4 *>(dz);
    }
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
        for (int o = 0; o < kOut; o++) atomicAdd(&gw4[(8 * lane + j) * kOut + o], gw[j][o]);
    if (lane == 0) {
        atomicAdd(&lsum, ls);
#pragma unroll
        for (int o = 0; o < kOut; o++) atomicAdd(&gb4[o], gb[o]);
    }
    __syncthreads();
    // row-major rows of the block (rows up to Bp: the padding is zero)
    for (int v = threadIdx.x; v < kHeadRows * (kH / 8); v += blockDim.x) {
        const int i = v / (kH / 8), q = v % (kH / 8);
        const long long r = rb + i;
        if (r < Bp)
            reinterpret_cast<int4 *>(dz_row + r * kH)[q] =
                reinterpret_cast<const int4 *>(&tile[i][0])[q];
    }
    // feature-major: 32 consecutive rows of each feature
    for (int v = threadIdx.x; v < kH * kHeadRows; v += blockDim.x) {
        const int c = v / kHeadRows, i = v % kHeadRows;
        const long long r = rb + i;
        if (r < Bp) dz_col[(long long)c * Bp + r] = tile[i][c];
    }
    for (int i = threadIdx.x; i < kH * kOut; i += blockDim.x)
        atomicAdd(&grad[kOffW4 + i], gw4[i]);
    if (threadIdx.x < kOut) atomicAdd(&grad[kOffB4 + threadIdx.x], gb4[threadIdx.x]);
    if (threadIdx.x == 0) atomicAdd(loss, lsum);
}

// Bias gradients: sum over the batch of each feature-major gradient row,
// each row split over gridDim.y blocks (8 rows per thread and step, as one
// 16-byte load).
__global__ void __launch_bounds__(256) mlp_bias_grad(const __nv_bfloat16 *__restrict__ dz_col,
                                                     long long Bp, int nfeat,
                                                     float *__restrict__ gb) {
    const int f = blockIdx.x;
    if (f >= nfeat) return;
    float s = 0.f;
    const int4 *p = reinterpret_cast<const int4 *>(dz_col + (long long)f * Bp);
    const long long nv = Bp / 8;  // Bp is a multiple of the 128-row tile
    for (long long q = blockIdx.y * (long long)blockDim.x + threadIdx.x; q < nv;
         q += (long long)gridDim.y * blockDim.x) {
        const int4 u = p[q];
        const __nv_bfloat16 *b = reinterpret_cast<const __nv_bfloat16 *>(&u);
#pragma unroll
        for (int j = 0; j < 8; j++) s += __bfloat162float(b[j]);
    }
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int t = 128; t > 0; t >>= 1) {
        if ((int)threadIdx.x < t) sh[threadIdx.x] += sh[threadIdx.x + t];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(&gb[f], sh[0]);
}

// Weight gradient from its per-split partials: out[i] += sum over s of
// part[s][i] (the splits of the batch, in a fixed order).
__global__ void __launch_bounds__(256) mlp_sum_partials(const float *__restrict__ part,
                                                        int splits, long n,
                                                        float *__restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // four independent running sums (loads in flight together), fixed order
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = 0;
    for (; k + 4 <= splits; k += 4) {
        s0 += part[(long)k * n + i];
        s1 += part[(long)(k + 1) * n + i];
        s2 += part[(long)(k + 2) * n + i];
        s3 += part[(long)(k + 3) * n + i];
    }
    for (; k < splits; k++) s0 += part[(long)k * n + i];
    out[i] += (s0 + s1) + (s2 + s3);
}

// ---- weights ----------------------------------------------------------------

__global__ void mlp_pack_weights(const float *__restrict__ p, BfWeights *W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kH * kH) {
        const int in = i / kH, out = i % kH;
        const __nv_bfloat16 a = __float2bfloat16(p[kOffW2 + i]);
        const __nv_bfloat16 b = __float2bfloat16(p[kOffW3 + i]);
        W->w2[i] = a;
        W->w3[i] = b;
        W->wt2[out * kH + in] = a;
        W->wt3[out * kH + in] = b;
    }
    if (i < kF * kH) {
        const int in = i / kH, out = i % kH;
        W->wt1[out * kF + in] = __float2bfloat16(p[kOffW1 + i]);
    }
    if (i < kH * kOut) W->w4[i] = __float2bfloat16(p[kOffW4 + i]);
}

__global__ void mlp_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                         float *__restrict__ v, long n, float lr, float b1, float b2, float eps,
                         float c1, float c2) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// ---- host side ----------------------------------------------------------------

struct Buffers {  // one batch of rows (training) or one chunk (inference)
    long long cap = 0;  // rows (a multiple of kTileM)
    bool train = false;
    __nv_bfloat16 *xr = nullptr, *xc = nullptr;
    __nv_bfloat16 *h1 = nullptr, *h2 = nullptr, *h3 = nullptr;     // row-major
    __nv_bfloat16 *h1c = nullptr, *h2c = nullptr;                  // feature-major
    __nv_bfloat16 *d3 = nullptr, *d2 = nullptr, *d3c = nullptr, *d2c = nullptr, *d1c = nullptr;
    long long *row_of = nullptr;
    float *y = nullptr;
    float *part = nullptr;  // weight-gradient partials [splits][256 x 256]
};

// Batch rows per K split of the weight-gradient GEMMs.
constexpr long kWgradRows = 512;

struct Mlp {
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    float *params = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    BfWeights *w = nullptr;
    float *mu = nullptr, *isd = nullptr;
    float *scen = nullptr, *tri = nullptr, *targets = nullptr;
    long long S = 0, N = 0;
    Buffers buf;
    long long *rows = nullptr;
    long long rows_cap = 0;
    float *loss = nullptr;
    int *status = nullptr;   // device-side failure of a tensor-core kernel
    bool unusable = false;   // a kernel reported SWGPU_ETIMEOUT
    long long adam_t = 0;
    std::vector<void *> allocs, data_allocs, buf_allocs;
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
int malloc_dev(Mlp *m, T **p, size_t count, std::vector<void *> *owner = nullptr) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
    if (e != cudaSuccess)
        return mfail(m, SWGPU_ENOMEM, "cudaMalloc %zu bytes: %s", count * sizeof(T),
                     cudaGetErrorString(e));
    (owner ? *owner : m->allocs).push_back(q);
    *p = static_cast<T *>(q);
    return SWGPU_OK;
}

void free_list(std::vector<void *> &v) {
    for (void *p : v) cudaFree(p);
    v.clear();
}

// Row buffers for `rows` rows (rounded up to the tile), reallocated only
// when they grow or when training needs the feature-major copies.
int ensure_buffers(Mlp *m, long long rows, bool train, std::vector<void *> &owned) {
    const long long cap = (rows + kTileM - 1) / kTileM * kTileM;
    Buffers &B = m->buf;
    if (cap <= B.cap && (B.train || !train)) return SWGPU_OK;
    MCK(cudaStreamSynchronize(m->stream));
    free_list(owned);
    B = Buffers{};
    int rc;
    const size_t hr = (size_t)cap * kH;
    if ((rc = malloc_dev(m, &B.xr, (size_t)cap * kF, &owned)) ||
        (rc = malloc_dev(m, &B.h1, hr, &owned)) || (rc = malloc_dev(m, &B.h2, hr, &owned)) ||
        (rc = malloc_dev(m, &B.h3, hr, &owned)) || (rc = malloc_dev(m, &B.y, (size_t)cap * kOut, &owned)))
        return rc;
    if (train) {
        if ((rc = malloc_dev(m, &B.xc, (size_t)cap * kF, &owned)) ||
            (rc = malloc_dev(m, &B.h1c, hr, &owned)) || (rc = malloc_dev(m, &B.h2c, hr, &owned)) ||
            (rc = malloc_dev(m, &B.d3, hr, &owned)) || (rc = malloc_dev(m, &B.d2, hr, &owned)) ||
            (rc = malloc_dev(m, &B.d3c, hr, &owned)) || (rc = malloc_dev(m, &B.d2c, hr, &owned)) ||
            (rc = malloc_dev(m, &B.d1c, hr, &owned)) ||
            (rc = malloc_dev(m, &B.row_of, (size_t)cap, &owned)) ||
            (rc = malloc_dev(m, &B.part, (size_t)((cap + kWgradRows - 1) / kWgradRows) * kH * kH,
                             &owned)))
            return rc;
    }
    B.cap = cap;
    B.train = train;
    return SWGPU_OK;
}

template <int N, int EPI>
int launch_gemm(Mlp *m, const GemmArgs &g, int splits) {
    const unsigned grid_x = (unsigned)((g.M + kTileM - 1) / kTileM);
    const size_t smem = sizeof(GemmSmem<N>) + 1024;
    tc_gemm<N, EPI><<<dim3(grid_x, (unsigned)splits), kGemmThreads, smem, m->stream>>>(g);
    MCK(cudaGetLastError());
    return SWGPU_OK;
}

template <int N, int EPI>
cudaError_t gemm_attr() {
    return cudaFuncSetAttribute(tc_gemm<N, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(GemmSmem<N>) + 1024));
}

FeatureTables tables(const Mlp *m) {
    return FeatureTables{m->scen, m->tri, m->mu, m->isd, m->N};
}

GemmArgs gemm_args(Mlp *m, const __nv_bfloat16 *A, long lda, const __nv_bfloat16 *B, long ldb,
                   long long M, long K) {
    GemmArgs g{};
    g.A = A;
    g.lda = lda;
    g.B = B;
    g.ldb = ldb;
    g.M = M;
    g.K = K;
    g.k_per_split = K;
    g.status = m->status;
    return g;
}

// Forward pass of Bp rows already in buf.xr (feature-major copies when train).
int forward(Mlp *m, long long Bp, bool train) {
    Buffers &B = m->buf;
    const BfWeights *W = m->w;
    int rc;
    GemmArgs g = gemm_args(m, B.xr, kF, W->wt1, kF, Bp, kF);
    g.bias = m->params + kOffB1;
    g.out_row = B.h1;
    g.out_col = train ? B.h1c : nullptr;
    g.ldc = Bp;
    if ((rc = launch_gemm<kH, kEpiHidden>(m, g, 1))) return rc;
    g = gemm_args(m, B.h1, kH, W->wt2, kH, Bp, kH);
    g.bias = m->params + kOffB2;
    g.out_row = B.h2;
    g.out_col = train ? B.h2c : nullptr;
    g.ldc = Bp;
    if ((rc = launch_gemm<kH, kEpiHidden>(m, g, 1))) return rc;
    g = gemm_args(m, B.h2, kH, W->wt3, kH, Bp, kH);
    g.bias = m->params + kOffB3;
    g.out_row = B.h3;
    g.out_col = nullptr;
    if ((rc = launch_gemm<kH, kEpiHidden>(m, g, 1))) return rc;
    return SWGPU_OK;
}

// Forward, backward and the gradient vector of nrows rows (Bp padded).
int batch_gradients(Mlp *m, const long long *d_rows, unsigned long long seed, long long nrows,
                    float w_d, float w_a, float w_e) {
    const long long Bp = (nrows + kTileM - 1) / kTileM * kTileM;
    int rc = ensure_buffers(m, nrows, true, m->buf_allocs);
    if (rc) return rc;
    Buffers &B = m->buf;
    const BfWeights *W = m->w;
    MCK(cudaMemsetAsync(m->grad, 0, sizeof(float) * kNumParams, m->stream));
    MCK(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
    mlp_features<<<(unsigned)((Bp + 255) / 256), 256, 0, m->stream>>>(
        tables(m), d_rows, seed, d_rows ? 0 : m->S * m->N, 0, nrows, Bp, B.xr, B.xc, B.row_of);
    if ((rc = forward(m, Bp, true))) return rc;
    mlp_head_train<<<(unsigned)((Bp + kHeadRows - 1) / kHeadRows), 256, 0, m->stream>>>(
        B.h3, W, m->params, m->targets, B.row_of, nrows, Bp, w_d, w_a, w_e, B.y, B.d3, B.d3c,
        m->grad, m->loss);
    MCK(cudaGetLastError());
    // weight gradients: one partial per split of the batch, then their sum
    const int splits = (int)((Bp + kWgradRows - 1) / kWgradRows);
    const dim3 bias_grid(kH, 16);
    auto sum_parts = [&](long n, long off) {
        mlp_sum_partials<<<(unsigned)((n + 255) / 256), 256, 0, m->stream>>>(B.part, splits, n,
                                                                            m->grad + off);
    };
    // layer 3: gW3 = H2^T dZ3 (in x out), gb3; dZ2 = (dZ3 W3^T) * relu'(H2)
    GemmArgs g = gemm_args(m, B.h2c, Bp, B.d3c, Bp, kH, Bp);
    g.k_per_split = kWgradRows;
    g.grad = B.part;
    if ((rc = launch_gemm<kH, kEpiWgrad>(m, g, splits))) return rc;
    sum_parts((long)kH * kH, kOffW3);
    mlp_bias_grad<<<bias_grid, 256, 0, m->stream>>>(B.d3c, Bp, kH, m->grad + kOffB3);
    g = gemm_args(m, B.d3, kH, W->w3, kH, Bp, kH);
    g.mask = B.h2;
    g.out_row = B.d2;
    g.out_col = B.d2c;
    g.ldc = Bp;
    if ((rc = launch_gemm<kH, kEpiDgrad>(m, g, 1))) return rc;
    // layer 2: gW2 = H1^T dZ2, gb2; dZ1 = (dZ2 W2^T) * relu'(H1)
    g = gemm_args(m, B.h1c, Bp, B.d2c, Bp, kH, Bp);
    g.k_per_split = kWgradRows;
    g.grad = B.part;
    if ((rc = launch_gemm<kH, kEpiWgrad>(m, g, splits))) return rc;
    sum_parts((long)kH * kH, kOffW2);
    mlp_bias_grad<<<bias_grid, 256, 0, m->stream>>>(B.d2c, Bp, kH, m->grad + kOffB2);
    g = gemm_args(m, B.d2, kH, W->w2, kH, Bp, kH);
    g.mask = B.h1;
    g.out_row = B.d3;  // dZ1 row-major is not needed again: B.d3 is free
    g.out_col = B.d1c;
    g.ldc = Bp;
    if ((rc = launch_gemm<kH, kEpiDgrad>(m, g, 1))) return rc;
    // layer 1: gW1^T = dZ1^T X (out x in), stored transposed into W1 [in][out]; gb1
    g = gemm_args(m, B.d1c, Bp, B.xc, Bp, kH, Bp);
    g.k_per_split = kWgradRows;
    g.grad = B.part;
    if ((rc = launch_gemm<kF, kEpiWgradT>(m, g, splits))) return rc;
    sum_parts((long)kF * kH, kOffW1);
    mlp_bias_grad<<<bias_grid, 256, 0, m->stream>>>(B.d1c, Bp, kH, m->grad + kOffB1);
    MCK(cudaGetLastError());
    return SWGPU_OK;
}

int read_status(Mlp *m, const char *what) {
    int st = 0;
    MCK(cudaMemcpy(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) {
        if (st == SWGPU_ETIMEOUT) m->unusable = true;
        return mfail(m, st, "%s: a tensor-core wait ran out; destroy the handle", what);
    }
    return SWGPU_OK;
}

int usable(Mlp *m, const char *what) {
    if (m && m->unusable)
        return mfail(m, SWGPU_ETIMEOUT,
                     "%s: handle unusable after a tensor-core wait ran out; destroy it", what);
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
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, m->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = gemm_attr<kH, kEpiHidden>();
    if (e == cudaSuccess) e = gemm_attr<kH, kEpiDgrad>();
    if (e == cudaSuccess) e = gemm_attr<kH, kEpiWgrad>();
    if (e == cudaSuccess) e = gemm_attr<kF, kEpiWgradT>();
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
        free_list(m->allocs);
        delete m;
        return rc;
    }
    e = cudaMemcpy(m->params, params, sizeof(float) * kNumParams, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(m->mu, feature_mean, sizeof(float) * kF, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(m->isd, feature_inv_std, sizeof(float) * kF, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->adam_m, 0, sizeof(float) * kNumParams);
    if (e == cudaSuccess) e = cudaMemset(m->adam_v, 0, sizeof(float) * kNumParams);
    if (e == cudaSuccess) e = cudaMemset(m->status, 0, sizeof(int));
    if (e == cudaSuccess) {
        mlp_pack_weights<<<(kH * kH + 255) / 256, 256, 0, m->stream>>>(m->params, m->w);
        e = cudaStreamSynchronize(m->stream);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        rc = mfail(m, SWGPU_ECUDA, "swgpu_mlp_create: %s", cudaGetErrorString(e));
        free_list(m->allocs);
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
    free_list(m->data_allocs);
    free_list(m->buf_allocs);
    free_list(m->allocs);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return SWGPU_OK;
}

const char *swgpu_mlp_last_error(void *handle) {
    Mlp *m = static_cast<Mlp *>(handle);
    return m ? m->err.c_str() : g_mlp_error.c_str();
}

int swgpu_mlp_set_data(void *handle, const float *tri, int64_t ntri, const float *scen,
                       int64_t nscen, const float *targets) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || !tri || !scen || ntri <= 0 || nscen <= 0)
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_set_data: bad argument");
    if (int rc = usable(m, "swgpu_mlp_set_data")) return rc;
    if ((long long)ntri * nscen >= (1LL << 40))
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_set_data: too many rows");
    MCK(cudaStreamSynchronize(m->stream));
    free_list(m->data_allocs);
    m->tri = m->scen = m->targets = nullptr;
    m->N = m->S = 0;
    int rc;
    if ((rc = malloc_dev(m, &m->tri, (size_t)ntri * kTri, &m->data_allocs)) ||
        (rc = malloc_dev(m, &m->scen, (size_t)nscen * kParams, &m->data_allocs)))
        return rc;
    MCK(cudaMemcpy(m->tri, tri, sizeof(float) * kTri * ntri, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->scen, scen, sizeof(float) * kParams * nscen, cudaMemcpyHostToDevice));
    if (targets) {
        if ((rc = malloc_dev(m, &m->targets, (size_t)ntri * nscen * kTargets, &m->data_allocs)))
            return rc;
        MCK(cudaMemcpy(m->targets, targets, sizeof(float) * kTargets * ntri * nscen,
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
    if (int rc = usable(m, "swgpu_mlp_predict")) return rc;
    // chunks of up to 2^21 rows through row buffers (1 GB per activation)
    const long long chunk = std::min<long long>(nrows, 1LL << 21);
    int rc = ensure_buffers(m, chunk, false, m->buf_allocs);
    if (rc) return rc;
    cudaEvent_t a, b;
    MCK(cudaEventCreate(&a));
    MCK(cudaEventCreate(&b));
    MCK(cudaEventRecord(a, m->stream));
    for (long long r0 = 0; r0 < nrows; r0 += chunk) {
        const long long n = std::min(chunk, nrows - r0);
        const long long Bp = (n + kTileM - 1) / kTileM * kTileM;
        mlp_features<<<(unsigned)((Bp + 255) / 256), 256, 0, m->stream>>>(
            tables(m), nullptr, 0, 0, row0 + r0, n, Bp, m->buf.xr, nullptr, nullptr);
        if ((rc = forward(m, Bp, false))) return rc;
        mlp_head_predict<<<(unsigned)((n + kPredictRows - 1) / kPredictRows), 256, 0, m->stream>>>(
            m->buf.h3, m->w, m->params, n, out_device + r0 * kOut);
        MCK(cudaGetLastError());
    }
    MCK(cudaEventRecord(b, m->stream));
    MCK(cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if ((rc = read_status(m, "swgpu_mlp_predict"))) return rc;
    if (elapsed_ms) *elapsed_ms = ms;
    return SWGPU_OK;
}

int swgpu_mlp_gradients(void *handle, const int64_t *rows, int64_t nrows, float w_depth,
                        float w_arrival, float w_error, float *outputs, float *grad,
                        float *loss) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || !rows || nrows <= 0 || !m->targets)
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_gradients: bad argument or no targets");
    if (int rc = usable(m, "swgpu_mlp_gradients")) return rc;
    for (int64_t i = 0; i < nrows; i++)
        if (rows[i] < 0 || rows[i] >= m->S * m->N)
            return mfail(m, SWGPU_EINVAL, "swgpu_mlp_gradients: row %lld out of range",
                         (long long)rows[i]);
    int rc;
    if (nrows > m->rows_cap) {
        if ((rc = malloc_dev(m, &m->rows, (size_t)nrows))) return rc;
        m->rows_cap = nrows;
    }
    MCK(cudaMemcpyAsync(m->rows, rows, sizeof(long long) * nrows, cudaMemcpyHostToDevice,
                        m->stream));
    if ((rc = batch_gradients(m, m->rows, 0, nrows, w_depth, w_arrival, w_error))) return rc;
    if (outputs)
        MCK(cudaMemcpyAsync(outputs, m->buf.y, sizeof(float) * kOut * nrows,
                            cudaMemcpyDeviceToHost, m->stream));
    if (grad)
        MCK(cudaMemcpyAsync(grad, m->grad, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost,
                            m->stream));
    if (loss)
        MCK(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return read_status(m, "swgpu_mlp_gradients");
}

int swgpu_mlp_train(void *handle, int steps, int64_t batch, uint64_t seed, float lr,
                    float w_depth, float w_arrival, float w_error, float *last_loss,
                    float *elapsed_ms) {
    Mlp *m = static_cast<Mlp *>(handle);
    if (!m || steps <= 0 || batch <= 0 || !m->targets)
        return mfail(m, SWGPU_EINVAL, "swgpu_mlp_train: bad argument or no targets");
    if (int rc = usable(m, "swgpu_mlp_train")) return rc;
    cudaEvent_t a, b;
    MCK(cudaEventCreate(&a));
    MCK(cudaEventCreate(&b));
    MCK(cudaEventRecord(a, m->stream));
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < steps; s++) {
        const unsigned long long step_seed = seed * 0x9E3779B97F4A7C15ull + (unsigned)s;
        int rc = batch_gradients(m, nullptr, step_seed, batch, w_depth, w_arrival, w_error);
        if (rc) return rc;
        m->adam_t++;
        const float c1 = 1.f / (1.f - powf(b1, (float)m->adam_t));
        const float c2 = 1.f / (1.f - powf(b2, (float)m->adam_t));
        mlp_adam<<<(unsigned)((kNumParams + 255) / 256), 256, 0, m->stream>>>(
            m->params, m->grad, m->adam_m, m->adam_v, kNumParams, lr, b1, b2, 1e-8f, c1, c2);
        mlp_pack_weights<<<(kH * kH + 255) / 256, 256, 0, m->stream>>>(m->params, m->w);
    }
    MCK(cudaGetLastError());
    MCK(cudaEventRecord(b, m->stream));
    MCK(cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (int rc = read_status(m, "swgpu_mlp_train")) return rc;
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

int swgpu_mlp_num_params(void) { return (int)kNumParams; }

}  // extern "C"
