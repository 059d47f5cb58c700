// swgpu_noalloc.cu -- water volume without any device allocation.
//
// swgpu_mass computes the volume sum(area * (stage - elevation)) of a
// handle's state with a block-partials scratch buffer that swgpu_create
// allocated.  Some callers cannot allocate device memory at the point where
// they need the volume: code running while a CUDA stream is being captured
// into a graph (cudaMalloc is not capturable), code whose device memory is
// handed out by a pool it does not control, and time-critical loops that
// must not take cudaMalloc's implicit device synchronisation.  They hold the
// arrays already (their own device buffers) and want only the reduction.
//
// swgpu_water_volume_noalloc serves them: the caller passes device pointers
// to its inputs and to its one-double output; the scratch is a file-scope
// __device__ array of kNoAllocMaxPartials doubles (128 KiB) that every GPU
// loading this library holds until the process exits.  One partial per
// 256-element block limits a call to kNoAllocMaxElements = 4,194,304
// elements; larger sizes are rejected with SWGPU_EINVAL.  The arithmetic and
// the reduction order (256-element block sums in a fixed tree, then one block
// summing the partials) are those of swgpu_mass on an FP64 handle, so given
// that handle's own centroid arrays, in its triangle order, the two results
// are bit-identical.  (A mixed-precision handle's swgpu_mass sums area times
// its FP64 depth instead of stage minus bed.)
#include <cstdio>
#include <mutex>

#include "swgpu_internal.cuh"

namespace swgpu {
void record_global_error(const char *message);  // swgpu_api.cu
}

namespace {

constexpr int kNoAllocBlock = 256;
constexpr long long kNoAllocMaxPartials = 16384;
constexpr long long kNoAllocMaxElements = kNoAllocMaxPartials * kNoAllocBlock;

// Shared by every call on a device; holds the last call's partial sums.
static __device__ __align__(256) double g_volume_partials[kNoAllocMaxPartials];

__global__ void __launch_bounds__(kNoAllocBlock)
    volume_partials_noalloc(const double *__restrict__ areas, const double *__restrict__ stage,
                            const double *__restrict__ elevation, int n,
                            double *__restrict__ partials) {
    __shared__ double sh[kNoAllocBlock];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    sh[threadIdx.x] = k < n ? areas[k] * (stage[k] - elevation[k]) : 0.0;
    __syncthreads();
    for (int s = kNoAllocBlock / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kNoAllocBlock)
    volume_final_noalloc(const double *__restrict__ partials, int nblocks,
                         double *__restrict__ out) {
    __shared__ double sh[kNoAllocBlock];
    double s = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) s += partials[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int t = kNoAllocBlock / 2; t > 0; t >>= 1) {
        if ((int)threadIdx.x < t) sh[threadIdx.x] += sh[threadIdx.x + t];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// Device address of g_volume_partials per device, looked up once per device
// with that device current.  In host code the symbol's name is a host-side
// stand-in, not a device address, so kernels only ever receive this pointer.
// The address belongs to the device's primary context as it was at the
// first call: a cudaDeviceReset after that call is not supported (the
// library's module, and the array, are loaded again in the new context).
struct ScratchSlot {
    int device;
    double *ptr;
};
std::mutex g_scratch_mutex;
ScratchSlot g_scratch_slots[64];
int g_scratch_count = 0;

int scratch_for_current_device(double **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof msg, "swgpu_water_volume_noalloc: cudaGetDevice: %s",
                 cudaGetErrorString(e));
        swgpu::record_global_error(msg);
        return SWGPU_ECUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    for (int i = 0; i < g_scratch_count; i++) {
        if (g_scratch_slots[i].device == dev) {
            *out = g_scratch_slots[i].ptr;
            return SWGPU_OK;
        }
    }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_volume_partials);
    if (e != cudaSuccess || p == nullptr) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "swgpu_water_volume_noalloc: cudaGetSymbolAddress on device %d: %s", dev,
                 cudaGetErrorString(e));
        swgpu::record_global_error(msg);
        return SWGPU_ECUDA;
    }
    if (g_scratch_count < (int)(sizeof g_scratch_slots / sizeof g_scratch_slots[0]))
        g_scratch_slots[g_scratch_count++] = {dev, static_cast<double *>(p)};
    *out = static_cast<double *>(p);
    return SWGPU_OK;
}

}  // namespace

extern "C" int swgpu_water_volume_noalloc(const double *areas, const double *stage,
                                          const double *elevation, int64_t n, double *volume,
                                          void *stream) {
    if (!areas || !stage || !elevation || !volume) {
        swgpu::record_global_error("swgpu_water_volume_noalloc: null pointer argument");
        return SWGPU_EINVAL;
    }
    if (n <= 0 || n > kNoAllocMaxElements) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "swgpu_water_volume_noalloc: n = %lld outside 1..%lld (the static scratch "
                 "holds %lld block partials of %d elements)",
                 (long long)n, kNoAllocMaxElements, kNoAllocMaxPartials, kNoAllocBlock);
        swgpu::record_global_error(msg);
        return SWGPU_EINVAL;
    }
    // an error left by the caller's earlier work is reported as such and left
    // in place, not taken for this call's launch failure
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "swgpu_water_volume_noalloc: a CUDA error was already pending before the "
                 "call (%s); nothing launched",
                 cudaGetErrorString(pending));
        swgpu::record_global_error(msg);
        return SWGPU_ECUDA;
    }
    double *partials = nullptr;
    int rc = scratch_for_current_device(&partials);
    if (rc != SWGPU_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nblocks = (int)((n + kNoAllocBlock - 1) / kNoAllocBlock);
    // every partial the final pass reads is written by this call first, so
    // nothing left in the scratch by an earlier call needs clearing
    volume_partials_noalloc<<<nblocks, kNoAllocBlock, 0, st>>>(areas, stage, elevation, (int)n,
                                                                partials);
    volume_final_noalloc<<<1, kNoAllocBlock, 0, st>>>(partials, nblocks, volume);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof msg, "swgpu_water_volume_noalloc: launch: %s", cudaGetErrorString(e));
        swgpu::record_global_error(msg);
        return SWGPU_ECUDA;
    }
    return SWGPU_OK;
}
