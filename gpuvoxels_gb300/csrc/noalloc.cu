// Centre of mass without any device allocation.
//
// Who needs this: callers that cannot call cudaMalloc.  A plugin that runs
// inside another framework's process often finds all device memory reserved by
// that framework's caching allocator or pool, so a cudaMalloc of its own fails
// or fragments the pool; a real-time control loop cannot take cudaMalloc's
// implicit device synchronisation and unbounded latency; a service that admits
// work against an HBM budget cannot have allocations it does not account for.
// They pass device inputs and a device output; the two-pass reduction's
// per-block partial sums live in a fixed scratch array compiled into this
// library.
//
// The scratch array holds kNoAllocBlocks x 4 doubles (64 KiB).  Every GPU
// that loads the library keeps it until the process exits.  All calls share
// it and it keeps the previous call's contents: every partial the second pass
// reads is written by the first pass of the same call, so nothing has to be
// cleared, but calls that overlap on the GPU (different streams, or different
// host threads on one device) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/gpuvoxels_gb300.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 8;
constexpr int kNoAllocBlocks = 2048;
constexpr int64_t kNoAllocMaxPoints = (int64_t)kNoAllocBlocks * kNoAllocThreads * kNoAllocPerThread;   // 4,194,304

static __device__ __align__(256) double g_noalloc_partials[kNoAllocBlocks * 4];

// Each block sums its points (mass*x, mass*y, mass*z, mass) in a fixed order.
__global__ void k_com_partials(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                               const float* __restrict__ mass, int64_t n, double* partials) {
    __shared__ double red[4][kNoAllocThreads];
    double a[4] = {0, 0, 0, 0};
    const int64_t base = (int64_t)blockIdx.x * kNoAllocThreads * kNoAllocPerThread;
    for (int k = 0; k < kNoAllocPerThread; k++) {
        const int64_t i = base + (int64_t)k * kNoAllocThreads + threadIdx.x;
        if (i < n) {
            const double w = mass[i];
            a[0] += x[i] * w; a[1] += y[i] * w; a[2] += z[i] * w; a[3] += w;
        }
    }
    for (int j = 0; j < 4; j++) red[j][threadIdx.x] = a[j];
    __syncthreads();
    for (int s = kNoAllocThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int j = 0; j < 4; j++) red[j][threadIdx.x] += red[j][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 4) partials[(size_t)blockIdx.x * 4 + threadIdx.x] = red[threadIdx.x][0];
}

// One block folds the partials in block order and writes (cx, cy, cz, total mass).
__global__ void k_com_finish(const double* __restrict__ partials, int nblocks, double* out4) {
    __shared__ double red[4][kNoAllocThreads];
    double a[4] = {0, 0, 0, 0};
    for (int b = threadIdx.x; b < nblocks; b += kNoAllocThreads)
        for (int j = 0; j < 4; j++) a[j] += partials[(size_t)b * 4 + j];
    for (int j = 0; j < 4; j++) red[j][threadIdx.x] = a[j];
    __syncthreads();
    for (int s = kNoAllocThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int j = 0; j < 4; j++) red[j][threadIdx.x] += red[j][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double m = red[3][0];
        out4[0] = m == 0 ? 0.0 : red[0][0] / m;
        out4[1] = m == 0 ? 0.0 : red[1][0] / m;
        out4[2] = m == 0 ? 0.0 : red[2][0] / m;
        out4[3] = m;
    }
}

// Device address of the scratch array, resolved once per device with that device current and
// kept for the life of the process (a cudaDeviceReset of that device invalidates it).
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch[kMaxDevices] = {};

}  // namespace

extern "C" int vx3_center_of_mass_noalloc(const double* x, const double* y, const double* z, const float* mass, int64_t n,
                                          double* out4, void* stream) {
    if (!x || !y || !z || !mass || !out4 || n < 0) return VX3_E_ARG;
    if (n > kNoAllocMaxPoints) return VX3_E_LIMIT;   // beyond the fixed scratch: 4,194,304 points at most
    // an error already pending on this thread belongs to the caller: leave it for them to
    // read, launch nothing, so that the status below speaks only of this call's launches
    if (cudaPeekAtLastError() != cudaSuccess) return VX3_E_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return VX3_E_CUDA;
    double* scratch = nullptr;
    {
        // set-up, once per device, with that device current: the device address of the
        // scratch array (the array's name in host code is not a device address)
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) return VX3_E_CUDA;
            g_scratch[dev] = p;
        }
        scratch = (double*)g_scratch[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int nblocks = n == 0 ? 1 : (int)((n + (int64_t)kNoAllocThreads * kNoAllocPerThread - 1) / ((int64_t)kNoAllocThreads * kNoAllocPerThread));
    k_com_partials<<<nblocks, kNoAllocThreads, 0, s>>>(x, y, z, mass, n, scratch);
    if (cudaGetLastError() != cudaSuccess) return VX3_E_CUDA;
    k_com_finish<<<1, kNoAllocThreads, 0, s>>>(scratch, nblocks, out4);
    return cudaGetLastError() == cudaSuccess ? VX3_OK : VX3_E_CUDA;
}

static_assert(kNoAllocMaxPoints == VX3_NOALLOC_MAX_POINTS, "header limit and scratch size disagree");
