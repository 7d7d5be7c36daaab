// natrix_residual_noalloc: the pressure-residual reduction for callers that
// cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at all: code that runs inside another
// framework's memory pool, a plugin that must not touch the allocator while
// a CUDA graph is being captured elsewhere, or embedded hosts with a fixed
// memory budget.  natrix_residual needs a per-handle block of partial sums
// that natrix_create allocates; this variant keeps that scratch in a
// file-scope __device__ array instead, so it allocates nothing: the caller
// passes its own device buffers for the inputs and the 5-double output.
//
// The array is sized for grids of up to NATRIX_NOALLOC_MAX_CELLS cells (see
// include/natrix.h) and stays resident on every GPU that loads the library
// until the process exits.  All calls share it: two calls whose kernels
// overlap on the GPU (different streams, no ordering between them) race on
// it and may return wrong sums.  Each block writes every partial it owns
// before the final pass reads it, so nothing has to start at zero.
//
// The device address of the array is looked up once per device with
// cudaGetSymbolAddress, the first time the entry point runs on that device
// (with that device current).  Make that first call before any stream
// capture, since the lookup itself is not a stream operation.  The address
// is kept for the life of the process: after cudaDeviceReset on a device
// (which unloads the library's device code there) the kept address is stale,
// so do not call this entry point on that device again.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <mutex>

#include "../../include/natrix.h"
#include "kernels.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 8;
constexpr long kCellsPerBlock = (long)kThreads * kCellsPerThread;
constexpr long kMaxBlocks = (NATRIX_NOALLOC_MAX_CELLS + kCellsPerBlock - 1) / kCellsPerBlock;
constexpr int kMaxDevices = 64;

// 5 partial sums per block: {n, sum r, sum r^2, sum b, sum b^2}
static __device__ __align__(256) double g_residual_partials[kMaxBlocks * 5];

std::mutex g_setup_mu;
double* g_partials_addr[kMaxDevices] = {};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Same sums, arithmetic (natrix::ResidSums) and block decomposition as the
// handle-based residual; the neighbour-substitution rule (obstacle neighbour
// or wall -> centre pressure, shader.Poisson.comp:32-35 with common.sh:9-19
// clamping) is evaluated from the mask here instead of precomputed flags.
__global__ void __launch_bounds__(kThreads)
    k_residual_noalloc(const float* __restrict__ p, const float* __restrict__ div,
                       const uint8_t* __restrict__ mask, int W, int H, int P,
                       double* __restrict__ partials) {
    natrix::ResidSums rs;
    const int total = W * H;  // at most NATRIX_NOALLOC_MAX_CELLS
    const int base = blockIdx.x * (int)kCellsPerBlock + threadIdx.x;
    natrix::CellWalk w(base, W);
#pragma unroll
    for (int k = 0; k < kCellsPerThread; ++k) {
        const int lin = base + k * kThreads;
        const int x = w.x, y = w.y;
        w.advance(kThreads, W);
        if (lin >= total) continue;
        const size_t c = (size_t)y * P + x;
        if (mask && mask[c]) continue;
        const size_t l = x > 0 ? c - 1 : c, r = x < W - 1 ? c + 1 : c;
        const size_t b = y > 0 ? c - P : c, t = y < H - 1 ? c + P : c;
        const bool sl = x == 0 || (mask && mask[l]);
        const bool sr = x == W - 1 || (mask && mask[r]);
        const bool sb = y == 0 || (mask && mask[b]);
        const bool st = y == H - 1 || (mask && mask[t]);
        const float pc = p[c];
        rs.add(div[c], pc, sl ? pc : p[l], sr ? pc : p[r], sb ? pc : p[b], st ? pc : p[t]);
    }
    __shared__ double s_part[kThreads / 32][5];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    rs.warp_sum();
    if (lane == 0) rs.to_double(s_part[wid]);
    __syncthreads();
    if (threadIdx.x < 5) {
        double s = 0;
        for (int w = 0; w < kThreads / 32; ++w) s += s_part[w][threadIdx.x];
        partials[(size_t)blockIdx.x * 5 + threadIdx.x] = s;
    }
}

// One block of 256 threads: each thread sums every 256th block's partials,
// then the warps and the block reduce (FP64 throughput on one SM bounds this
// kernel, so few threads: the work is the partials' additions).
constexpr int kFinalThreads = 256;

__global__ void __launch_bounds__(kFinalThreads)
    k_residual_noalloc_final(const double* __restrict__ partials, int nblocks,
                             double* __restrict__ out) {
    __shared__ double s[kFinalThreads / 32][5];
    double acc[5] = {0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nblocks; b += kFinalThreads)
#pragma unroll
        for (int j = 0; j < 5; ++j) acc[j] += partials[(size_t)b * 5 + j];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const double v = warp_sum(acc[j]);
        if (lane == 0) s[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double t = 0;
        for (int w = 0; w < kFinalThreads / 32; ++w) t += s[w][threadIdx.x];
        out[threadIdx.x] = t;
    }
}

int noalloc_fail(int code, const char* msg) { return natrix::set_last_error(code, msg); }

// Device address of the scratch array on the current device, looked up once.
int partials_on_current_device(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(NATRIX_ECUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(NATRIX_ERANGE, "device ordinal too large");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_partials_addr[dev]) {
        void* addr = nullptr;
        e = cudaGetSymbolAddress(&addr, g_residual_partials);
        if (e != cudaSuccess) return noalloc_fail(NATRIX_ECUDA, cudaGetErrorString(e));
        g_partials_addr[dev] = static_cast<double*>(addr);
    }
    *out = g_partials_addr[dev];
    return NATRIX_OK;
}

}  // namespace

extern "C" int natrix_residual_noalloc(const float* p, const float* div, const uint8_t* mask,
                                       int32_t width, int32_t height, int64_t pitch,
                                       double* out_dev, void* stream) {
    if (!p || !div || !out_dev)
        return noalloc_fail(NATRIX_EINVAL, "natrix_residual_noalloc: NULL pressure, "
                                           "divergence or output pointer");
    if (width < 1 || height < 1 || pitch < width)
        return noalloc_fail(NATRIX_EINVAL, "natrix_residual_noalloc: bad width/height/pitch");
    if ((long long)width * height > NATRIX_NOALLOC_MAX_CELLS) {
        char buf[160];
        snprintf(buf, sizeof buf,
                 "natrix_residual_noalloc: %dx%d grid exceeds the %d-cell maximum of the "
                 "static scratch", width, height, NATRIX_NOALLOC_MAX_CELLS);
        return noalloc_fail(NATRIX_ERANGE, buf);
    }
    // the kernel indexes rows with a 32-bit pitch
    if (pitch > INT_MAX) {
        char buf[160];
        snprintf(buf, sizeof buf,
                 "natrix_residual_noalloc: row pitch %lld exceeds the largest supported "
                 "pitch %d", (long long)pitch, INT_MAX);
        return noalloc_fail(NATRIX_ERANGE, buf);
    }
    double* partials = nullptr;
    int rc = partials_on_current_device(&partials);
    if (rc) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const long total = (long)width * height;
    const int nblocks = (int)((total + kCellsPerBlock - 1) / kCellsPerBlock);
    k_residual_noalloc<<<nblocks, kThreads, 0, st>>>(p, div, mask, width, height, (int)pitch,
                                                     partials);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_residual_noalloc_final<<<1, kFinalThreads, 0, st>>>(partials, nblocks, out_dev);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return noalloc_fail(NATRIX_ECUDA, cudaGetErrorString(e));
    return NATRIX_OK;
}
