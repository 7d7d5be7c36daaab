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
// capture, since the lookup itself is not a stream operation.
#include <cuda_runtime.h>

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

// Same sums and the same block decomposition as the handle-based residual;
// the neighbour-substitution rule (obstacle neighbour or wall -> centre
// pressure, shader.Poisson.comp:32-35 with common.sh:9-19 clamping) is
// evaluated from the mask here instead of precomputed flags.
__global__ void __launch_bounds__(kThreads)
    k_residual_noalloc(const float* __restrict__ p, const float* __restrict__ div,
                       const uint8_t* __restrict__ mask, int W, int H, int P,
                       double* __restrict__ partials) {
    double acc[5] = {0, 0, 0, 0, 0};
    const long total = (long)W * H;
    const long base = (long)blockIdx.x * kCellsPerBlock + threadIdx.x;
    for (int k = 0; k < kCellsPerThread; ++k) {
        const long lin = base + (long)k * kThreads;
        if (lin >= total) break;
        const int y = (int)(lin / W), x = (int)(lin % W);
        const int xl = x > 0 ? x - 1 : 0, xr = x < W - 1 ? x + 1 : W - 1;
        const int yb = y > 0 ? y - 1 : 0, yt = y < H - 1 ? y + 1 : H - 1;
        const size_t c = (size_t)y * P + x;
        const size_t l = (size_t)y * P + xl, r = (size_t)y * P + xr;
        const size_t b = (size_t)yb * P + x, t = (size_t)yt * P + x;
        if (mask && mask[c]) continue;
        const bool sl = x == 0 || (mask && mask[l]);
        const bool sr = x == W - 1 || (mask && mask[r]);
        const bool sb = y == 0 || (mask && mask[b]);
        const bool st = y == H - 1 || (mask && mask[t]);
        const double pc = p[c];
        const double x1 = sl ? pc : (double)p[l];
        const double x2 = sr ? pc : (double)p[r];
        const double y1 = sb ? pc : (double)p[b];
        const double y2 = st ? pc : (double)p[t];
        const double bb = div[c];
        const double rr = bb - ((x1 + x2 + y1 + y2) - 4.0 * pc);
        acc[0] += 1.0;
        acc[1] += rr;
        acc[2] += rr * rr;
        acc[3] += bb;
        acc[4] += bb * bb;
    }
    __shared__ double s_part[kThreads / 32][5];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const double v = warp_sum(acc[j]);
        if (lane == 0) s_part[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double s = 0;
        for (int w = 0; w < kThreads / 32; ++w) s += s_part[w][threadIdx.x];
        partials[(size_t)blockIdx.x * 5 + threadIdx.x] = s;
    }
}

__global__ void k_residual_noalloc_final(const double* __restrict__ partials, int nblocks,
                                         double* __restrict__ out) {
    __shared__ double s[32][5];
    const int lane = threadIdx.x;
    double acc[5] = {0, 0, 0, 0, 0};
    for (int b = lane; b < nblocks; b += 32)
        for (int j = 0; j < 5; ++j) acc[j] += partials[(size_t)b * 5 + j];
    for (int j = 0; j < 5; ++j) s[lane][j] = acc[j];
    __syncwarp();
    if (lane < 5) {
        double t = 0;
        for (int k = 0; k < 32; ++k) t += s[k][lane];
        out[lane] = t;
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
    if ((long long)width * height > NATRIX_NOALLOC_MAX_CELLS || pitch > (1LL << 31)) {
        char buf[160];
        snprintf(buf, sizeof buf,
                 "natrix_residual_noalloc: %dx%d grid exceeds the %d-cell maximum of the "
                 "static scratch", width, height, NATRIX_NOALLOC_MAX_CELLS);
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
        k_residual_noalloc_final<<<1, 32, 0, st>>>(partials, nblocks, out_dev);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return noalloc_fail(NATRIX_ECUDA, cudaGetErrorString(e));
    return NATRIX_OK;
}
