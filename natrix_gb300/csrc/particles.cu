// Lagrangian particles carried by a simulator's velocity field and splatted
// into a density grid of the simulator's size.  No reference counterpart:
// the reference's "particles" are an Eulerian density grid (natrix_density);
// these are point particles with the same velocity sampler.
//
// One fused kernel per step: each thread moves one particle by RK2 (midpoint)
// through the velocity field, sampled with the bilinear rule of
// shader.AdvectVelocity.comp:38-48 (clamped corners, unclamped delta),
// displacement v * dt * speed as the reference advects; the new position is
// clamped to [0, W-1] x [0, H-1]; then the particle deposits unit mass into the
// 3x3 cells around its nearest cell centre c = floor(p + 0.5) with a
// normalised linear hat of half-width 1.5 (weights (0.5-f, 1.5-|f|, 0.5+f) /
// (2.5-|f|) per axis, f = p - c), clamping targets onto the grid.  The
// deposits are fire-and-forget FP32 atomic adds (red.global.add.f32) into the
// L2-resident grid; their order is not fixed, so density matches the oracle
// to rounding while positions and cells match it bit for bit.
//
// Compiled with -fmad=false (see common.cuh): every operation rounds as the
// oracle's float restatement does.
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/natrix.h"
#include "kernels.cuh"

using namespace natrix;

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float2 rk2(float2 p, const float2* __restrict__ v, const Grid& g,
                                      float h, float hh) {
    const Corners c1 = corners(p.x, p.y, g.W, g.H);
    const float2 u1 = sample_vel(v, g.P, c1);
    const float mx = p.x + hh * u1.x, my = p.y + hh * u1.y;
    const Corners c2 = corners(mx, my, g.W, g.H);
    const float2 u2 = sample_vel(v, g.P, c2);
    float qx = p.x + h * u2.x, qy = p.y + h * u2.y;
    const float bx = (float)(g.W - 1), by = (float)(g.H - 1);
    qx = qx > 0.0f ? qx : 0.0f;
    qx = qx < bx ? qx : bx;
    qy = qy > 0.0f ? qy : 0.0f;
    qy = qy < by ? qy : by;
    return make_float2(qx, qy);
}

__device__ __forceinline__ int cell_of(float p) { return (int)floorf(p + 0.5f); }

__device__ __forceinline__ void tent3(float p, int c, float w[3]) {
    const float f = p - (float)c;
    const float af = fabsf(f);
    const float s = 2.5f - af;
    w[0] = (0.5f - f) / s;
    w[1] = (1.5f - af) / s;
    w[2] = (0.5f + f) / s;
}

__device__ __forceinline__ void red_add(float* addr, float v) {
    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(addr), "f"(v) : "memory");
}

__global__ void __launch_bounds__(kThreads)
    k_particles_step(float2* __restrict__ pos, long n, const float2* __restrict__ vel, Grid g,
                     float h, float hh, float* __restrict__ rho) {
    const long k = (long)blockIdx.x * kThreads + threadIdx.x;
    if (k >= n) return;
    const float2 q = rk2(pos[k], vel, g, h, hh);
    pos[k] = q;
    if (!rho) return;
    const int cx = cell_of(q.x), cy = cell_of(q.y);
    float wx[3], wy[3];
    tent3(q.x, cx, wx);
    tent3(q.y, cy, wy);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        int yy = cy + j - 1;
        yy = yy < 0 ? 0 : (yy > g.H - 1 ? g.H - 1 : yy);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int xx = cx + i - 1;
            xx = xx < 0 ? 0 : (xx > g.W - 1 ? g.W - 1 : xx);
            red_add(rho + (size_t)yy * g.P + xx, wx[i] * wy[j]);
        }
    }
}

__global__ void __launch_bounds__(kThreads)
    k_particle_cells(const float2* __restrict__ pos, long n, int2* __restrict__ cells) {
    const long k = (long)blockIdx.x * kThreads + threadIdx.x;
    if (k >= n) return;
    const float2 q = pos[k];
    cells[k] = make_int2(cell_of(q.x), cell_of(q.y));
}

int fail(int code, const char* msg) { return set_last_error(code, msg); }

int cuda_fail(cudaError_t e) { return set_last_error(NATRIX_ECUDA, cudaGetErrorString(e)); }

}  // namespace

struct natrix_particles {
    natrix_sim* fluid = nullptr;
    int device = 0;
    long n = 0;
    Grid g{};
    float2* pos = nullptr;
    float* rho = nullptr;
    int2* cells = nullptr;  // allocated on first natrix_particles_cells call
};

extern "C" {

int natrix_particles_create(natrix_sim* fluid, int64_t n, natrix_particles** out) {
    if (!fluid || !out) return fail(NATRIX_EINVAL, "NULL argument");
    *out = nullptr;
    if (n < 0 || n > (int64_t)1 << 31) return fail(NATRIX_ERANGE, "particle count out of range");
    SimView sv;
    sim_describe(fluid, &sv);
    DeviceGuard dg(sv.device);
    natrix_particles* p = new natrix_particles();
    p->fluid = fluid;
    p->device = sv.device;
    p->n = (long)n;
    p->g = sv.g;
    cudaError_t e = cudaMalloc(&p->pos, (size_t)(n > 0 ? n : 1) * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&p->rho, (size_t)p->g.P * p->g.H * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->rho, 0, (size_t)p->g.P * p->g.H * sizeof(float));
    if (e != cudaSuccess) {
        cudaFree(p->pos);
        cudaFree(p->rho);
        delete p;
        return fail(NATRIX_ENOMEM, cudaGetErrorString(e));
    }
    *out = p;
    return NATRIX_OK;
}

int natrix_particles_destroy(natrix_particles* p) {
    if (!p) return NATRIX_OK;
    DeviceGuard dg(p->device);
    cudaDeviceSynchronize();
    cudaFree(p->pos);
    cudaFree(p->rho);
    cudaFree(p->cells);
    delete p;
    return NATRIX_OK;
}

int natrix_particles_upload(natrix_particles* p, const float* host_xy, void* stream) {
    if (!p || (!host_xy && p->n)) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(p->device);
    cudaError_t e = cudaMemcpyAsync(p->pos, host_xy, (size_t)p->n * sizeof(float2),
                                    cudaMemcpyHostToDevice, (cudaStream_t)stream);
    return e == cudaSuccess ? NATRIX_OK : cuda_fail(e);
}

int natrix_particles_download(natrix_particles* p, float* host_xy, void* stream) {
    if (!p || (!host_xy && p->n)) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(p->device);
    cudaError_t e = cudaMemcpyAsync(host_xy, p->pos, (size_t)p->n * sizeof(float2),
                                    cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    return e == cudaSuccess ? NATRIX_OK : cuda_fail(e);
}

int natrix_particles_step(natrix_particles* p, float dt, int32_t splat, void* stream) {
    if (!p) return fail(NATRIX_EINVAL, "NULL handle");
    cudaStream_t st = (cudaStream_t)stream;
    SimView sv;
    int rc = sim_prepare_read(p->fluid, st, &sv);
    if (rc) return rc;
    DeviceGuard dg(p->device);
    const float h = dt * sv.speed;
    const float hh = h * 0.5f;
    if (splat) {
        cudaError_t e = cudaMemsetAsync(p->rho, 0, (size_t)p->g.P * p->g.H * sizeof(float), st);
        if (e != cudaSuccess) return cuda_fail(e);
    }
    if (p->n == 0) return NATRIX_OK;
    const long blocks = (p->n + kThreads - 1) / kThreads;
    k_particles_step<<<(unsigned)blocks, kThreads, 0, st>>>(p->pos, p->n, sv.vel, sv.g, h, hh,
                                                            splat ? p->rho : nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e);
    sim_count_launches(p->fluid, 1);
    return NATRIX_OK;
}

int natrix_particles_cells(natrix_particles* p, int32_t* host_cells, void* stream) {
    if (!p || (!host_cells && p->n)) return fail(NATRIX_EINVAL, "NULL argument");
    if (p->n == 0) return NATRIX_OK;
    DeviceGuard dg(p->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (!p->cells) {
        cudaError_t e = cudaMalloc(&p->cells, (size_t)p->n * sizeof(int2));
        if (e != cudaSuccess) return fail(NATRIX_ENOMEM, cudaGetErrorString(e));
    }
    const long blocks = (p->n + kThreads - 1) / kThreads;
    k_particle_cells<<<(unsigned)blocks, kThreads, 0, st>>>(p->pos, p->n, p->cells);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_cells, p->cells, (size_t)p->n * sizeof(int2),
                            cudaMemcpyDeviceToHost, st);
    return e == cudaSuccess ? NATRIX_OK : cuda_fail(e);
}

int natrix_particles_field(natrix_particles* p, void** pos, void** density, int64_t* pitch) {
    if (!p || !pos || !density || !pitch) return fail(NATRIX_EINVAL, "NULL argument");
    *pos = p->pos;
    *density = p->rho;
    *pitch = p->g.P;
    return NATRIX_OK;
}

}  // extern "C"
