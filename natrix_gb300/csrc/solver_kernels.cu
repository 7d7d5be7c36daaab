// Per-cell solver kernels: forcing, obstacle rasterisation, advection,
// vorticity confinement, viscosity, divergence, gradient subtraction, density
// advection and the pressure residual.
//
// One thread per cell, 32x8 blocks (a warp spans 32 consecutive cells of a
// row, so float2 velocity loads and stores coalesce into 256-byte segments).
// Compiled with -fmad=false: see common.cuh for the arithmetic contract.
#include "cells.cuh"

namespace natrix {

namespace {

inline dim3 grid_for(const Grid& g) { return dim3((g.W + BX - 1) / BX, (g.H + BY - 1) / BY); }

// The streaming stencil kernels give each thread CPT cells of one column,
// BY rows apart, so every thread has CPT independent load chains in flight
// (one 8-byte load per thread per block leaves HBM under-subscribed).
constexpr int CPT = 4;
inline dim3 grid_cpt(const Grid& g) {
    return dim3((g.W + BX - 1) / BX, (g.H + BY * CPT - 1) / (BY * CPT));
}
#define NX_CELLS(call)                                               \
    do {                                                             \
        const int x = blockIdx.x * BX + threadIdx.x;                 \
        const int y0 = blockIdx.y * (BY * CPT) + threadIdx.y;        \
        _Pragma("unroll") for (int k = 0; k < CPT; ++k) {            \
            const int y = y0 + k * BY;                               \
            call;                                                    \
        }                                                            \
    } while (0)

__global__ void __launch_bounds__(BX* BY)
    k_obstacles(uint8_t* __restrict__ mask, Grid g, const ShapeOp* __restrict__ ops, int n,
                int fresh) {
    block_obstacles(mask, g, ops, n, fresh, blockIdx.x * BX, blockIdx.y * BY);
}

__global__ void __launch_bounds__(BX* BY)
    k_forcing(float2* __restrict__ vel, Grid gv, float* __restrict__ rho, Grid gd,
              const ForceOp* __restrict__ ops, int n) {
    block_forcing(vel, gv, rho, gd, ops, n, blockIdx.x * BX, blockIdx.y * BY);
}

__global__ void __launch_bounds__(BX* BY) k_advect(const float2* __restrict__ vin, float2* __restrict__ vout,
             const uint8_t* __restrict__ mask, Grid g, const StepParams* __restrict__ sp) {
    NX_CELLS(cell_advect(vin, vout, mask, g, sp, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_calc_vorticity(const float2* __restrict__ v, float* __restrict__ w, Grid g) {
    NX_CELLS(cell_calc_vorticity(v, w, g, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_apply_vorticity(const float2* __restrict__ vin, float2* __restrict__ vout,
                      const float* __restrict__ w, Grid g, const StepParams* __restrict__ sp) {
    NX_CELLS(cell_apply_vorticity(vin, vout, w, g, sp, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_viscosity(const float2* __restrict__ vin, float2* __restrict__ vout, Grid g,
                const StepParams* __restrict__ sp) {
    NX_CELLS(cell_viscosity(vin, vout, g, sp, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_divergence(const float2* __restrict__ v, const uint8_t* __restrict__ mask,
                 float* __restrict__ div, uint8_t* __restrict__ flags, float* __restrict__ p1,
                 Grid g, const StepParams* __restrict__ sp) {
    NX_CELLS(cell_divergence(v, mask, div, flags, p1, g, sp, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_subtract_gradient(const float2* __restrict__ vin, float2* __restrict__ vout,
                        const float* __restrict__ p, const uint8_t* __restrict__ flags,
                        Grid g) {
    NX_CELLS(cell_subtract_gradient(vin, vout, p, flags, g, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_density_advect(const float* __restrict__ rin, float* __restrict__ rout, Grid gd,
                     const float2* __restrict__ v, const uint8_t* __restrict__ mask, Grid gv,
                     const StepParams* __restrict__ sp) {
    NX_CELLS(cell_density_advect(rin, rout, gd, v, mask, gv, sp, x, y));
}

// Vorticity confinement in one pass: shader.CalcVorticity.comp then
// shader.ApplyVorticity.comp on a 32 x 16 output tile.  The block stages the
// velocity of the tile plus 2 cells (index-clamped, as GetNeighbours reads),
// computes the curl of the tile plus 1 cell into shared memory (each at its
// clamped grid position, so a clamped neighbour of an edge cell reads the edge
// cell's own curl), then applies the confinement force.  Same expressions as
// cell_calc_vorticity / cell_apply_vorticity, so the results are identical;
// the curl of the tile is still written out (the vorticity field).
constexpr int VT_W = BX, VT_H = BY * CPT;
constexpr int VV_W = VT_W + 4, VV_H = VT_H + 4;  // staged velocity
constexpr int VW_W = VT_W + 2, VW_H = VT_H + 2;  // staged curl

__global__ void __launch_bounds__(BX* BY)
    k_vorticity(const float2* __restrict__ vin, float2* __restrict__ vout, float* __restrict__ w,
                Grid g, const StepParams* __restrict__ sp) {
    __shared__ float2 sv[VV_H][VV_W];
    __shared__ float sw[VW_H][VW_W];
    const int x0 = blockIdx.x * VT_W, y0 = blockIdx.y * VT_H;
    const int tid = threadIdx.y * BX + threadIdx.x;
    for (int i = tid; i < VV_H * VV_W; i += BX * BY) {
        const int ry = i / VV_W, rx = i % VV_W;
        const int gx = min(max(x0 - 2 + rx, 0), g.W - 1), gy = min(max(y0 - 2 + ry, 0), g.H - 1);
        sv[ry][rx] = __ldg(vin + (size_t)gy * g.P + gx);
    }
    __syncthreads();
    for (int i = tid; i < VW_H * VW_W; i += BX * BY) {
        const int ry = i / VW_W, rx = i % VW_W;
        // curl at the clamped grid position, from its clamped neighbours
        const int gx = min(max(x0 - 1 + rx, 0), g.W - 1), gy = min(max(y0 - 1 + ry, 0), g.H - 1);
        const int cx = gx - x0 + 2, cy = gy - y0 + 2;  // its staged velocity position
        const float2 vl = sv[cy][cx - 1], vr = sv[cy][cx + 1], vb = sv[cy - 1][cx],
                     vt = sv[cy + 1][cx];
        sw[ry][rx] = 0.5f * ((vr.y - vl.y) - (vt.x - vb.x));
    }
    __syncthreads();
    const float eps = 2.4414e-4f;
    const float vort = sp->vorticity, dt = sp->dt;
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int tx = threadIdx.x, ty = threadIdx.y + k * BY;
        const int x = x0 + tx, y = y0 + ty;
        if (x >= g.W || y >= g.H) continue;
        const int xl = max(x - 1, 0) - x0 + 1, xr = min(x + 1, g.W - 1) - x0 + 1;
        const int yb = max(y - 1, 0) - y0 + 1, yt = min(y + 1, g.H - 1) - y0 + 1;
        const float wl = sw[ty + 1][xl], wr = sw[ty + 1][xr], wb = sw[yb][tx + 1],
                    wt = sw[yt][tx + 1], wc = sw[ty + 1][tx + 1];
        float fx = 0.5f * (fabsf(wt) - fabsf(wb));
        float fy = 0.5f * (fabsf(wr) - fabsf(wl));
        const float d = fx * fx + fy * fy;
        const float m = eps > d ? eps : d;
        const float rs = 1.0f / sqrtf(m);
        fx = fx * rs;
        fy = fy * rs;
        const float s = vort * wc;
        fx = fx * (s * 1.0f);
        fy = fy * (s * -1.0f);
        const float2 v = sv[ty + 2][tx + 2];
        const size_t c = (size_t)y * g.P + x;
        vout[c] = make_float2(v.x + fx * dt, v.y + fy * dt);
        w[c] = wc;
    }
}

// ----------------------------------------------------------------- residual
// r = b - (sum of substituted neighbours - 4 p) over fluid cells, in double;
// warp-shuffle then shared-memory reduction per block, block partials summed
// by a second one-block kernel in a fixed order (deterministic).
constexpr int RES_THREADS = 256;
constexpr int RES_CELLS_PER_THREAD = 8;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(RES_THREADS)
    k_residual(const float* __restrict__ p, const float* __restrict__ div,
               const uint8_t* __restrict__ mask, const uint8_t* __restrict__ flags, Grid g,
               const StepParams* __restrict__ sp, double* __restrict__ partials) {
    double acc[5] = {0, 0, 0, 0, 0};
    const long total = (long)g.W * g.H;
    const long base = (long)blockIdx.x * RES_THREADS * RES_CELLS_PER_THREAD + threadIdx.x;
    const bool mz = sp->mask_zero != 0;
    for (int k = 0; k < RES_CELLS_PER_THREAD; ++k) {
        const long lin = base + (long)k * RES_THREADS;
        if (lin >= total) break;
        const int y = (int)(lin / g.W), x = (int)(lin % g.W);
        const Nbr n = nbrs(g, x, y);
        if (!mz && mask[n.c]) continue;
        const uint8_t f = flags[n.c];
        const double pc = p[n.c];
        const double x1 = (f & NB_L) ? pc : (double)p[n.l];
        const double x2 = (f & NB_R) ? pc : (double)p[n.r];
        const double y1 = (f & NB_B) ? pc : (double)p[n.b];
        const double y2 = (f & NB_T) ? pc : (double)p[n.t];
        const double b = div[n.c];
        const double r = b - ((x1 + x2 + y1 + y2) - 4.0 * pc);
        acc[0] += 1.0;
        acc[1] += r;
        acc[2] += r * r;
        acc[3] += b;
        acc[4] += b * b;
    }
    __shared__ double s_part[RES_THREADS / 32][5];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const double v = warp_sum(acc[j]);
        if (lane == 0) s_part[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double s = 0;
        for (int w = 0; w < RES_THREADS / 32; ++w) s += s_part[w][threadIdx.x];
        partials[(size_t)blockIdx.x * 5 + threadIdx.x] = s;
    }
}

// The same sums per connected fluid region: labels[y*W + x] in [0, n) for
// fluid cells, < 0 for obstacle cells.  The pressure system is pure Neumann
// on each region, so its residual is only defined up to each region's mean.
// Warps whose lanes share one label (the common case) reduce first and add
// once; mixed warps add per lane.
__global__ void __launch_bounds__(RES_THREADS)
    k_residual_labels(const float* __restrict__ p, const float* __restrict__ div,
                      const uint8_t* __restrict__ flags, const int* __restrict__ labels, Grid g,
                      double* __restrict__ sums) {
    const long total = (long)g.W * g.H;
    const long lin = (long)blockIdx.x * RES_THREADS + threadIdx.x;
    int lab = -1;
    double v[5] = {0, 0, 0, 0, 0};
    if (lin < total) {
        const int y = (int)(lin / g.W), x = (int)(lin % g.W);
        lab = labels[lin];
        if (lab >= 0) {
            const Nbr n = nbrs(g, x, y);
            const uint8_t f = flags[n.c];
            const double pc = p[n.c];
            const double x1 = (f & NB_L) ? pc : (double)p[n.l];
            const double x2 = (f & NB_R) ? pc : (double)p[n.r];
            const double y1 = (f & NB_B) ? pc : (double)p[n.b];
            const double y2 = (f & NB_T) ? pc : (double)p[n.t];
            const double b = div[n.c];
            const double r = b - ((x1 + x2 + y1 + y2) - 4.0 * pc);
            v[0] = 1.0;
            v[1] = r;
            v[2] = r * r;
            v[3] = b;
            v[4] = b * b;
        }
    }
    const int l0 = __shfl_sync(0xffffffffu, lab, 0);
    const bool uniform = __all_sync(0xffffffffu, lab == l0);
    if (uniform) {
        if (l0 < 0) return;
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const double t = warp_sum(v[j]);
            if ((threadIdx.x & 31) == 0) atomicAdd(sums + (size_t)l0 * 5 + j, t);
        }
    } else if (lab >= 0) {
#pragma unroll
        for (int j = 0; j < 5; ++j) atomicAdd(sums + (size_t)lab * 5 + j, v[j]);
    }
}

__global__ void k_residual_final(const double* __restrict__ partials, int nblocks,
                                 double* __restrict__ out) {
    __shared__ double s[32][5];
    const int lane = threadIdx.x;  // 32 threads
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

}  // namespace

cudaError_t launch_residual_labels(const float* p, const float* div, const uint8_t* flags,
                                   const int* labels, int n_labels, Grid g, double* sums,
                                   cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(sums, 0, (size_t)n_labels * 5 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    const long total = (long)g.W * g.H;
    k_residual_labels<<<(unsigned)((total + RES_THREADS - 1) / RES_THREADS), RES_THREADS, 0, st>>>(
        p, div, flags, labels, g, sums);
    return cudaGetLastError();
}

cudaError_t launch_obstacles(uint8_t* mask, Grid g, const ShapeOp* ops, int n, int fresh,
                             cudaStream_t st) {
    k_obstacles<<<grid_for(g), dim3(BX, BY), 0, st>>>(mask, g, ops, n, fresh);
    return cudaGetLastError();
}

cudaError_t launch_forcing(float2* vel, Grid gv, float* rho, Grid gd, const ForceOp* ops,
                           int n, cudaStream_t st) {
    Grid gg = vel ? gv : gd;
    if (vel && rho) gg = Grid{gv.W > gd.W ? gv.W : gd.W, gv.H > gd.H ? gv.H : gd.H, 0};
    k_forcing<<<grid_for(gg), dim3(BX, BY), 0, st>>>(vel, gv, rho, gd, ops, n);
    return cudaGetLastError();
}

cudaError_t launch_advect(const float2* vin, float2* vout, const uint8_t* mask, Grid g,
                          const StepParams* sp, cudaStream_t st) {
    k_advect<<<grid_cpt(g), dim3(BX, BY), 0, st>>>(vin, vout, mask, g, sp);
    return cudaGetLastError();
}

cudaError_t launch_calc_vorticity(const float2* v, float* w, Grid g, cudaStream_t st) {
    k_calc_vorticity<<<grid_cpt(g), dim3(BX, BY), 0, st>>>(v, w, g);
    return cudaGetLastError();
}

cudaError_t launch_apply_vorticity(const float2* vin, float2* vout, const float* w, Grid g,
                                   const StepParams* sp, cudaStream_t st) {
    k_apply_vorticity<<<grid_cpt(g), dim3(BX, BY), 0, st>>>(vin, vout, w, g, sp);
    return cudaGetLastError();
}

cudaError_t launch_vorticity(const float2* vin, float2* vout, float* w, Grid g,
                             const StepParams* sp, cudaStream_t st) {
    k_vorticity<<<dim3((g.W + VT_W - 1) / VT_W, (g.H + VT_H - 1) / VT_H), dim3(BX, BY), 0, st>>>(
        vin, vout, w, g, sp);
    return cudaGetLastError();
}

cudaError_t launch_viscosity(const float2* vin, float2* vout, Grid g, const StepParams* sp,
                             cudaStream_t st) {
    k_viscosity<<<grid_cpt(g), dim3(BX, BY), 0, st>>>(vin, vout, g, sp);
    return cudaGetLastError();
}

cudaError_t launch_divergence(const float2* v, const uint8_t* mask, float* div,
                              uint8_t* flags, float* p1, Grid g, const StepParams* sp,
                              cudaStream_t st) {
    k_divergence<<<grid_cpt(g), dim3(BX, BY), 0, st>>>(v, mask, div, flags, p1, g, sp);
    return cudaGetLastError();
}

cudaError_t launch_subtract_gradient(const float2* vin, float2* vout, const float* p,
                                     const uint8_t* flags, Grid g, cudaStream_t st) {
    k_subtract_gradient<<<grid_cpt(g), dim3(BX, BY), 0, st>>>(vin, vout, p, flags, g);
    return cudaGetLastError();
}

cudaError_t launch_density_advect(const float* rin, float* rout, Grid gd, const float2* v,
                                  const uint8_t* mask, Grid gv, const StepParams* sp,
                                  cudaStream_t st) {
    k_density_advect<<<grid_cpt(gd), dim3(BX, BY), 0, st>>>(rin, rout, gd, v, mask, gv, sp);
    return cudaGetLastError();
}

int residual_partials(Grid g) {
    const long total = (long)g.W * g.H;
    const long per = (long)RES_THREADS * RES_CELLS_PER_THREAD;
    return (int)((total + per - 1) / per);
}

cudaError_t launch_residual(const float* p, const float* div, const uint8_t* mask,
                            const uint8_t* flags, Grid g, const StepParams* sp,
                            double* partials, double* out, cudaStream_t st) {
    const int nb = residual_partials(g);
    k_residual<<<nb, RES_THREADS, 0, st>>>(p, div, mask, flags, g, sp, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_residual_final<<<1, 32, 0, st>>>(partials, nb, out);
    return cudaGetLastError();
}

}  // namespace natrix
