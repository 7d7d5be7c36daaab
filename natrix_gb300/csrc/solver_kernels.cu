// Per-cell solver kernels: forcing, obstacle rasterisation, advection,
// vorticity confinement, viscosity, divergence, gradient subtraction, density
// advection and the pressure residual.
//
// One thread per cell, 32x8 blocks (a warp spans 32 consecutive cells of a
// row, so float2 velocity loads and stores coalesce into 256-byte segments).
// Compiled with -fmad=false: see common.cuh for the arithmetic contract.
#include <climits>
#include <cstdlib>
#include <algorithm>
#include <vector>

#include "cells.cuh"

namespace natrix {

namespace {

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

// Forcing and obstacles: FORCE_ROWS rows of cells per thread, so the op list
// is loaded and culled once per BX x (BY * FORCE_ROWS) cells.
constexpr int FORCE_ROWS = 4;

// The op list travels in the launch's parameter block (no host-to-device
// copy on the stream); CAP is the smallest of 16 / 64 / 256 that holds it.
template <int CAP>
__global__ void __launch_bounds__(BX* BY)
    k_obstacles(uint8_t* __restrict__ mask, Grid g, const __grid_constant__ OpBlock<ShapeOp, CAP> ob,
                int fresh) {
    pdl_enter();
    block_obstacles<FORCE_ROWS>(mask, g, ob.op, ob.n, fresh, blockIdx.x * BX,
                                blockIdx.y * BY * FORCE_ROWS);
}

template <int CAP>
__global__ void __launch_bounds__(BX* BY)
    k_forcing(float2* __restrict__ vel, Grid gv, float* __restrict__ rho, Grid gd,
              const __grid_constant__ OpBlock<ForceOp, CAP> ob, int zero_border) {
    pdl_enter();
    block_forcing<FORCE_ROWS>(vel, gv, rho, gd, ob.op, ob.n, blockIdx.x * BX,
                              blockIdx.y * BY * FORCE_ROWS, zero_border != 0);
}

// Density-only forcing touches cells inside the ops' footprints only, so the
// launch covers just the 32x32 blocks a conservative footprint box reaches
// (block ids in the parameter block); the in-kernel cull is unchanged.
static_assert(BX == kRasterBlock && BY * FORCE_ROWS == kRasterBlock, "raster block geometry");
struct ForceTiles {
    int n, tiles_x;
    uint16_t id[kMaxRasterBlocks];
};

// Obstacle raster over listed blocks only (the host keeps the mask zero
// outside the blocks it lists).
template <int CAP>
__global__ void __launch_bounds__(BX* BY)
    k_obstacles_blocks(uint8_t* __restrict__ mask, Grid g,
                       const __grid_constant__ OpBlock<ShapeOp, CAP> ob, int fresh,
                       const __grid_constant__ ForceTiles tl) {
    pdl_enter();
    const int t = tl.id[blockIdx.x];
    block_obstacles<FORCE_ROWS>(mask, g, ob.op, ob.n, fresh, (t % tl.tiles_x) * BX,
                                (t / tl.tiles_x) * BY * FORCE_ROWS);
}

template <int CAP>
__global__ void __launch_bounds__(BX* BY)
    k_forcing_tiles(float* __restrict__ rho, Grid gd, const __grid_constant__ OpBlock<ForceOp, CAP> ob,
                    const __grid_constant__ ForceTiles tl) {
    pdl_enter();
    const int t = tl.id[blockIdx.x];
    block_forcing<FORCE_ROWS>(nullptr, Grid{}, rho, gd, ob.op, ob.n, (t % tl.tiles_x) * BX,
                              (t / tl.tiles_x) * BY * FORCE_ROWS);
}

// Velocity forcing over listed blocks (launch_forcing_sparse): the same
// block body as k_forcing, so a listed block's cells come out identical.
template <int CAP>
__global__ void __launch_bounds__(BX* BY)
    k_vforcing_tiles(float2* __restrict__ vel, Grid gv,
                     const __grid_constant__ OpBlock<ForceOp, CAP> ob,
                     const __grid_constant__ ForceTiles tl, int zero_border) {
    pdl_enter();
    const int t = tl.id[blockIdx.x];
    block_forcing<FORCE_ROWS>(vel, gv, nullptr, Grid{}, ob.op, ob.n, (t % tl.tiles_x) * BX,
                              (t / tl.tiles_x) * BY * FORCE_ROWS, zero_border != 0);
}

template <typename Op, int CAP>
OpBlock<Op, CAP> op_block(const Op* ops, int n) {
    OpBlock<Op, CAP> ob;
    ob.n = n;
    for (int i = 0; i < n; ++i) ob.op[i] = ops[i];
    return ob;
}

// shader.AdvectVelocity.comp:19-51 (cell_advect's arithmetic, 32-bit cell
// indices).  ZB: border cells read as zero (shader.InitBoundaries.comp fused
// on read); false when has_borders is off or when this step's forcing launch
// already wrote the zero border in place, as the reference's InitBoundaries
// dispatch does before advecting.
// CLAMP: the step's first velocity op clamped only the blocks it listed
// (launch_forcing_sparse); every velocity read is clamped here instead, which
// leaves the listed blocks' (already clamped) values unchanged.
__device__ __forceinline__ float2 clamp_vel(float2 v) {
    return make_float2(clampf(v.x, -1.0f, 1.0f), clampf(v.y, -1.0f, 1.0f));
}

template <bool ZB, bool CLAMP = false>
__global__ void __launch_bounds__(BX* BY)
    k_advect(const float2* __restrict__ vin, float2* __restrict__ vout,
             const uint8_t* __restrict__ mask, Grid g, const __grid_constant__ StepParams sp) {
    pdl_enter();
    const int x = blockIdx.x * BX + threadIdx.x;
    if (x >= g.W) return;
    const bool mz = sp.mask_zero != 0;
    const float dt = sp.dt, speed = sp.speed, diss = sp.dissipation;
    const bool xb = ZB && (x == 0 || x == g.W - 1);
    const float2 zero = make_float2(0.0f, 0.0f);
    const int y0 = blockIdx.y * (BY * CPT) + threadIdx.y;
    // every cell's own velocity and obstacle byte first (loads in flight
    // together instead of one cell's chain after another)
    float2 vc[CPT];
    bool ob[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int y = y0 + k * BY;
        const int i = y * g.P + x;
        if (y < g.H) {
            vc[k] = __ldg(vin + i);
            ob[k] = !mz && mask[i];
        }
    }
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int y = y0 + k * BY;
        if (y >= g.H) break;
        const int i = y * g.P + x;
        if (ob[k]) {
            vout[i] = zero;
            continue;
        }
        float2 vel = CLAMP ? clamp_vel(vc[k]) : vc[k];
        if (ZB && (xb || y == 0 || y == g.H - 1)) vel = zero;
        const float fx = (float)x - vel.x * dt * speed;
        const float fy = (float)y - vel.y * dt * speed;
        const Corners c = corners(fx, fy, g.W, g.H);
        const int rl = c.lo_y * g.P, rh = c.hi_y * g.P;
        float2 lt = __ldg(vin + rh + c.lo_x), rt = __ldg(vin + rh + c.hi_x);
        float2 lb = __ldg(vin + rl + c.lo_x), rb = __ldg(vin + rl + c.hi_x);
        if (CLAMP) {
            lt = clamp_vel(lt);
            rt = clamp_vel(rt);
            lb = clamp_vel(lb);
            rb = clamp_vel(rb);
        }
        if (ZB) {
            const bool bxl = c.lo_x == 0 || c.lo_x == g.W - 1;
            const bool bxh = c.hi_x == 0 || c.hi_x == g.W - 1;
            const bool byl = c.lo_y == 0 || c.lo_y == g.H - 1;
            const bool byh = c.hi_y == 0 || c.hi_y == g.H - 1;
            if (bxl || byh) lt = zero;
            if (bxh || byh) rt = zero;
            if (bxl || byl) lb = zero;
            if (bxh || byl) rb = zero;
        }
        const float h1x = mixf(lt.x, rt.x, c.dx), h1y = mixf(lt.y, rt.y, c.dx);
        const float h2x = mixf(lb.x, rb.x, c.dx), h2y = mixf(lb.y, rb.y, c.dx);
        const float sx = mixf(h2x, h1x, c.dy), sy = mixf(h2y, h1y, c.dy);
        vout[i] = make_float2(clampf(sx * diss, -1.0f, 1.0f), clampf(sy * diss, -1.0f, 1.0f));
    }
}

__global__ void __launch_bounds__(BX* BY) k_viscosity(const float2* __restrict__ vin, float2* __restrict__ vout, Grid g,
                const __grid_constant__ StepParams spv) {
    pdl_enter();
    const StepParams* sp = &spv;
    NX_CELLS(cell_viscosity(vin, vout, g, sp, x, y));
}

// Zero the previous step's tile marks (first block of the grid).
__device__ __forceinline__ void clear_marks(const TileMarks& tm) {
    if (tm.clear && blockIdx.x == 0 && blockIdx.y == 0)
        for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < tm.words;
             i += blockDim.x * blockDim.y)
            tm.clear[i] = 0u;
}

__device__ __forceinline__ int ceil_div_signed(int a, int b) {
    return a > 0 ? (a + b - 1) / b : -((-a) / b);
}

// Mark every sweep tile whose region meets the cell box [x0, x1] x [y0, y1]
// (coordinates >= 0).
__device__ void mark_tiles(const TileMarks& tm, int x0, int x1, int y0, int y1) {
    const int i0 = max(ceil_div_signed(x0 + tm.hxp - tm.rx + 1, tm.tx), 0);
    const int i1 = min((x1 + tm.hxp) / tm.tx, tm.tiles_x - 1);
    const int j0 = max(ceil_div_signed(y0 + tm.halo - tm.ry + 1, tm.ty), 0);
    const int j1 = min((y1 + tm.halo) / tm.ty, tm.tiles_y - 1);
    for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            const int t = j * tm.tiles_x + i;
            atomicOr(tm.mark + (t >> 5), 1u << (t & 31));
        }
}

__global__ void __launch_bounds__(BX* BY) k_divergence(const float2* __restrict__ v, const uint8_t* __restrict__ mask,
                 float* __restrict__ div, uint8_t* __restrict__ flags, float* __restrict__ p1,
                 Grid g, const __grid_constant__ StepParams spv, const __grid_constant__ TileMarks tm) {
    pdl_enter();
    const StepParams* sp = &spv;
    clear_marks(tm);  // this variant leaves the marks empty (static tile order)
    NX_CELLS(cell_divergence(v, mask, div, flags, p1, g, sp, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_subtract_gradient(const float2* __restrict__ vin, float2* __restrict__ vout,
                        const float* __restrict__ p, const uint8_t* __restrict__ flags,
                        Grid g) {
    pdl_enter();
    NX_CELLS(cell_subtract_gradient(vin, vout, p, flags, g, x, y));
}

__global__ void __launch_bounds__(BX* BY) k_density_advect(const float* __restrict__ rin, float* __restrict__ rout, Grid gd,
                     const float2* __restrict__ v, const uint8_t* __restrict__ mask, Grid gv,
                     const __grid_constant__ StepParams spv) {
    pdl_enter();
    const StepParams* sp = &spv;
    NX_CELLS(cell_density_advect(rin, rout, gd, v, mask, gv, sp, x, y));
}

// Density and velocity grids of one power-of-two size: the matching velocity
// position x / W * W is x exactly (both operations exact), so the velocity is
// the cell's own and its obstacle test the cell's own (cell_density_advect's
// arithmetic otherwise; see its cell-centre note for the -0 case).
__global__ void __launch_bounds__(BX* BY)
    k_density_advect_same(const float* __restrict__ rin, float* __restrict__ rout, Grid gd,
                          const float2* __restrict__ v, const uint8_t* __restrict__ mask, Grid gv,
                          const __grid_constant__ StepParams sp) {
    pdl_enter();
    const int x = blockIdx.x * BX + threadIdx.x;
    if (x >= gd.W) return;
    const bool mz = sp.mask_zero != 0;
    const float dt = sp.dt, speed = sp.d_speed, diss = sp.d_dissipation;
    const int y0 = blockIdx.y * (BY * CPT) + threadIdx.y;
    float2 uc[CPT];
    bool ob[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int y = y0 + k * BY;
        const int vi = y * gv.P + x;
        if (y < gd.H) {
            uc[k] = __ldg(v + vi);
            ob[k] = !mz && mask[vi];
        }
    }
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int y = y0 + k * BY;
        if (y >= gd.H) break;
        const int i = y * gd.P + x;
        if (ob[k]) {
            rout[i] = 0.0f;
            continue;
        }
        const float2 u = uc[k];
        const float fx = (float)x - u.x * dt * speed;
        const float fy = (float)y - u.y * dt * speed;
        const Corners c = corners(fx, fy, gd.W, gd.H);
        rout[i] = sample_scalar(rin, gd.P, c) * diss;
    }
}

// Vorticity confinement in one pass: shader.CalcVorticity.comp then
// shader.ApplyVorticity.comp on a 64 x 32 output tile (each thread two
// adjacent columns, four rows 8 apart).  The block stages the velocity of the
// tile plus 2 cells (index-clamped, as GetNeighbours reads), computes the
// curl of the tile plus 1 cell into shared memory (each at its clamped grid
// position, so a clamped neighbour of an edge cell reads the edge cell's own
// curl), then applies the confinement force.  Same expressions as
// cell_calc_vorticity / cell_apply_vorticity, so the results are identical;
// the curl of the tile is still written out (the vorticity field).
constexpr int VT_W = 2 * BX, VT_H = BY * CPT;
constexpr int VV_W = VT_W + 4, VV_H = VT_H + 4;  // staged velocity
constexpr int VW_W = VT_W + 2, VW_H = VT_H + 2;  // staged curl

__device__ __forceinline__ float curl_at(const float2 (*sv)[VV_W], int cx, int cy) {
    return 0.5f * ((sv[cy][cx + 1].y - sv[cy][cx - 1].y) - (sv[cy + 1][cx].x - sv[cy - 1][cx].x));
}

// shader.ApplyVorticity.comp:19-40 for one cell from its staged curls.
__device__ __forceinline__ float2 confine(float wl, float wr, float wb, float wt, float wc,
                                          float2 v, float vort, float dt) {
    const float eps = 2.4414e-4f;
    float fx = 0.5f * (fabsf(wt) - fabsf(wb));
    float fy = 0.5f * (fabsf(wr) - fabsf(wl));
    const float d = fx * fx + fy * fy;
    const float m = eps > d ? eps : d;
    // 1/sqrt(m) with both operations correctly rounded, as sqrtf and the IEEE
    // division give (m >= eps is normal)
    const float rs = __frcp_rn(__fsqrt_rn(m));
    fx = fx * rs;
    fy = fy * rs;
    const float s = vort * wc;
    fx = fx * (s * 1.0f);
    fy = fy * (s * -1.0f);
    return make_float2(v.x + fx * dt, v.y + fy * dt);
}

// Staging, curl and confinement of one tile.  INTERIOR: the tile plus its
// 2-cell halo lies inside the grid, so no index is clamped, velocity rows are
// staged as 16-byte pairs (x0 - 2 is even and rows are pitched to 32 cells)
// and each thread's two cells are read and written as pairs; otherwise every
// staged and sampled index is clamped to the grid as GetNeighbours clamps it.
// Both paths evaluate the same expressions on the same values.
template <bool INTERIOR>
__device__ __forceinline__ void vorticity_tile(const float2* __restrict__ vin,
                                               float2* __restrict__ vout, float* __restrict__ w,
                                               const Grid& g, const StepParams* sp,
                                               float2 (*sv)[VV_W], float (*sw)[VW_W], int x0,
                                               int y0) {
    const int lane = threadIdx.x, wy = threadIdx.y;
    if (INTERIOR) {
        const float4* src = reinterpret_cast<const float4*>(vin + (y0 - 2) * g.P + (x0 - 2));
        const int qp = g.P / 2;
        for (int ry = wy; ry < VV_H; ry += BY) {
            *reinterpret_cast<float4*>(&sv[ry][2 * lane]) = __ldg(src + ry * qp + lane);
            if (lane < VV_W / 2 - BX)
                *reinterpret_cast<float4*>(&sv[ry][2 * BX + 2 * lane]) =
                    __ldg(src + ry * qp + BX + lane);
        }
    } else {
        for (int i = wy * BX + lane; i < VV_H * VV_W; i += BX * BY) {
            const int ry = i / VV_W, rx = i % VV_W;
            const int gx = min(max(x0 - 2 + rx, 0), g.W - 1), gy = min(max(y0 - 2 + ry, 0), g.H - 1);
            sv[ry][rx] = __ldg(vin + gy * g.P + gx);
        }
    }
    __syncthreads();
    if (INTERIOR) {
        for (int ry = wy; ry < VW_H; ry += BY) {
            sw[ry][lane] = curl_at(sv, lane + 1, ry + 1);
            sw[ry][lane + BX] = curl_at(sv, lane + BX + 1, ry + 1);
        }
        const int i = wy * BX + lane;  // the last two curl columns
        if (i < 2 * VW_H) {
            const int ry = i >> 1, rx = 2 * BX + (i & 1);
            sw[ry][rx] = curl_at(sv, rx + 1, ry + 1);
        }
    } else {
        for (int i = wy * BX + lane; i < VW_H * VW_W; i += BX * BY) {
            const int ry = i / VW_W, rx = i % VW_W;
            // curl at the clamped grid position, from its clamped neighbours,
            // read at that position's staged velocity
            const int gx = min(max(x0 - 1 + rx, 0), g.W - 1), gy = min(max(y0 - 1 + ry, 0), g.H - 1);
            sw[ry][rx] = curl_at(sv, gx - x0 + 2, gy - y0 + 2);
        }
    }
    __syncthreads();
    const float vort = sp->vorticity, dt = sp->dt;
    const int tx = 2 * lane;
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const int ty = wy + k * BY;
        const int x = x0 + tx, y = y0 + ty;
        if (INTERIOR) {
            const float2 a = *reinterpret_cast<const float2*>(&sw[ty + 1][tx]);      // wl0, wc0
            const float2 b = *reinterpret_cast<const float2*>(&sw[ty + 1][tx + 2]);  // wc1, wr1
            const float4 v = *reinterpret_cast<const float4*>(&sv[ty + 2][tx + 2]);
            const float2 o0 = confine(a.x, b.x, sw[ty][tx + 1], sw[ty + 2][tx + 1], a.y,
                                      make_float2(v.x, v.y), vort, dt);
            const float2 o1 = confine(a.y, b.y, sw[ty][tx + 2], sw[ty + 2][tx + 2], b.x,
                                      make_float2(v.z, v.w), vort, dt);
            const int c = y * g.P + x;
            *reinterpret_cast<float4*>(vout + c) = make_float4(o0.x, o0.y, o1.x, o1.y);
            *reinterpret_cast<float2*>(w + c) = make_float2(a.y, b.x);
        } else {
            if (y >= g.H) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int xh = x + h, th = tx + h;
                if (xh >= g.W) continue;
                const int xl = max(xh - 1, 0) - x0 + 1, xr = min(xh + 1, g.W - 1) - x0 + 1;
                const int yb = max(y - 1, 0) - y0 + 1, yt = min(y + 1, g.H - 1) - y0 + 1;
                const float wc = sw[ty + 1][th + 1];
                const int c = y * g.P + xh;
                vout[c] = confine(sw[ty + 1][xl], sw[ty + 1][xr], sw[yb][th + 1], sw[yt][th + 1],
                                  wc, sv[ty + 2][th + 2], vort, dt);
                w[c] = wc;
            }
        }
    }
}

__global__ void __launch_bounds__(BX* BY)
    k_vorticity(const float2* __restrict__ vin, float2* __restrict__ vout, float* __restrict__ w,
                Grid g, const __grid_constant__ StepParams spv) {
    pdl_enter();
    __shared__ __align__(16) float2 sv[VV_H][VV_W];
    __shared__ __align__(16) float sw[VW_H][VW_W];
    const int x0 = blockIdx.x * VT_W, y0 = blockIdx.y * VT_H;
    const bool interior = x0 >= 2 && y0 >= 2 && x0 + VT_W + 2 <= g.W && y0 + VT_H + 2 <= g.H &&
                          (g.P & 1) == 0;
    if (interior)
        vorticity_tile<true>(vin, vout, w, g, &spv, sv, sw, x0, y0);
    else
        vorticity_tile<false>(vin, vout, w, g, &spv, sv, sw, x0, y0);
}

// Row-streaming 5-point stencils (divergence, gradient subtraction).  A warp
// owns 64 consecutive columns (two per lane, so every row is one 16-byte
// velocity load, one 8-byte scalar load and one 2-byte mask load per lane)
// and walks ST_ROWS rows down, keeping the rows above and below in
// registers; the left / right neighbours come from the adjacent lanes by
// shuffle, and the warp's two edge lanes load the one column beyond.  Each
// cell's arithmetic is cell_divergence / cell_subtract_gradient's, so the
// results are identical; these kernels need an even width (the host falls
// back to the per-cell kernels otherwise).
constexpr int ST_WARPS = 4, ST_COLS = 64 * ST_WARPS, ST_ROWS = 8;

struct VRow {  // velocity and obstacle flag of a lane's two cells
    float2 a, b;
    uint8_t ma, mb;
};

__device__ __forceinline__ VRow load_vrow(const float2* __restrict__ v,
                                          const uint8_t* __restrict__ mask, const Grid& g, int y,
                                          int c, bool mz) {
    y = min(max(y, 0), g.H - 1);
    VRow r;
    const float4 q = __ldg(reinterpret_cast<const float4*>(v + (size_t)y * g.P + c));
    r.a = make_float2(q.x, q.y);
    r.b = make_float2(q.z, q.w);
    if (mz) {
        r.ma = r.mb = 0;
    } else {
        const uint16_t m = __ldg(reinterpret_cast<const uint16_t*>(mask + (size_t)y * g.P + c));
        r.ma = (uint8_t)(m & 0xff);
        r.mb = (uint8_t)(m >> 8);
    }
    return r;
}

__global__ void __launch_bounds__(32 * ST_WARPS)
    k_divergence_st(const float2* __restrict__ v, const uint8_t* __restrict__ mask,
                    float* __restrict__ div, uint8_t* __restrict__ flags, float* __restrict__ p1,
                    Grid g, const __grid_constant__ StepParams spv,
                    const __grid_constant__ TileMarks tm) {
    pdl_enter();
    const StepParams* sp = &spv;
    clear_marks(tm);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = blockIdx.x * ST_COLS + warp * 64 + 2 * lane;  // this lane's first column
    const int y0 = blockIdx.y * ST_ROWS;
    const bool live = c < g.W;  // W even: c + 1 < W too
    const int cc = live ? c : g.W - 2;  // dead lanes load a valid pair
    const bool mz = sp->mask_zero != 0;
    const unsigned FULL = 0xffffffffu;
    VRow up = load_vrow(v, mask, g, y0 - 1, cc, mz);
    VRow mid = load_vrow(v, mask, g, y0, cc, mz);
    const int y1 = min(y0 + ST_ROWS, g.H);
    int near_lo = INT_MAX, near_hi = -1;  // rows of this lane with a cell next to an obstacle
    for (int y = y0; y < y1; ++y) {
        const VRow dn = load_vrow(v, mask, g, y + 1, cc, mz);
        // left neighbour of column c (clamped), right neighbour of c + 1
        float lx = __shfl_up_sync(FULL, mid.b.x, 1);
        uint8_t lm = (uint8_t)__shfl_up_sync(FULL, (int)mid.mb, 1);
        float rx = __shfl_down_sync(FULL, mid.a.x, 1);
        uint8_t rm = (uint8_t)__shfl_down_sync(FULL, (int)mid.ma, 1);
        const size_t row = (size_t)y * g.P;
        if (lane == 0) {
            const int xl = max(cc - 1, 0);
            lx = __ldg(v + row + xl).x;
            lm = mz ? 0 : __ldg(mask + row + xl);
        }
        if (lane == 31 || cc + 2 >= g.W) {
            const int xr = min(cc + 2, g.W - 1);
            rx = __ldg(v + row + xr).x;
            rm = mz ? 0 : __ldg(mask + row + xr);
        }
        if (live) {
            // cell c: left = lx/lm, right = c+1; cell c+1: left = c, right = rx/rm
            const bool ol0 = lm != 0, or0 = mid.mb != 0, ob0 = up.ma != 0, ot0 = dn.ma != 0;
            const bool ol1 = mid.ma != 0, or1 = rm != 0, ob1 = up.mb != 0, ot1 = dn.mb != 0;
            const float b0 = 0.5f * (((or0 ? 0.0f : mid.b.x) - (ol0 ? 0.0f : lx)) +
                                     ((ot0 ? 0.0f : dn.a.y) - (ob0 ? 0.0f : up.a.y)));
            const float b1 = 0.5f * (((or1 ? 0.0f : rx) - (ol1 ? 0.0f : mid.a.x)) +
                                     ((ot1 ? 0.0f : dn.b.y) - (ob1 ? 0.0f : up.b.y)));
            *reinterpret_cast<float2*>(div + row + c) = make_float2(b0, b1);
            uint8_t f0 = 0, f1 = 0;
            if (c == 0 || ol0) f0 |= NB_L;
            if (or0) f0 |= NB_R;
            if (y == 0 || ob0) f0 |= NB_B;
            if (y == g.H - 1 || ot0) f0 |= NB_T;
            if (ol1) f1 |= NB_L;
            if (c + 1 == g.W - 1 || or1) f1 |= NB_R;
            if (y == 0 || ob1) f1 |= NB_B;
            if (y == g.H - 1 || ot1) f1 |= NB_T;
            *reinterpret_cast<uint16_t*>(flags + row + c) = (uint16_t)(f0 | (f1 << 8));
            if (ol0 | or0 | ob0 | ot0 | ol1 | or1 | ob1 | ot1) {
                near_lo = min(near_lo, y);
                near_hi = y;
            }
            if (p1)
                *reinterpret_cast<float2*>(p1 + row + c) =
                    make_float2((0.0f - b0) * 0.25f, (0.0f - b1) * 0.25f);
        }
        up = mid;
        mid = dn;
    }
    if (tm.mark) {
        // bounding box of this warp's cells next to an obstacle
        const bool near = near_hi >= 0;
        const int ylo = __reduce_min_sync(FULL, near ? near_lo : INT_MAX);
        const int yhi = __reduce_max_sync(FULL, near ? near_hi : -1);
        const int xlo = __reduce_min_sync(FULL, near ? c : INT_MAX);
        const int xhi = __reduce_max_sync(FULL, near ? c + 1 : -1);
        if (lane == 0 && yhi >= 0) mark_tiles(tm, xlo, xhi, ylo, yhi);
    }
}

__global__ void __launch_bounds__(32 * ST_WARPS)
    k_subtract_gradient_st(const float2* __restrict__ vin, float2* __restrict__ vout,
                           const float* __restrict__ p, const uint8_t* __restrict__ flags, Grid g) {
    pdl_enter();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = blockIdx.x * ST_COLS + warp * 64 + 2 * lane;
    const int y0 = blockIdx.y * ST_ROWS;
    const bool live = c < g.W;
    const int cc = live ? c : g.W - 2;
    const unsigned FULL = 0xffffffffu;
    const bool edge_l = lane == 0, edge_r = lane == 31 || cc + 2 >= g.W;
    auto prow = [&](int y) {
        y = min(max(y, 0), g.H - 1);
        return __ldg(reinterpret_cast<const float2*>(p + (size_t)y * g.P + cc));
    };
    // one row's own loads: velocity pair, flags pair, and the pressure one
    // column beyond the warp on the edge lanes
    struct RowIn {
        float4 q;
        uint16_t fw;
        float lp, rp;
    };
    auto load_row = [&](int y) {
        RowIn r;
        const size_t row = (size_t)y * g.P;
        r.q = *reinterpret_cast<const float4*>(vin + row + cc);
        r.fw = *reinterpret_cast<const uint16_t*>(flags + row + cc);
        r.lp = edge_l ? __ldg(p + row + max(cc - 1, 0)) : 0.0f;
        r.rp = edge_r ? __ldg(p + row + min(cc + 2, g.W - 1)) : 0.0f;
        return r;
    };
    const int y1 = min(y0 + ST_ROWS, g.H);
    // rows y0 - 1 .. y0 + 1 of pressure and row y0's own loads up front; each
    // iteration then issues the next row's loads before computing its own
    float2 up = prow(y0 - 1), mid = prow(y0), dn = prow(y0 + 1);
    RowIn cur = load_row(y0);
    for (int y = y0; y < y1; ++y) {
        float2 dn2 = dn;
        RowIn nxt = cur;
        if (y + 1 < y1) {
            dn2 = prow(y + 2);
            nxt = load_row(y + 1);
        }
        const size_t row = (size_t)y * g.P;
        float lp = __shfl_up_sync(FULL, mid.y, 1);
        float rp = __shfl_down_sync(FULL, mid.x, 1);
        if (edge_l) lp = cur.lp;
        if (edge_r) rp = cur.rp;
        if (live) {
            const uint8_t f0 = (uint8_t)(cur.fw & 0xff), f1 = (uint8_t)(cur.fw >> 8);
            float2 v0 = make_float2(cur.q.x, cur.q.y), v1 = make_float2(cur.q.z, cur.q.w);
            {
                const float pc = mid.x;
                const float x1 = (f0 & NB_L) ? pc : lp;
                const float x2 = (f0 & NB_R) ? pc : mid.y;
                const float yb = (f0 & NB_B) ? pc : up.x;
                const float yt = (f0 & NB_T) ? pc : dn.x;
                v0.x -= 0.5f * (x2 - x1);
                v0.y -= 0.5f * (yt - yb);
            }
            {
                const float pc = mid.y;
                const float x1 = (f1 & NB_L) ? pc : mid.x;
                const float x2 = (f1 & NB_R) ? pc : rp;
                const float yb = (f1 & NB_B) ? pc : up.y;
                const float yt = (f1 & NB_T) ? pc : dn.y;
                v1.x -= 0.5f * (x2 - x1);
                v1.y -= 0.5f * (yt - yb);
            }
            *reinterpret_cast<float4*>(vout + row + c) = make_float4(v0.x, v0.y, v1.x, v1.y);
        }
        up = mid;
        mid = dn;
        dn = dn2;
        cur = nxt;
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
               const __grid_constant__ StepParams spv, double* __restrict__ partials) {
    const StepParams* sp = &spv;
    ResidSums rs;
    const int total = g.W * g.H;  // at most 32768^2 = 2^30 cells
    const int base = blockIdx.x * RES_THREADS * RES_CELLS_PER_THREAD + threadIdx.x;
    const bool mz = sp->mask_zero != 0;
    CellWalk w(base, g.W);
#pragma unroll
    for (int k = 0; k < RES_CELLS_PER_THREAD; ++k) {
        const int lin = base + k * RES_THREADS;
        if (lin < total) {
            const Nbr n = nbrs_at(g, w.x, w.y);
            if (mz || !mask[n.c]) {
                const uint8_t f = flags[n.c];
                const float pc = p[n.c];
                rs.add(div[n.c], pc, (f & NB_L) ? pc : p[n.l], (f & NB_R) ? pc : p[n.r],
                       (f & NB_B) ? pc : p[n.b], (f & NB_T) ? pc : p[n.t]);
            }
        }
        w.advance(RES_THREADS, g.W);
    }
    __shared__ double s_part[RES_THREADS / 32][5];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    rs.warp_sum();
    if (lane == 0) rs.to_double(s_part[wid]);
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
// Each thread takes RES_CELLS_PER_THREAD cells, as k_residual does.
__global__ void __launch_bounds__(RES_THREADS)
    k_residual_labels(const float* __restrict__ p, const float* __restrict__ div,
                      const uint8_t* __restrict__ flags, const int* __restrict__ labels, Grid g,
                      double* __restrict__ sums) {
    const int total = g.W * g.H;  // at most 32768^2 = 2^30 cells
    const int base = blockIdx.x * RES_THREADS * RES_CELLS_PER_THREAD + threadIdx.x;
    // each thread sums its cells per run of one label and adds a run to the
    // label's sums when the label changes (only at region boundaries)
    int cur = -1;
    ResidSums rs;
    double v[5];
    CellWalk w(base, g.W);
#pragma unroll
    for (int k = 0; k < RES_CELLS_PER_THREAD; ++k) {
        const int lin = base + k * RES_THREADS;
        const int lab = lin < total ? labels[lin] : -1;
        if (lab >= 0) {
            if (lab != cur) {
                if (cur >= 0) {
                    rs.to_double(v);
#pragma unroll
                    for (int j = 0; j < 5; ++j) atomicAdd(sums + (size_t)cur * 5 + j, v[j]);
                    rs = ResidSums();
                }
                cur = lab;
            }
            const Nbr n = nbrs_at(g, w.x, w.y);
            const uint8_t f = flags[n.c];
            const float pc = p[n.c];
            rs.add(div[n.c], pc, (f & NB_L) ? pc : p[n.l], (f & NB_R) ? pc : p[n.r],
                   (f & NB_B) ? pc : p[n.b], (f & NB_T) ? pc : p[n.t]);
        }
        w.advance(RES_THREADS, g.W);
    }
    // a warp whose threads hold one label (or none) sums it with shuffles;
    // the block then adds each run of consecutive warps with one label as one
    // atomic per value (the sums are a few addresses every block shares)
    __shared__ double s_part[RES_THREADS / 32][5];
    __shared__ int s_lab[RES_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int l0 = __reduce_max_sync(0xffffffffu, cur);
    if (__all_sync(0xffffffffu, cur == l0 || cur < 0)) {
        rs.warp_sum();
        if (lane == 0) {
            rs.to_double(s_part[wid]);
            s_lab[wid] = l0;
        }
    } else {
        if (cur >= 0) {
            rs.to_double(v);
#pragma unroll
            for (int j = 0; j < 5; ++j) atomicAdd(sums + (size_t)cur * 5 + j, v[j]);
        }
        if (lane == 0) s_lab[wid] = -1;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        int run = -1;
        double acc = 0.0;
        for (int w = 0; w < RES_THREADS / 32; ++w) {
            const int l = s_lab[w];
            if (l < 0) continue;
            if (l != run) {
                if (run >= 0) atomicAdd(sums + (size_t)run * 5 + threadIdx.x, acc);
                run = l;
                acc = 0.0;
            }
            acc += s_part[w][threadIdx.x];
        }
        if (run >= 0) atomicAdd(sums + (size_t)run * 5 + threadIdx.x, acc);
    }
}

// One block of 256 threads: each thread sums every 256th block's partials,
// then the warps and the block reduce (FP64 throughput on one SM bounds this
// kernel, so few threads: the work is the partials' additions).
constexpr int RES_FINAL_THREADS = 256;

__global__ void __launch_bounds__(RES_FINAL_THREADS)
    k_residual_final(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    __shared__ double s[RES_FINAL_THREADS / 32][5];
    double acc[5] = {0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nblocks; b += RES_FINAL_THREADS)
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
        for (int w = 0; w < RES_FINAL_THREADS / 32; ++w) t += s[w][threadIdx.x];
        out[threadIdx.x] = t;
    }
}

}  // namespace

cudaError_t launch_residual_labels(const float* p, const float* div, const uint8_t* flags,
                                   const int* labels, int n_labels, Grid g, double* sums,
                                   cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(sums, 0, (size_t)n_labels * 5 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    const long total = (long)g.W * g.H;
    const long per_block = (long)RES_THREADS * RES_CELLS_PER_THREAD;
    k_residual_labels<<<(unsigned)((total + per_block - 1) / per_block), RES_THREADS, 0, st>>>(
        p, div, flags, labels, g, sums);
    return cudaGetLastError();
}

bool pdl_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("NATRIX_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

cudaError_t launch_obstacles(uint8_t* mask, Grid g, const ShapeOp* ops, int n, int fresh,
                             cudaStream_t st) {
    if (n < 0 || n > kMaxOpsPerLaunch) return cudaErrorInvalidValue;
    const dim3 grid((g.W + BX - 1) / BX, (g.H + BY * FORCE_ROWS - 1) / (BY * FORCE_ROWS));
    const bool pdl = pdl_enabled();
    if (n <= 16)
        return launch_kernel(pdl, k_obstacles<16>, grid, dim3(BX, BY), 0, st, mask, g,
                             op_block<ShapeOp, 16>(ops, n), fresh);
    if (n <= 64)
        return launch_kernel(pdl, k_obstacles<64>, grid, dim3(BX, BY), 0, st, mask, g,
                             op_block<ShapeOp, 64>(ops, n), fresh);
    return launch_kernel(pdl, k_obstacles<kMaxOpsPerLaunch>, grid, dim3(BX, BY), 0, st, mask, g,
                         op_block<ShapeOp, kMaxOpsPerLaunch>(ops, n), fresh);
}

// Blocks (BX x BY*FORCE_ROWS cells) a density op can reach: its footprint's
// bounding box with two cells of margin (the in-kernel cull keeps one).
// Returns false when the list would not fit (launch the full grid then).
bool density_force_tiles(const ForceOp* ops, int n, Grid gd, ForceTiles* tl) {
    const int th = BY * FORCE_ROWS;
    const int tx = (gd.W + BX - 1) / BX, ty = (gd.H + th - 1) / th;
    if ((long)tx * ty > 65536) return false;
    std::vector<uint8_t> hit((size_t)tx * ty, 0);
    for (int k = 0; k < n; ++k) {
        const ForceOp& op = ops[k];
        float reach;
        int y_end = gd.H;
        if (op.kind == FORCE_GAUSS)
            reach = 3.0f * op.r;
        else if (op.kind == FORCE_CONE_DENSITY) {
            reach = op.r;
            y_end = op.rows < gd.H ? op.rows : gd.H;
        } else
            continue;
        if (!(reach >= 0.0f) || y_end <= 0) continue;
        const double cx = (double)op.px * gd.W, cy = (double)op.py * gd.H, rr = (double)reach + 2.0;
        const double fx0 = std::max(cx - rr, 0.0), fx1 = std::min(cx + rr, (double)(gd.W - 1));
        const double fy0 = std::max(cy - rr, 0.0), fy1 = std::min(cy + rr, (double)(y_end - 1));
        if (!(fx0 <= fx1) || !(fy0 <= fy1)) continue;
        for (int j = (int)fy0 / th; j <= (int)fy1 / th; ++j)
            for (int i = (int)fx0 / BX; i <= (int)fx1 / BX; ++i) hit[(size_t)j * tx + i] = 1;
    }
    tl->n = 0;
    tl->tiles_x = tx;
    for (size_t t = 0; t < hit.size(); ++t)
        if (hit[t]) {
            if (tl->n == kMaxRasterBlocks) return false;
            tl->id[tl->n++] = (uint16_t)t;
        }
    return true;
}

template <int CAP>
cudaError_t launch_density_tiles(float* rho, Grid gd, const ForceOp* ops, int n,
                                 const ForceTiles& tl, cudaStream_t st) {
    if (tl.n == 0) return cudaSuccess;
    return launch_kernel(pdl_enabled(), k_forcing_tiles<CAP>, dim3(tl.n), dim3(BX, BY), 0, st,
                         rho, gd, op_block<ForceOp, CAP>(ops, n), tl);
}

bool shape_blocks(const ShapeOp* ops, int n, Grid g, uint8_t* hit) {
    const int tx = (g.W + kRasterBlock - 1) / kRasterBlock;
    for (int k = 0; k < n; ++k) {
        const ShapeOp& op = ops[k];
        if (op.kind != SHAPE_CIRCLE) return false;  // triangles are never culled
        // a cell is marked when its distance to the centre is <= r
        if (!(op.a[2] >= 0.0f)) continue;
        const double cx = (double)op.a[0] * g.W, cy = (double)op.a[1] * g.H;
        const double rr = (double)op.a[2] + 2.0;
        const double fx0 = std::max(cx - rr, 0.0), fx1 = std::min(cx + rr, (double)(g.W - 1));
        const double fy0 = std::max(cy - rr, 0.0), fy1 = std::min(cy + rr, (double)(g.H - 1));
        if (!(fx0 <= fx1) || !(fy0 <= fy1)) continue;
        for (int j = (int)fy0 / kRasterBlock; j <= (int)fy1 / kRasterBlock; ++j)
            for (int i = (int)fx0 / kRasterBlock; i <= (int)fx1 / kRasterBlock; ++i)
                hit[(size_t)j * tx + i] = 1;
    }
    return true;
}

cudaError_t launch_obstacles_blocks(uint8_t* mask, Grid g, const ShapeOp* ops, int n, int fresh,
                                    const uint16_t* ids, int n_ids, cudaStream_t st) {
    if (n < 0 || n > kMaxOpsPerLaunch || n_ids < 0 || n_ids > kMaxRasterBlocks)
        return cudaErrorInvalidValue;
    if (n_ids == 0) return cudaSuccess;
    ForceTiles tl;
    tl.n = n_ids;
    tl.tiles_x = (g.W + kRasterBlock - 1) / kRasterBlock;
    for (int i = 0; i < n_ids; ++i) tl.id[i] = ids[i];
    const bool pdl = pdl_enabled();
    if (n <= 16)
        return launch_kernel(pdl, k_obstacles_blocks<16>, dim3(n_ids), dim3(BX, BY), 0, st, mask, g,
                             op_block<ShapeOp, 16>(ops, n), fresh, tl);
    if (n <= 64)
        return launch_kernel(pdl, k_obstacles_blocks<64>, dim3(n_ids), dim3(BX, BY), 0, st, mask, g,
                             op_block<ShapeOp, 64>(ops, n), fresh, tl);
    return launch_kernel(pdl, k_obstacles_blocks<kMaxOpsPerLaunch>, dim3(n_ids), dim3(BX, BY), 0,
                         st, mask, g, op_block<ShapeOp, kMaxOpsPerLaunch>(ops, n), fresh, tl);
}

// Blocks holding a cell that a velocity op may change (its footprint box, two
// cells wider than the in-kernel tests: the cone's radius, the Gaussian's 3r
// cut), plus the edge blocks when the border is zeroed.  false when a list
// holds no velocity op or more blocks than a launch can carry.
bool velocity_force_tiles(const ForceOp* ops, int n, Grid gv, bool border, ForceTiles* tl) {
    const int th = BY * FORCE_ROWS;
    const int tx = (gv.W + BX - 1) / BX, ty = (gv.H + th - 1) / th;
    if ((long)tx * ty > 65536) return false;
    std::vector<uint8_t> hit((size_t)tx * ty, 0);
    bool any_velocity = false;
    for (int k = 0; k < n; ++k) {
        const ForceOp& op = ops[k];
        float reach;
        if (op.kind == FORCE_GAUSS)
            reach = 3.0f * op.r;
        else if (op.kind == FORCE_CONE_VELOCITY)
            reach = op.r;
        else
            return false;
        any_velocity = true;
        // a negative or NaN reach changes no cell (the kernel's tests fail)
        if (!(reach >= 0.0f)) continue;
        const double cx = (double)op.px * gv.W, cy = (double)op.py * gv.H, rr = (double)reach + 2.0;
        const double fx0 = std::max(cx - rr, 0.0), fx1 = std::min(cx + rr, (double)(gv.W - 1));
        const double fy0 = std::max(cy - rr, 0.0), fy1 = std::min(cy + rr, (double)(gv.H - 1));
        if (!(fx0 <= fx1) || !(fy0 <= fy1)) continue;
        for (int j = (int)fy0 / th; j <= (int)fy1 / th; ++j)
            for (int i = (int)fx0 / BX; i <= (int)fx1 / BX; ++i) hit[(size_t)j * tx + i] = 1;
    }
    if (!any_velocity) return false;
    if (border) {
        for (int i = 0; i < tx; ++i) hit[i] = hit[(size_t)(ty - 1) * tx + i] = 1;
        for (int j = 0; j < ty; ++j) hit[(size_t)j * tx] = hit[(size_t)j * tx + tx - 1] = 1;
    }
    tl->n = 0;
    tl->tiles_x = tx;
    for (size_t t = 0; t < hit.size(); ++t)
        if (hit[t]) {
            if (tl->n == kMaxRasterBlocks) return false;
            tl->id[tl->n++] = (uint16_t)t;
        }
    return true;
}

template <int CAP>
cudaError_t launch_velocity_tiles(float2* vel, Grid gv, const ForceOp* ops, int n,
                                  const ForceTiles& tl, int zero_border, cudaStream_t st) {
    if (tl.n == 0) return cudaSuccess;
    return launch_kernel(pdl_enabled(), k_vforcing_tiles<CAP>, dim3(tl.n), dim3(BX, BY), 0, st,
                         vel, gv, op_block<ForceOp, CAP>(ops, n), tl, zero_border);
}

bool launch_forcing_sparse(float2* vel, Grid gv, const ForceOp* ops, int n, int zero_border,
                           cudaStream_t st, cudaError_t* err) {
    *err = cudaSuccess;
    if (n < 1 || n > kMaxOpsPerLaunch || !vel) return false;
    // Below 1024 blocks the whole-grid launch is one or a few waves and the
    // block list costs more host time than it saves (256x256, 8 splats:
    // 40.0 us per step whole-grid, 42.6 us listed); above half the blocks
    // the advection's clamps cost more than the blocks skipped.
    const long blocks = (long)((gv.W + BX - 1) / BX) * ((gv.H + BY * FORCE_ROWS - 1) / (BY * FORCE_ROWS));
    if (blocks < 1024) return false;
    ForceTiles tl;
    if (!velocity_force_tiles(ops, n, gv, zero_border != 0, &tl) || 2L * tl.n > blocks) return false;
    if (n <= 16)
        *err = launch_velocity_tiles<16>(vel, gv, ops, n, tl, zero_border, st);
    else if (n <= 64)
        *err = launch_velocity_tiles<64>(vel, gv, ops, n, tl, zero_border, st);
    else
        *err = launch_velocity_tiles<kMaxOpsPerLaunch>(vel, gv, ops, n, tl, zero_border, st);
    return true;
}

cudaError_t launch_forcing(float2* vel, Grid gv, float* rho, Grid gd, const ForceOp* ops,
                           int n, int zero_border, cudaStream_t st) {
    if (n < 0 || n > kMaxOpsPerLaunch) return cudaErrorInvalidValue;
    if (!vel && rho) {
        ForceTiles tl;
        if (density_force_tiles(ops, n, gd, &tl)) {
            if (n <= 16) return launch_density_tiles<16>(rho, gd, ops, n, tl, st);
            if (n <= 64) return launch_density_tiles<64>(rho, gd, ops, n, tl, st);
            return launch_density_tiles<kMaxOpsPerLaunch>(rho, gd, ops, n, tl, st);
        }
    }
    Grid gg = vel ? gv : gd;
    if (vel && rho) gg = Grid{gv.W > gd.W ? gv.W : gd.W, gv.H > gd.H ? gv.H : gd.H, 0};
    const dim3 grid((gg.W + BX - 1) / BX, (gg.H + BY * FORCE_ROWS - 1) / (BY * FORCE_ROWS));
    const bool pdl = pdl_enabled();
    if (n <= 16)
        return launch_kernel(pdl, k_forcing<16>, grid, dim3(BX, BY), 0, st, vel, gv, rho, gd,
                             op_block<ForceOp, 16>(ops, n), zero_border);
    if (n <= 64)
        return launch_kernel(pdl, k_forcing<64>, grid, dim3(BX, BY), 0, st, vel, gv, rho, gd,
                             op_block<ForceOp, 64>(ops, n), zero_border);
    return launch_kernel(pdl, k_forcing<kMaxOpsPerLaunch>, grid, dim3(BX, BY), 0, st, vel, gv,
                         rho, gd, op_block<ForceOp, kMaxOpsPerLaunch>(ops, n), zero_border);
}

cudaError_t launch_advect(const float2* vin, float2* vout, const uint8_t* mask, Grid g,
                          const StepParams& sp, bool border_zeroed, cudaStream_t st,
                          bool clamp_on_read) {
    if (clamp_on_read) {
        if (sp.has_borders && !border_zeroed) return cudaErrorInvalidValue;
        return launch_kernel(pdl_enabled(), k_advect<false, true>, grid_cpt(g), dim3(BX, BY), 0,
                             st, vin, vout, mask, g, sp);
    }
    if (sp.has_borders && !border_zeroed)
        return launch_kernel(pdl_enabled(), k_advect<true>, grid_cpt(g), dim3(BX, BY), 0, st, vin,
                             vout, mask, g, sp);
    return launch_kernel(pdl_enabled(), k_advect<false>, grid_cpt(g), dim3(BX, BY), 0, st, vin,
                         vout, mask, g, sp);
}

cudaError_t launch_vorticity(const float2* vin, float2* vout, float* w, Grid g,
                             const StepParams& sp, cudaStream_t st) {
    return launch_kernel(pdl_enabled(), k_vorticity,
                         dim3((g.W + VT_W - 1) / VT_W, (g.H + VT_H - 1) / VT_H), dim3(BX, BY), 0,
                         st, vin, vout, w, g, sp);
}

cudaError_t launch_viscosity(const float2* vin, float2* vout, Grid g, const StepParams& sp,
                             cudaStream_t st) {
    return launch_kernel(pdl_enabled(), k_viscosity, grid_cpt(g), dim3(BX, BY), 0, st, vin, vout,
                         g, sp);
}

cudaError_t launch_divergence(const float2* v, const uint8_t* mask, float* div,
                              uint8_t* flags, float* p1, Grid g, const StepParams& sp,
                              const TileMarks& marks, cudaStream_t st) {
    if (marks.words > kMaxBalancedTiles / 32) return cudaErrorInvalidValue;
    if (g.W % 2 == 0 && g.W >= 2)
        return launch_kernel(pdl_enabled(), k_divergence_st,
                             dim3((g.W + ST_COLS - 1) / ST_COLS, (g.H + ST_ROWS - 1) / ST_ROWS),
                             dim3(32 * ST_WARPS), 0, st, v, mask, div, flags, p1, g, sp, marks);
    return launch_kernel(pdl_enabled(), k_divergence, grid_cpt(g), dim3(BX, BY), 0, st, v, mask,
                         div, flags, p1, g, sp, marks);
}

cudaError_t launch_subtract_gradient(const float2* vin, float2* vout, const float* p,
                                     const uint8_t* flags, Grid g, cudaStream_t st) {
    if (g.W % 2 == 0 && g.W >= 2)
        return launch_kernel(pdl_enabled(), k_subtract_gradient_st,
                             dim3((g.W + ST_COLS - 1) / ST_COLS, (g.H + ST_ROWS - 1) / ST_ROWS),
                             dim3(32 * ST_WARPS), 0, st, vin, vout, p, flags, g);
    return launch_kernel(pdl_enabled(), k_subtract_gradient, grid_cpt(g), dim3(BX, BY), 0, st, vin,
                         vout, p, flags, g);
}

cudaError_t launch_density_advect(const float* rin, float* rout, Grid gd, const float2* v,
                                  const uint8_t* mask, Grid gv, const StepParams& sp,
                                  cudaStream_t st) {
    const auto pow2 = [](int n) { return (n & (n - 1)) == 0; };
    if (gd.W == gv.W && gd.H == gv.H && pow2(gd.W) && pow2(gd.H))
        return launch_kernel(pdl_enabled(), k_density_advect_same, grid_cpt(gd), dim3(BX, BY), 0,
                             st, rin, rout, gd, v, mask, gv, sp);
    return launch_kernel(pdl_enabled(), k_density_advect, grid_cpt(gd), dim3(BX, BY), 0, st, rin,
                         rout, gd, v, mask, gv, sp);
}

int residual_partials(Grid g) {
    const long total = (long)g.W * g.H;
    const long per = (long)RES_THREADS * RES_CELLS_PER_THREAD;
    return (int)((total + per - 1) / per);
}

cudaError_t launch_residual(const float* p, const float* div, const uint8_t* mask,
                            const uint8_t* flags, Grid g, const StepParams& sp,
                            double* partials, double* out, cudaStream_t st) {
    const int nb = residual_partials(g);
    k_residual<<<nb, RES_THREADS, 0, st>>>(p, div, mask, flags, g, sp, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_residual_final<<<1, RES_FINAL_THREADS, 0, st>>>(partials, nb, out);
    return cudaGetLastError();
}

}  // namespace natrix
