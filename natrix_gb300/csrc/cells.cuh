// Per-cell and per-block bodies of the solver kernels, shared by the
// single-grid kernels (solver_kernels.cu) and the batched multi-simulation
// kernels (batch.cu) so both evaluate the same expressions.
//
// Arithmetic contract: see common.cuh (-fmad=false, IEEE div/sqrt, shader
// operation order).
#pragma once

#include "kernels.cuh"

namespace natrix {

constexpr int BX = 32, BY = 8;

// ---------------------------------------------------------------- obstacles
// shader.AddCircleObstacle.comp:17-37 and shader.AddTriangleObstacle.comp:19-52,
// all queued shapes in one pass; `fresh` = start from an empty mask (the
// reference clears the obstacle buffer at the end of every update).
__device__ __forceinline__ float tri_sign(float p1x, float p1y, float p2x, float p2y,
                                          float p3x, float p3y) {
    return ((p1x - p3x) * (p2y - p3y)) - ((p2x - p3x) * (p1y - p3y));
}

// Block-level culling: warp 0 compacts, in order, the indices of the ops
// whose conservative footprint (expanded by one cell) meets this block's
// cells; `test(k)` decides.  Every cell then walks the kept list only.
template <class Test>
__device__ __forceinline__ int cull_ops(int n, int* kept, Test test) {
    __shared__ int s_n;
    if (threadIdx.y == 0) {
        int count = 0;
        for (int base = 0; base < n; base += 32) {
            const int k = base + threadIdx.x;
            const bool keep = k < n && test(k);
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) kept[count + __popc(m & ((1u << threadIdx.x) - 1u))] = k;
            count += __popc(m);
        }
        if (threadIdx.x == 0) s_n = count;
    }
    __syncthreads();
    return s_n;
}

// Does a disc of radius `r` around (cx, cy) meet the cell box [x0,x1]x[y0,y1]?
// (conservative: one cell of margin)
__device__ __forceinline__ bool disc_meets_box(float cx, float cy, float r, int x0, int x1,
                                               int y0, int y1) {
    const float dx = fmaxf(fmaxf((float)x0 - cx, cx - (float)x1), 0.0f);
    const float dy = fmaxf(fmaxf((float)y0 - cy, cy - (float)y1), 0.0f);
    const float rr = r + 1.0f;
    return dx * dx + dy * dy <= rr * rr;
}

// ROWS: rows of cells per thread (the block covers BX x TBY*ROWS cells, the
// shape list is loaded and culled once for all of them); the block has BX x
// TBY threads.
template <int ROWS = 1, int TBY = BY>
__device__ __forceinline__ void block_obstacles(uint8_t* __restrict__ mask, Grid g,
                                                const ShapeOp* __restrict__ ops, int n, int fresh,
                                                int bx0, int by0) {
    __shared__ ShapeOp s_ops[kMaxOpsPerLaunch];
    __shared__ int s_kept[kMaxOpsPerLaunch];
    const int tid = threadIdx.y * BX + threadIdx.x;
    for (int i = tid; i < n; i += BX * TBY) s_ops[i] = ops[i];
    __syncthreads();
    const int bx1 = bx0 + BX - 1, by1 = by0 + TBY * ROWS - 1;
    const int nk = cull_ops(n, s_kept, [&](int k) {
        const ShapeOp& op = s_ops[k];
        // triangles are never culled: the reference's same-sign test marks
        // cells far outside a degenerate (zero-area) triangle's bounding box
        if (op.kind != SHAPE_CIRCLE) return true;
        return disc_meets_box(op.a[0] * (float)g.W, op.a[1] * (float)g.H, op.a[2], bx0, bx1,
                              by0, by1);
    });
    if (nk == 0 && !fresh) return;
    const int x = bx0 + threadIdx.x;
    if (x >= g.W) return;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const int y = by0 + threadIdx.y + r * TBY;
        if (y >= g.H) break;
        const size_t i = (size_t)y * g.P + x;
        uint8_t m = fresh ? 0 : mask[i];
        for (int kk = 0; kk < nk; ++kk) {
            const ShapeOp& op = s_ops[s_kept[kk]];
            if (op.kind == SHAPE_CIRCLE) {
                const float spx = op.a[0] * (float)g.W, spy = op.a[1] * (float)g.H;
                const float dx = spx - (float)x, dy = spy - (float)y;
                if (sqrtf(dx * dx + dy * dy) <= op.a[2]) m = 1;  // vec2(1, 0), both branches
            } else {
                const float ptx = (float)x / (float)g.W, pty = (float)y / (float)g.H;
                const bool b1 = tri_sign(ptx, pty, op.a[0], op.a[1], op.a[2], op.a[3]) < 0.0f;
                const bool b2 = tri_sign(ptx, pty, op.a[2], op.a[3], op.a[4], op.a[5]) < 0.0f;
                const bool b3 = tri_sign(ptx, pty, op.a[4], op.a[5], op.a[0], op.a[1]) < 0.0f;
                if (b1 == b2 && b2 == b3) m = (uint8_t)((m & ~3) | (op.is_static ? 2 : 1));
            }
        }
        mask[i] = m;
    }
}

// ------------------------------------------------------------------ forcing
// Queued forcing ops applied in order to each cell of the velocity grid
// and/or the density grid (both when they have the same size).
//  FORCE_CONE_VELOCITY  shader.AddVelocity.comp:26-35: inside the radius
//      v += V*(r - d)/r, then every cell is clamped to [-1, 1].
//  FORCE_GAUSS          w = exp(-d^2/r^2) inside 3r: v = clamp(v + w V, -1, 1)
//      for every cell, rho = clamp(rho + w s, 0, 255) inside the cut-off.
//  FORCE_CONE_DENSITY   demo/shaders/shader.AddParticle.comp:25-34 on rows the
//      reference's dispatch reaches.
// Ops whose footprint misses the block are culled.  For velocity that is
// exact because a velocity op outside its footprint is a clamp, and clamp is
// idempotent: the only trace a culled or missing op leaves is the clamp of the
// first velocity op when it does not touch the cell (a cell whose first op
// touches it starts from the unclamped value, as in the reference).
__device__ __forceinline__ bool op_is_velocity(int kind) {
    return kind == FORCE_CONE_VELOCITY || kind == FORCE_GAUSS;
}

// zero_border: after the ops, write the border cells of the velocity grid as
// zero (shader.InitBoundaries.comp, which the reference dispatches next when
// the step starts); only meaningful when the list holds a velocity op, since
// then every cell is written.
template <int ROWS = 1, int TBY = BY, bool CG = false>
__device__ __forceinline__ void block_forcing(float2* __restrict__ vel, Grid gv,
                                              float* __restrict__ rho, Grid gd,
                                              const ForceOp* __restrict__ ops, int n, int bx0,
                                              int by0, bool zero_border = false) {
    __shared__ ForceOp s_ops[kMaxOpsPerLaunch];
    __shared__ int s_kept[kMaxOpsPerLaunch];
    const int x = bx0 + threadIdx.x;
    // the velocity rows' loads go out before the op list is staged and culled
    // (several DRAM reads in flight per thread while the block prologue runs)
    float2 va[ROWS];
    if (vel) {
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const int y = by0 + threadIdx.y + r * TBY;
            if (x < gv.W && y < gv.H) va[r] = ldp<CG>(vel + (size_t)y * gv.P + x);
        }
    }
    const int tid = threadIdx.y * BX + threadIdx.x;
    for (int i = tid; i < n; i += BX * TBY) s_ops[i] = ops[i];
    __syncthreads();
    const int bx1 = bx0 + BX - 1, by1 = by0 + TBY * ROWS - 1;
    if (vel) {
        int first_vel = -1;
        for (int k = 0; k < n; ++k)
            if (op_is_velocity(s_ops[k].kind)) {
                first_vel = k;
                break;
            }
        const int nk = cull_ops(n, s_kept, [&](int k) {
            const ForceOp& op = s_ops[k];
            if (op.kind == FORCE_CONE_VELOCITY)
                return disc_meets_box(op.px * (float)gv.W, op.py * (float)gv.H, op.r, bx0, bx1,
                                      by0, by1);
            if (op.kind == FORCE_GAUSS)
                return disc_meets_box(op.px * (float)gv.W, op.py * (float)gv.H, 3.0f * op.r, bx0,
                                      bx1, by0, by1);
            return false;
        });
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const int y = by0 + threadIdx.y + r * TBY;
            if (first_vel < 0 || x >= gv.W || y >= gv.H) continue;
            const size_t i = (size_t)y * gv.P + x;
            float2 a = va[r];
            // the first velocity op culled for this block: it clamps the cell
            bool started = !(nk > 0 && s_kept[0] == first_vel);
            if (started) {
                a.x = clampf(a.x, -1.0f, 1.0f);
                a.y = clampf(a.y, -1.0f, 1.0f);
            }
            for (int kk = 0; kk < nk; ++kk) {
                const ForceOp& op = s_ops[s_kept[kk]];
                bool hit = false;
                float ax = a.x, ay = a.y;
                if (op.kind == FORCE_CONE_VELOCITY) {
                    const float spx = op.px * (float)gv.W, spy = op.py * (float)gv.H;
                    const float dx = spx - (float)x, dy = spy - (float)y;
                    const float len = sqrtf(dx * dx + dy * dy);
                    if (len <= op.r) {
                        ax = a.x + op.vx * (op.r - len) / op.r;
                        ay = a.y + op.vy * (op.r - len) / op.r;
                        hit = true;
                    }
                } else {
                    const float cx = op.px * (float)gv.W, cy = op.py * (float)gv.H;
                    const float dx = (float)x - cx, dy = (float)y - cy;
                    const float cut = 3.0f * op.r;
                    if (dx * dx + dy * dy <= cut * cut) {
                        const float w = nx_expf(-(dx * dx + dy * dy) / (op.r * op.r));
                        ax = a.x + w * op.vx;
                        ay = a.y + w * op.vy;
                        hit = true;
                    }
                }
                if (hit || !started) {
                    a.x = clampf(ax, -1.0f, 1.0f);
                    a.y = clampf(ay, -1.0f, 1.0f);
                    started = true;
                }
            }
            if (zero_border && (x == 0 || x == gv.W - 1 || y == 0 || y == gv.H - 1))
                a = make_float2(0.0f, 0.0f);
            vel[i] = a;
        }
        __syncthreads();  // s_kept is reused below
    }
    if (rho) {
        const int nk = cull_ops(n, s_kept, [&](int k) {
            const ForceOp& op = s_ops[k];
            if (op.kind == FORCE_GAUSS)
                return disc_meets_box(op.px * (float)gd.W, op.py * (float)gd.H, 3.0f * op.r, bx0,
                                      bx1, by0, by1);
            if (op.kind == FORCE_CONE_DENSITY)
                return by0 < op.rows && disc_meets_box(op.px * (float)gd.W, op.py * (float)gd.H,
                                                       op.r, bx0, bx1, by0, by1);
            return false;
        });
        float ra[ROWS];
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const int y = by0 + threadIdx.y + r * TBY;
            if (nk != 0 && x < gd.W && y < gd.H) ra[r] = ldp<CG>(rho + (size_t)y * gd.P + x);
        }
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const int y = by0 + threadIdx.y + r * TBY;
            if (nk == 0 || x >= gd.W || y >= gd.H) continue;
            const size_t i = (size_t)y * gd.P + x;
            float a = ra[r];
            for (int kk = 0; kk < nk; ++kk) {
                const ForceOp& op = s_ops[s_kept[kk]];
                if (op.kind == FORCE_GAUSS) {
                    const float cx = op.px * (float)gd.W, cy = op.py * (float)gd.H;
                    const float dx = (float)x - cx, dy = (float)y - cy;
                    const float cut = 3.0f * op.r;
                    if (dx * dx + dy * dy <= cut * cut) {
                        const float w = nx_expf(-(dx * dx + dy * dy) / (op.r * op.r));
                        a = clampf(a + w * op.s, 0.0f, 255.0f);
                    }
                } else if (y < op.rows) {
                    const float spx = op.px * (float)gd.W, spy = op.py * (float)gd.H;
                    const float dx = spx - (float)x, dy = spy - (float)y;
                    const float len = sqrtf(dx * dx + dy * dy);
                    if (len <= op.r) a = clampf(a + op.s * (op.r - len) / op.r, 0.0f, 255.0f);
                }
            }
            rho[i] = a;
        }
    }
}

// ---------------------------------------------------------------- advection
// shader.AdvectVelocity.comp:19-51, with shader.InitBoundaries.comp:11-35
// fused: the reference zeroes the border of the read buffer in place before
// advecting, so border cells read as zero here (centre and gathers alike).
// CG: loads through L2 (see ldf in common.cuh).
template <bool CG = false>
__device__ __forceinline__ float2 vel_at(const float2* __restrict__ v, const Grid& g, int x,
                                         int y, bool zero_border) {
    if (zero_border && (x == 0 || x == g.W - 1 || y == 0 || y == g.H - 1))
        return make_float2(0.0f, 0.0f);
    return ldf<CG>(v + (size_t)y * g.P + x);
}

// Backtrace position of a cell from its own velocity.
__device__ __forceinline__ Corners advect_corners(float2 vel, int x, int y, const Grid& g,
                                                  const StepParams* __restrict__ sp) {
    const float dt = sp->dt, speed = sp->speed;
    const float fx = (float)x - vel.x * dt * speed;
    const float fy = (float)y - vel.y * dt * speed;
    return corners(fx, fy, g.W, g.H);
}

// The arithmetic after the bilinear gathers (shader.AdvectVelocity.comp:38-50).
__device__ __forceinline__ float2 advect_mix(float2 lt, float2 rt, float2 lb, float2 rb,
                                             const Corners& c, float diss) {
    const float h1x = mixf(lt.x, rt.x, c.dx), h1y = mixf(lt.y, rt.y, c.dx);
    const float h2x = mixf(lb.x, rb.x, c.dx), h2y = mixf(lb.y, rb.y, c.dx);
    const float sx = mixf(h2x, h1x, c.dy), sy = mixf(h2y, h1y, c.dy);
    return make_float2(clampf(sx * diss, -1.0f, 1.0f), clampf(sy * diss, -1.0f, 1.0f));
}

template <bool CG = false>
__device__ __forceinline__ void cell_advect(const float2* __restrict__ vin, float2* __restrict__ vout,
             const uint8_t* __restrict__ mask, Grid g, const StepParams* __restrict__ sp, int x, int y) {
    if (x >= g.W || y >= g.H) return;
    const size_t i = (size_t)y * g.P + x;
    const bool zb = sp->has_borders != 0;
    if (!sp->mask_zero && ldp<CG>(mask + i)) {
        vout[i] = make_float2(0.0f, 0.0f);
        return;
    }
    const float2 vel = vel_at<CG>(vin, g, x, y, zb);
    const Corners c = advect_corners(vel, x, y, g, sp);
    const float2 lt = vel_at<CG>(vin, g, c.lo_x, c.hi_y, zb);
    const float2 rt = vel_at<CG>(vin, g, c.hi_x, c.hi_y, zb);
    const float2 lb = vel_at<CG>(vin, g, c.lo_x, c.lo_y, zb);
    const float2 rb = vel_at<CG>(vin, g, c.hi_x, c.lo_y, zb);
    vout[i] = advect_mix(lt, rt, lb, rb, c, sp->dissipation);
}

// Clamped neighbour coordinates (natrix/core/shaders/originals/common.sh:9-19).
struct Nbr {
    size_t c, l, r, b, t;
};
__device__ __forceinline__ Nbr nbrs(const Grid& g, int x, int y) {
    Nbr n;
    const int xl = x > 0 ? x - 1 : 0, xr = x < g.W - 1 ? x + 1 : g.W - 1;
    const int yb = y > 0 ? y - 1 : 0, yt = y < g.H - 1 ? y + 1 : g.H - 1;
    n.c = (size_t)y * g.P + x;
    n.l = (size_t)y * g.P + xl;
    n.r = (size_t)y * g.P + xr;
    n.b = (size_t)yb * g.P + x;
    n.t = (size_t)yt * g.P + x;
    return n;
}

// The same clamped indices from one row offset (no per-neighbour multiply).
__device__ __forceinline__ Nbr nbrs_at(const Grid& g, int x, int y) {
    Nbr n;
    n.c = (size_t)y * g.P + x;
    n.l = x > 0 ? n.c - 1 : n.c;
    n.r = x < g.W - 1 ? n.c + 1 : n.c;
    n.b = y > 0 ? n.c - g.P : n.c;
    n.t = y < g.H - 1 ? n.c + g.P : n.c;
    return n;
}

// ------------------------------------------------------ vorticity confinement
// shader.CalcVorticity.comp:13-27.
template <bool CG = false>
__device__ __forceinline__ void cell_calc_vorticity(const float2* __restrict__ v, float* __restrict__ w, Grid g, int x, int y) {
    if (x >= g.W || y >= g.H) return;
    const Nbr n = nbrs(g, x, y);
    const float2 vl = ldf<CG>(v + n.l), vr = ldf<CG>(v + n.r), vb = ldf<CG>(v + n.b),
                 vt = ldf<CG>(v + n.t);
    w[n.c] = 0.5f * ((vr.y - vl.y) - (vt.x - vb.x));
}

// shader.ApplyVorticity.comp:19-40.
template <bool CG = false>
__device__ __forceinline__ void cell_apply_vorticity(const float2* __restrict__ vin, float2* __restrict__ vout,
                      const float* __restrict__ w, Grid g, const StepParams* __restrict__ sp, int x, int y) {
    if (x >= g.W || y >= g.H) return;
    const Nbr n = nbrs(g, x, y);
    const float wl = ldf<CG>(w + n.l), wr = ldf<CG>(w + n.r), wb = ldf<CG>(w + n.b),
                wt = ldf<CG>(w + n.t), wc = ldf<CG>(w + n.c);
    float fx = 0.5f * (fabsf(wt) - fabsf(wb));
    float fy = 0.5f * (fabsf(wr) - fabsf(wl));
    const float eps = 2.4414e-4f;
    const float d = fx * fx + fy * fy;
    const float m = eps > d ? eps : d;
    const float rs = 1.0f / sqrtf(m);  // inversesqrt, correctly rounded
    fx = fx * rs;
    fy = fy * rs;
    const float s = sp->vorticity * wc;
    fx = fx * (s * 1.0f);
    fy = fy * (s * -1.0f);
    const float dt = sp->dt;
    const float2 v = ldp<CG>(vin + n.c);
    vout[n.c] = make_float2(v.x + fx * dt, v.y + fy * dt);
}

// ---------------------------------------------------------------- viscosity
// shader.Viscosity.comp:17-32, one smoothing sweep.
template <bool CG = false>
__device__ __forceinline__ void cell_viscosity(const float2* __restrict__ vin, float2* __restrict__ vout, Grid g,
                const StepParams* __restrict__ sp, int x, int y) {
    if (x >= g.W || y >= g.H) return;
    const Nbr n = nbrs(g, x, y);
    const float alpha = sp->alpha, rbeta = sp->rbeta;
    const float2 a = ldf<CG>(vin + n.l), b = ldf<CG>(vin + n.r), c = ldf<CG>(vin + n.b),
                 d = ldf<CG>(vin + n.t), e = ldf<CG>(vin + n.c);
    vout[n.c] = make_float2((a.x + b.x + c.x + d.x + e.x * alpha) * rbeta,
                            (a.y + b.y + c.y + d.y + e.y * alpha) * rbeta);
}

// --------------------------------------------------------------- divergence
// shader.Divergence.comp:15-41.  Also writes, for the pressure sweeps, the
// neighbour-substitution flags and the first Jacobi sweep from the zero guess:
// with p = 0 everywhere, shader.Poisson.comp:37 gives (0+0+0+0 - b)*0.25,
// which is (0 - b)*0.25 bit for bit; the reference's clear of the pressure
// buffer (fluid_simulator.py:235-248) is thereby folded away.
__device__ __forceinline__ float divergence_of(float x1, float x2, float y1, float y2) {
    return 0.5f * ((x2 - x1) + (y2 - y1));
}

// Neighbour-substitution flags of a cell: wall or obstacle neighbour.
__device__ __forceinline__ uint8_t nb_flags(int x, int y, const Grid& g, bool ol, bool orr,
                                            bool ob, bool ot) {
    uint8_t f = 0;
    if (x == 0 || ol) f |= NB_L;
    if (x == g.W - 1 || orr) f |= NB_R;
    if (y == 0 || ob) f |= NB_B;
    if (y == g.H - 1 || ot) f |= NB_T;
    return f;
}

template <bool CG = false>
__device__ __forceinline__ void cell_divergence(const float2* __restrict__ v, const uint8_t* __restrict__ mask,
                 float* __restrict__ div, uint8_t* __restrict__ flags, float* __restrict__ p1,
                 Grid g, const StepParams* __restrict__ sp, int x, int y) {
    if (x >= g.W || y >= g.H) return;
    const Nbr n = nbrs(g, x, y);
    const bool mz = sp->mask_zero != 0;
    const bool ol = !mz && ldp<CG>(mask + n.l), orr = !mz && ldp<CG>(mask + n.r);
    const bool ob = !mz && ldp<CG>(mask + n.b), ot = !mz && ldp<CG>(mask + n.t);
    const float x1 = ol ? 0.0f : ldf<CG>(v + n.l).x;
    const float x2 = orr ? 0.0f : ldf<CG>(v + n.r).x;
    const float y1 = ob ? 0.0f : ldf<CG>(v + n.b).y;
    const float y2 = ot ? 0.0f : ldf<CG>(v + n.t).y;
    const float b = divergence_of(x1, x2, y1, y2);
    div[n.c] = b;
    flags[n.c] = nb_flags(x, y, g, ol, orr, ob, ot);
    if (p1) p1[n.c] = (0.0f - b) * 0.25f;
}

// -------------------------------------------------------- gradient subtract
// shader.SubtractGradient.comp:17-47 (same neighbour rule as the sweep).
__device__ __forceinline__ float2 subtract_gradient_of(float2 vel, uint8_t f, float pc, float pl,
                                                       float pr, float pb, float pt) {
    const float x1 = (f & NB_L) ? pc : pl;
    const float x2 = (f & NB_R) ? pc : pr;
    const float y1 = (f & NB_B) ? pc : pb;
    const float y2 = (f & NB_T) ? pc : pt;
    vel.x -= 0.5f * (x2 - x1);
    vel.y -= 0.5f * (y2 - y1);
    return vel;
}

template <bool CG = false>
__device__ __forceinline__ void cell_subtract_gradient(const float2* __restrict__ vin, float2* __restrict__ vout,
                        const float* __restrict__ p, const uint8_t* __restrict__ flags,
                        Grid g, int x, int y) {
    if (x >= g.W || y >= g.H) return;
    const Nbr n = nbrs(g, x, y);
    const uint8_t f = ldp<CG>(flags + n.c);
    const float pc = ldf<CG>(p + n.c);
    const float pl = (f & NB_L) ? pc : ldf<CG>(p + n.l);
    const float pr = (f & NB_R) ? pc : ldf<CG>(p + n.r);
    const float pb = (f & NB_B) ? pc : ldf<CG>(p + n.b);
    const float pt = (f & NB_T) ? pc : ldf<CG>(p + n.t);
    vout[n.c] = subtract_gradient_of(ldp<CG>(vin + n.c), f, pc, pl, pr, pb, pt);
}

// --------------------------------------------------------- density advection
// demo/shaders/shader.AdvectParticle.comp:21-71: the density grid (its own
// size) is advected by the velocity sampled at the matching position of the
// velocity grid, scaled by the grid-size ratio.
__device__ __forceinline__ Corners density_vel_corners(int x, int y, const Grid& gd,
                                                       const Grid& gv) {
    const float nx = (float)x / (float)gd.W * (float)gv.W;
    const float ny = (float)y / (float)gd.H * (float)gv.H;
    return corners(nx, ny, gv.W, gv.H);
}

// On a cell centre (equal grid sizes) the four corners are one cell and the
// bilinear mix of a finite velocity returns it (a -0 comes back as +0, which
// the backtrace x - u*dt*speed cannot tell apart), so one load gives the same
// result.
__device__ __forceinline__ bool on_centre(const Corners& cv) {
    return cv.lo_x == cv.hi_x && cv.lo_y == cv.hi_y && cv.dx == 0.0f && cv.dy == 0.0f;
}

// Backtrace position in the density grid from the sampled velocity.
__device__ __forceinline__ Corners density_corners(float2 u, int x, int y, const Grid& gd,
                                                   const Grid& gv,
                                                   const StepParams* __restrict__ sp) {
    u.x = u.x * ((float)gd.W / (float)gv.W);
    u.y = u.y * ((float)gd.H / (float)gv.H);
    const float dt = sp->dt, speed = sp->d_speed;
    const float fx = (float)x - u.x * dt * speed;
    const float fy = (float)y - u.y * dt * speed;
    return corners(fx, fy, gd.W, gd.H);
}

template <bool CG = false>
__device__ __forceinline__ void cell_density_advect(const float* __restrict__ rin, float* __restrict__ rout, Grid gd,
                     const float2* __restrict__ v, const uint8_t* __restrict__ mask, Grid gv,
                     const StepParams* __restrict__ sp, int x, int y) {
    if (x >= gd.W || y >= gd.H) return;
    const size_t i = (size_t)y * gd.P + x;
    const float nx = (float)x / (float)gd.W * (float)gv.W;
    const float ny = (float)y / (float)gd.H * (float)gv.H;
    if (!sp->mask_zero) {
        const size_t oi = (size_t)(unsigned)ny * gv.P + (unsigned)nx;
        if (ldp<CG>(mask + oi)) {
            rout[i] = 0.0f;
            return;
        }
    }
    const Corners cv = density_vel_corners(x, y, gd, gv);
    const float2 u = on_centre(cv) ? ldf<CG>(v + (size_t)cv.lo_y * gv.P + cv.lo_x)
                                   : sample_vel<CG>(v, gv.P, cv);
    const Corners c = density_corners(u, x, y, gd, gv, sp);
    rout[i] = sample_scalar<CG>(rin, gd.P, c) * sp->d_dissipation;
}

}  // namespace natrix
