// Batched simulations: many independent FluidSimulator + density grids of
// uneven sizes advanced together, one launch per phase for all of them, the
// whole step captured once as a CUDA graph and replayed.  No reference
// counterpart (the reference runs one simulator per FluidSimulator object);
// each simulation of a batch gives the same result, bit for bit, as a single
// simulator stepped through the same calls.
//
// Layout: one device arena holds every simulation's fields (same per-field
// layout as a single simulator).  Per-cell phases run one 32x8 block per
// (simulation, block) item of a flat list; each block reads its simulation's
// descriptor and runs the same cell bodies as the single-grid kernels
// (cells.cuh).  Pressure sweeps run as batched tile launches: launch m holds,
// for every simulation that still has sweeps to do, all its tiles with
// min(S, remaining) sweeps, in the tile configuration of the simulation's
// size class (config and S per class are set by natrix_batch_set_tuning,
// which the Python autotuner drives).
//
// Per step the host uploads one block (dt, per-simulation op ranges, forcing
// ops, obstacle shapes) and launches the graph; the graph's first kernel
// copies dt and the obstacle state into every descriptor.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../../include/natrix.h"
#include "cells.cuh"
#include "jacobi_tile.cuh"

using namespace natrix;

namespace {

constexpr int kClasses = 3;  // size classes: side <= 128, <= 256, larger

int size_class(const Grid& g) {
    const int side = g.W > g.H ? g.W : g.H;
    return side <= 128 ? 0 : (side <= 256 ? 1 : 2);
}

struct BatchSimDesc {
    Grid g;
    StepParams sp;
    float2* vel[3];
    float* p[2];
    float* div;
    float* vort;
    uint8_t* mask;
    uint8_t* flags;
    float* rho[2];
    int vort_in, vort_out, visc_in, visc_out, last, p_final;
};

struct StepHeader {
    float dt;
    int n_sims;
    int rho_cur;  // density buffer holding the state (persistent step kernel)
    int pad;
    unsigned long long epoch;  // steps since the work list was built
    unsigned long long pad2;
};

// item = {sim, block x origin, block y origin, 0}
__global__ void k_batch_prepare(BatchSimDesc* __restrict__ d, const StepHeader* __restrict__ h,
                                const int* __restrict__ shape_count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= h->n_sims) return;
    d[i].sp.dt = h->dt;
    // obstacles are reset every step: a simulation without shapes this step
    // has an empty mask
    d[i].sp.mask_zero = shape_count[i] == 0 ? 1 : 0;
}

__global__ void __launch_bounds__(BX* BY)
    k_batch_obstacles(const int4* __restrict__ items, const BatchSimDesc* __restrict__ d,
                      const ShapeOp* __restrict__ shapes, const int* __restrict__ begin,
                      const int* __restrict__ count) {
    const int4 it = items[blockIdx.x];
    const int n = count[it.x];
    if (n == 0) return;
    const BatchSimDesc& s = d[it.x];
    block_obstacles(s.mask, s.g, shapes + begin[it.x], n, 1, it.y, it.z);
}

__global__ void __launch_bounds__(BX* BY)
    k_batch_forcing(const int4* __restrict__ items, BatchSimDesc* __restrict__ d, int rho_cur,
                    const ForceOp* __restrict__ ops, const int* __restrict__ begin,
                    const int* __restrict__ count) {
    const int4 it = items[blockIdx.x];
    const int n = count[it.x];
    if (n == 0) return;
    const BatchSimDesc& s = d[it.x];
    block_forcing(s.vel[0], s.g, s.rho[rho_cur], s.g, ops + begin[it.x], n, it.y, it.z);
}

#define BATCH_CELL_KERNEL(name, call)                                                     \
    __global__ void __launch_bounds__(BX* BY)                                             \
        name(const int4* __restrict__ items, const BatchSimDesc* __restrict__ d, int rc) { \
        const int4 it = items[blockIdx.x];                                                \
        const BatchSimDesc& s = d[it.x];                                                  \
        const int x = it.y + threadIdx.x, y = it.z + threadIdx.y;                         \
        (void)rc;                                                                         \
        call;                                                                             \
    }

BATCH_CELL_KERNEL(k_batch_advect, cell_advect(s.vel[0], s.vel[1], s.mask, s.g, &s.sp, x, y))
BATCH_CELL_KERNEL(k_batch_calc_vort, cell_calc_vorticity(s.vel[s.vort_in], s.vort, s.g, x, y))
BATCH_CELL_KERNEL(k_batch_apply_vort, cell_apply_vorticity(s.vel[s.vort_in], s.vel[s.vort_out],
                                                           s.vort, s.g, &s.sp, x, y))
BATCH_CELL_KERNEL(k_batch_visc, cell_viscosity(s.vel[s.visc_in], s.vel[s.visc_out], s.g, &s.sp,
                                               x, y))
BATCH_CELL_KERNEL(k_batch_divergence, cell_divergence(s.vel[s.last], s.mask, s.div, s.flags,
                                                      s.p[0], s.g, &s.sp, x, y))
BATCH_CELL_KERNEL(k_batch_subgrad, cell_subtract_gradient(s.vel[s.last], s.vel[0],
                                                          s.p[s.p_final], s.flags, s.g, x, y))
// The fluid update resets the obstacles before the density update runs
// (natrix/core/fluid_simulator.py:267-280), so density advection sees none.
__global__ void __launch_bounds__(BX* BY)
    k_batch_density(const int4* __restrict__ items, const BatchSimDesc* __restrict__ d, int rc) {
    const int4 it = items[blockIdx.x];
    const BatchSimDesc& s = d[it.x];
    StepParams sp = s.sp;
    sp.mask_zero = 1;
    cell_density_advect(s.rho[rc], s.rho[1 - rc], s.g, s.vel[0], s.mask, s.g, &sp,
                        it.y + threadIdx.x, it.z + threadIdx.y);
}

// ----------------------------------------------------------------------------
// Persistent step kernel: the whole batch step in one launch.
//
// The host lays the step out as a list of work items in dependency order:
// for every phase (forcing, advection, vorticity, viscosity, divergence,
// Jacobi chunks 1..M, gradient subtraction, density advection), every
// simulation's items of that phase (bands of rows for the per-cell phases,
// tiles for the sweeps).  Resident CTAs claim items in list order from a
// global counter (the next claim is issued while the current item runs).  An
// item first waits until every item of its simulation's previous phase has
// finished (a per-(simulation, phase) completion counter), runs the same
// arithmetic as the per-phase kernels, then counts itself done.  Dependencies
// only point to earlier items, so the earliest unfinished item can always
// run and the kernel cannot deadlock, whatever the number of resident CTAs.
//
// Counters never reset: the claim counter and the completion counters grow by
// a fixed amount per step, and the step's epoch (in the step block) gives the
// targets.  A wait that runs out (about a second) sets status bit 2 and the
// item runs anyway, so the launch always ends.
//
// Fields written earlier in the launch by other CTAs are read through L2
// (CG loads, coherent across SMs); the sweep tiles read them by TMA after a
// proxy fence.
enum StepItemKind : int {
    ITEM_FORCE = 0,
    ITEM_ADVECT,
    ITEM_CALC_VORT,
    ITEM_APPLY_VORT,
    ITEM_VISC,
    ITEM_DIV,
    ITEM_JACOBI,  // tile configuration in `config`
    ITEM_SUBGRAD,
    ITEM_DENSITY
};

// 48 bytes: three 16-byte cp.async copies move one into shared memory
struct StepItem {
    int kind;
    int sim;
    int a, b;    // per-cell items: rows [a, b); Jacobi: tile origin (a, b)
    int src;     // Jacobi: source pressure buffer
    int sweeps;  // Jacobi: sweeps of this chunk
    int config;  // Jacobi: tile configuration
    int wait;    // completion counter to wait on (-1: none)
    int need;    // items that counter gains per step
    int done;    // completion counter this item increments
    int pad[2];
};

static_assert(sizeof(StepItem) % 16 == 0, "StepItem moves in 16-byte copies");
constexpr int kStepThreadsY = 16;  // CTA of 32 x 16 threads (16 warps)
using TbStep = TbCfg<64, 32, 8, kStepThreadsY>;  // Tb's tile on 512 threads
static_assert(RtB::THREADS == 32 * kStepThreadsY && RtA::THREADS == 32 * kStepThreadsY,
              "register tiles run with the step kernel's 512 threads");

struct StepArgs {
    const StepItem* items;
    int n_items;
    int n_sims;
    const BatchSimDesc* desc;
    const JacobiBatchSim* jsims;
    unsigned long long* counters;
    unsigned long long* claim;
    const unsigned char* step;  // step block: header, op / shape ranges, ops, shapes
    size_t ops_off, shapes_off;
    int* status;
};

// A register tile of the step kernel.  `issued`: its copies were already
// issued (prefetched during the previous item).  Once the tile sits in
// registers, `prefetch()` may issue the next item's copies into the freed
// staging buffers.
template <class C, class Prefetch>
__device__ __forceinline__ void step_rt_tile(const TileJob& job, unsigned char* smem,
                                             uint64_t* bar, uint32_t parity, int* status,
                                             int tid, bool issued, Prefetch prefetch) {
    __shared__ int s_ok;
    if (tid == 0) {
        if (!issued) {
            fence_before_tma();
            issue_tile_loads<C>(smem, bar, job);
        }
        bool ok = wait_phase(bar, parity);
        if (!ok) {
            atomicOr(status, 1);
            wait_phase(bar, parity);
        }
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    if (s_ok) rt_tile_body<C>(job, smem, prefetch);
}

__device__ __forceinline__ void step_tb_tile(const TileJob& job, unsigned char* smem,
                                             uint64_t* bar, uint32_t parity, int* status,
                                             int tid) {
    using C = TbStep;
    __shared__ int s_ok;
    if (tid == 0) {
        fence_before_tma();
        mbar_expect_tx(bar, 2 * C::P_BYTES + C::F_BYTES);
        tma_load_2d(smem + C::OFF_A, job.p, job.tile_x - C::HXP, job.tile_y - C::HALO, bar);
        tma_load_2d(smem + C::OFF_D, job.d, job.tile_x - C::HXP, job.tile_y - C::HALO, bar);
        tma_load_2d(smem + C::OFF_F, job.f, job.tile_x - C::HXF, job.tile_y - C::HALO, bar);
        bool ok = wait_phase(bar, parity);
        if (!ok) {
            atomicOr(status, 1);
            wait_phase(bar, parity);
        }
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    if (s_ok) tb_tile_body<C>(job, smem);
}

// Per-cell phases of the step kernel (advection, divergence, gradient
// subtraction, density advection) on a band of rows [a, b) of one
// simulation.  Thread 0 brings the rows each phase reads into shared memory
// with bulk asynchronous copies (one copy per field: a band of full pitched
// rows is contiguous in global memory, and every field starts 256-byte
// aligned with 128-byte rows), plus the halo rows the stencils and samplers
// reach; the threads then compute from shared memory, one cell per thread
// at a time.  A bilinear sample outside the staged rows (a backtrace longer
// than the halo) reads global memory through L2.  The arithmetic is the cell
// bodies' own helpers (cells.cuh), so the values are the same.  Offsets are
// 32-bit: natrix_batch_create takes sides of at most 32768 cells, so a
// simulation's offsets stay below 2^30.
constexpr int kStageBytes = 192 * 1024;  // staging space of a band item
constexpr int kAdvectHalo = 2;           // rows staged beyond a band for the samplers

// Rows of a staged band for a simulation of row pitch P: the largest
// staging need per row is the gradient subtraction's 13 bytes per cell
// (velocity, pressure, flags) plus the halo rows.
// Widest row pitch whose band of one row and its halos fits the staging.
constexpr int kMaxStagedPitch = kStageBytes / (13 * (1 + 2 * kAdvectHalo)) / 32 * 32;
static_assert(kMaxStagedPitch >= 3008, "staging space for rows of 3008 cells");

inline int staged_band_rows(int P) {
    const int r = kStageBytes / (13 * P) - 2 * kAdvectHalo;
    return r < 1 ? 1 : (r > 64 ? 64 : r);
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Thread 0 issues up to three row-range copies on the step barrier and
// waits for them (bounded); every thread returns once they have landed.
struct RowCopy {
    unsigned char* dst;
    const unsigned char* src;
    uint32_t bytes;
};

__device__ __forceinline__ void stage_rows(const RowCopy* c, int n, uint64_t* bar,
                                           uint32_t* s_parity, int* status) {
    if (threadIdx.x + 32 * threadIdx.y == 0) {
        uint32_t total = 0;
        for (int k = 0; k < n; ++k) total += c[k].bytes;
        fence_before_tma();
        mbar_expect_tx(bar, total);
        for (int k = 0; k < n; ++k)
            if (c[k].bytes) bulk_copy(c[k].dst, c[k].src, c[k].bytes, bar);
        const uint32_t parity = *s_parity;
        *s_parity ^= 1u;
        if (!wait_phase(bar, parity)) {
            atomicOr(status, 1);
            wait_phase(bar, parity);
        }
    }
    __syncthreads();
}

// Rows [lo, hi) of a pitched field as a copy into shared memory at dst.
template <class T>
__device__ __forceinline__ RowCopy rows_of(unsigned char* dst, const T* field, const Grid& g,
                                           int lo, int hi) {
    return RowCopy{dst, reinterpret_cast<const unsigned char*>(field + (size_t)lo * g.P),
                   (uint32_t)((hi - lo) * g.P * sizeof(T))};
}

__device__ __forceinline__ int align_up_256(int b) { return (b + 255) / 256 * 256; }

// Obstacles and forcing of a band (rows [a, b), a multiple of 32 rows unless
// it is the grid's last): the obstacle raster writes the mask; when the
// band's velocity and density rows fit the staging space they are staged,
// the queued ops applied in shared memory by the forcing body (through a
// row-rebased pointer, so it indexes the staged rows with its grid
// coordinates) and the rows written back; wider bands read and write the
// fields in place (plain loads: forcing is a simulation's first phase in the
// launch, so no other CTA has written these rows yet).
constexpr int kForceRows = 2 * kStepThreadsY;  // rows per forcing block call

__device__ __forceinline__ void band_force(const BatchSimDesc* sd, int a, int b,
                                           const ShapeOp* shapes, int ns, const ForceOp* ops,
                                           int no, int rc, unsigned char* smem, uint64_t* bar,
                                           uint32_t* s_parity, int* status) {
    const Grid g = sd->g;
    if (ns)
        for (int by = a; by < b; by += kForceRows)
            for (int bx = 0; bx < g.W; bx += BX)
                block_obstacles<2, kStepThreadsY>(sd->mask, g, shapes, ns, 1, bx, by);
    if (!no) return;
    const int vbytes = align_up_256((b - a) * g.P * 8);
    if (vbytes + (b - a) * g.P * 4 > kStageBytes) {
        for (int by = a; by < b; by += kForceRows)
            for (int bx = 0; bx < g.W; bx += BX)
                block_forcing<2, kStepThreadsY, false>(sd->vel[0], g, sd->rho[rc], g, ops, no,
                                                       bx, by);
        return;
    }
    RowCopy c[2] = {rows_of(smem, sd->vel[0], g, a, b),
                    rows_of(smem + vbytes, sd->rho[rc], g, a, b)};
    stage_rows(c, 2, bar, s_parity, status);
    float2* sv = reinterpret_cast<float2*>(smem) - (size_t)a * g.P;
    float* sr = reinterpret_cast<float*>(smem + vbytes) - (size_t)a * g.P;
    for (int by = a; by < b; by += kForceRows)
        for (int bx = 0; bx < g.W; bx += BX)
            block_forcing<2, kStepThreadsY, false>(sv, g, sr, g, ops, no, bx, by);
    __syncthreads();
    // the staged rows back to global memory, 16 bytes per thread and access
    const int n4v = (b - a) * g.P / 2, n4r = (b - a) * g.P / 4;
    const float4* s4 = reinterpret_cast<const float4*>(smem);
    float4* v4 = reinterpret_cast<float4*>(sd->vel[0] + (size_t)a * g.P);
    for (int i = threadIdx.x + 32 * threadIdx.y; i < n4v; i += 32 * kStepThreadsY) v4[i] = s4[i];
    const float4* r4s = reinterpret_cast<const float4*>(smem + vbytes);
    float4* r4 = reinterpret_cast<float4*>(sd->rho[rc] + (size_t)a * g.P);
    for (int i = threadIdx.x + 32 * threadIdx.y; i < n4r; i += 32 * kStepThreadsY) r4[i] = r4s[i];
}

__device__ __forceinline__ void band_advect(const BatchSimDesc* sd, float dt, int mask_zero,
                                            int a, int b, unsigned char* smem, uint64_t* bar,
                                            uint32_t* s_parity, int* status) {
    const Grid g = sd->g;
    const int r0 = max(a - kAdvectHalo, 0), r1 = min(b + kAdvectHalo, g.H);
    const float2* vin = sd->vel[0];
    const float2* sv = reinterpret_cast<const float2*>(smem);
    const uint8_t* sm = smem + align_up_256((r1 - r0) * g.P * 8);
    RowCopy c[2] = {rows_of(smem, vin, g, r0, r1),
                    rows_of(smem + align_up_256((r1 - r0) * g.P * 8), sd->mask, g, a, b)};
    stage_rows(c, mask_zero ? 1 : 2, bar, s_parity, status);
    StepParams sp{};
    sp.dt = dt;
    sp.speed = sd->sp.speed;
    const float diss = sd->sp.dissipation;
    const bool zb = sd->sp.has_borders != 0;
    auto vel = [&](int x, int y) {
        if (zb && (x == 0 || x == g.W - 1 || y == 0 || y == g.H - 1))
            return make_float2(0.0f, 0.0f);
        return (y >= r0 && y < r1) ? sv[(y - r0) * g.P + x] : __ldcg(vin + y * g.P + x);
    };
    float2* vout = sd->vel[1];
    for (int y = a + (int)threadIdx.y; y < b; y += kStepThreadsY)
        for (int x = threadIdx.x; x < g.W; x += BX) {
            if (!mask_zero && sm[(y - a) * g.P + x]) {
                vout[y * g.P + x] = make_float2(0.0f, 0.0f);
                continue;
            }
            const Corners q = advect_corners(vel(x, y), x, y, g, &sp);
            vout[y * g.P + x] = advect_mix(vel(q.lo_x, q.hi_y), vel(q.hi_x, q.hi_y),
                                           vel(q.lo_x, q.lo_y), vel(q.hi_x, q.lo_y), q, diss);
        }
}

__device__ __forceinline__ void band_divergence(const BatchSimDesc* sd, int mask_zero, int a,
                                                int b, unsigned char* smem, uint64_t* bar,
                                                uint32_t* s_parity, int* status) {
    const Grid g = sd->g;
    const int r0 = max(a - 1, 0), r1 = min(b + 1, g.H);
    const float2* sv = reinterpret_cast<const float2*>(smem);
    const uint8_t* sm = smem + align_up_256((r1 - r0) * g.P * 8);
    RowCopy c[2] = {rows_of(smem, sd->vel[sd->last], g, r0, r1),
                    rows_of(smem + align_up_256((r1 - r0) * g.P * 8), sd->mask, g, r0, r1)};
    stage_rows(c, mask_zero ? 1 : 2, bar, s_parity, status);
    for (int y = a + (int)threadIdx.y; y < b; y += kStepThreadsY)
        for (int x = threadIdx.x; x < g.W; x += BX) {
            // clamped neighbours (common.sh:9-19) as staged offsets
            const int xl = x > 0 ? x - 1 : x, xr = x < g.W - 1 ? x + 1 : x;
            const int yb = y > 0 ? y - 1 : y, yt = y < g.H - 1 ? y + 1 : y;
            const int rc = (y - r0) * g.P, rb = (yb - r0) * g.P, rt = (yt - r0) * g.P;
            const bool ol = !mask_zero && sm[rc + xl], orr = !mask_zero && sm[rc + xr];
            const bool ob = !mask_zero && sm[rb + x], ot = !mask_zero && sm[rt + x];
            const float bv = divergence_of(ol ? 0.0f : sv[rc + xl].x, orr ? 0.0f : sv[rc + xr].x,
                                           ob ? 0.0f : sv[rb + x].y, ot ? 0.0f : sv[rt + x].y);
            const int o = y * g.P + x;
            sd->div[o] = bv;
            sd->flags[o] = nb_flags(x, y, g, ol, orr, ob, ot);
            sd->p[0][o] = (0.0f - bv) * 0.25f;
        }
}

__device__ __forceinline__ void band_subgrad(const BatchSimDesc* sd, int a, int b,
                                             unsigned char* smem, uint64_t* bar,
                                             uint32_t* s_parity, int* status) {
    const Grid g = sd->g;
    const int r0 = max(a - 1, 0), r1 = min(b + 1, g.H);
    const int vbytes = align_up_256((b - a) * g.P * 8);
    const int pbytes = align_up_256((r1 - r0) * g.P * 4);
    const float2* sv = reinterpret_cast<const float2*>(smem);
    const float* spp = reinterpret_cast<const float*>(smem + vbytes);
    const uint8_t* sf = smem + vbytes + pbytes;
    RowCopy c[3] = {rows_of(smem, sd->vel[sd->last], g, a, b),
                    rows_of(smem + vbytes, sd->p[sd->p_final], g, r0, r1),
                    rows_of(smem + vbytes + pbytes, sd->flags, g, a, b)};
    stage_rows(c, 3, bar, s_parity, status);
    float2* vout = sd->vel[0];
    for (int y = a + (int)threadIdx.y; y < b; y += kStepThreadsY)
        for (int x = threadIdx.x; x < g.W; x += BX) {
            const int xl = x > 0 ? x - 1 : x, xr = x < g.W - 1 ? x + 1 : x;
            const int yb = y > 0 ? y - 1 : y, yt = y < g.H - 1 ? y + 1 : y;
            const int rc = (y - r0) * g.P;
            const uint8_t f = sf[(y - a) * g.P + x];
            vout[y * g.P + x] = subtract_gradient_of(
                sv[(y - a) * g.P + x], f, spp[rc + x], spp[rc + xl], spp[rc + xr],
                spp[(yb - r0) * g.P + x], spp[(yt - r0) * g.P + x]);
        }
}

// Density advection on a density grid of the velocity grid's size (the batch
// keeps them equal); the obstacles are reset before it runs.
__device__ __forceinline__ void band_density(const BatchSimDesc* sd, float dt, int rc, int a,
                                             int b, unsigned char* smem, uint64_t* bar,
                                             uint32_t* s_parity, int* status) {
    const Grid g = sd->g;
    const int q0 = max(a - kAdvectHalo, 0), q1 = min(b + kAdvectHalo, g.H);  // density rows
    const int v0 = max(a - 1, 0), v1 = min(b + 1, g.H);                     // velocity rows
    const float* rin = sd->rho[rc];
    const float2* v = sd->vel[0];
    const int rbytes = align_up_256((q1 - q0) * g.P * 4);
    const float* sr = reinterpret_cast<const float*>(smem);
    const float2* sv = reinterpret_cast<const float2*>(smem + rbytes);
    RowCopy c[2] = {rows_of(smem, rin, g, q0, q1), rows_of(smem + rbytes, v, g, v0, v1)};
    stage_rows(c, 2, bar, s_parity, status);
    StepParams sp{};
    sp.dt = dt;
    sp.d_speed = sd->sp.d_speed;
    const float diss = sd->sp.d_dissipation;
    auto vel = [&](int x, int y) {
        return (y >= v0 && y < v1) ? sv[(y - v0) * g.P + x] : __ldcg(v + y * g.P + x);
    };
    auto rho = [&](int x, int y) {
        return (y >= q0 && y < q1) ? sr[(y - q0) * g.P + x] : __ldcg(rin + y * g.P + x);
    };
    float* rout = sd->rho[1 - rc];
    for (int y = a + (int)threadIdx.y; y < b; y += kStepThreadsY)
        for (int x = threadIdx.x; x < g.W; x += BX) {
            const Corners cv = density_vel_corners(x, y, g, g);
            float2 u;
            if (on_centre(cv)) {
                u = vel(cv.lo_x, cv.lo_y);
            } else {  // sample_vel's arithmetic
                const float2 lt = vel(cv.lo_x, cv.hi_y), rt = vel(cv.hi_x, cv.hi_y);
                const float2 lb = vel(cv.lo_x, cv.lo_y), rb = vel(cv.hi_x, cv.lo_y);
                const float h1x = mixf(lt.x, rt.x, cv.dx), h1y = mixf(lt.y, rt.y, cv.dx);
                const float h2x = mixf(lb.x, rb.x, cv.dx), h2y = mixf(lb.y, rb.y, cv.dx);
                u = make_float2(mixf(h2x, h1x, cv.dy), mixf(h2y, h1y, cv.dy));
            }
            const Corners q = density_corners(u, x, y, g, g, &sp);
            // sample_scalar's arithmetic
            const float h1 = mixf(rho(q.lo_x, q.hi_y), rho(q.hi_x, q.hi_y), q.dx);
            const float h2 = mixf(rho(q.lo_x, q.lo_y), rho(q.hi_x, q.lo_y), q.dx);
            rout[y * g.P + x] = mixf(h2, h1, q.dy) * diss;
        }
}

// Cells of rows [a, b), one cell per thread at a time (vorticity and
// viscosity items).
template <class F>
__device__ __forceinline__ void band_cells(int a, int b, int W, F f) {
    for (int y = a + (int)threadIdx.y; y < b; y += kStepThreadsY)
        for (int x = threadIdx.x; x < W; x += BX) f(x, y);
}

// A register-tile sweep item, item k of the list.  Thread 0 keeps the
// tile barrier's parity and the prefetch flag in shared memory (nothing of
// the item loop stays in registers across the sweep, which needs nearly all
// of them).  nk: the item this CTA claimed next (>= n_items: none).  When
// that next item is a tile of the same configuration whose dependency is
// already complete, its copies are issued into the staging buffers as soon
// as this tile sits in registers, and the flag tells the next item so.
// epoch1: the step's epoch + 1 (completion targets are epoch1 * need).
template <class C>
__device__ __forceinline__ void jacobi_item(int k, long long nk, const StepItem* items,
                                            int n_items, const JacobiBatchSim* jsims,
                                            const unsigned long long* counters,
                                            unsigned long long epoch1, unsigned char* smem,
                                            uint64_t* bar, uint32_t* s_parity, int* status,
                                            int* s_pref) {
    const int tid = threadIdx.x + 32 * threadIdx.y;
    const StepItem it = items[k];
    const JacobiBatchSim& js = jsims[it.sim];
    const TileJob job{&js.maps.p[it.src], &js.maps.div, &js.maps.flags, js.p[1 - it.src], js.g,
                      it.sweeps, it.a, it.b, nullptr, nullptr};
    bool issued = false;
    uint32_t parity = 0;
    if (tid == 0) {
        issued = *s_pref != 0;
        *s_pref = 0;
        parity = *s_parity;
        *s_parity ^= 1u;
    }
    step_rt_tile<C>(job, smem, bar, parity, status, tid, issued, [&] {
        if (tid != 0 || nk >= n_items) return;
        const StepItem nx = items[nk];
        if (nx.kind != ITEM_JACOBI || nx.config != it.config) return;
        if (nx.wait >= 0 &&
            ld_acquire_u64(counters + nx.wait) < epoch1 * (unsigned long long)nx.need)
            return;
        const JacobiBatchSim& ns = jsims[nx.sim];
        const TileJob nj{&ns.maps.p[nx.src], &ns.maps.div, &ns.maps.flags, ns.p[1 - nx.src],
                         ns.g, nx.sweeps, nx.a, nx.b, nullptr, nullptr};
        fence_before_tma();
        issue_tile_loads<C>(smem, bar, nj);
        *s_pref = 1;
    });
}

__device__ __forceinline__ void jacobi_tb_item(int k, const StepItem* items,
                                               const JacobiBatchSim* jsims, unsigned char* smem,
                                               uint64_t* bar, uint32_t* s_parity, int* status) {
    const int tid = threadIdx.x + 32 * threadIdx.y;
    const StepItem it = items[k];
    const JacobiBatchSim& js = jsims[it.sim];
    const TileJob job{&js.maps.p[it.src], &js.maps.div, &js.maps.flags, js.p[1 - it.src], js.g,
                      it.sweeps, it.a, it.b, nullptr, nullptr};
    uint32_t parity = 0;
    if (tid == 0) {
        parity = *s_parity;
        *s_parity ^= 1u;
    }
    step_tb_tile(job, smem, bar, parity, status, tid);
}

// Per-step values of the step block, kept in shared memory so no register
// holds them across the items.
struct StepShared {
    unsigned long long epoch, base;
    const int* op_begin;
    const int* op_count;
    const int* sh_begin;
    const int* sh_count;
    const ForceOp* ops;
    const ShapeOp* shapes;
    float dt;
    int rc;
};

__device__ __forceinline__ StepParams step_params(const BatchSimDesc* sd, const StepShared& ss,
                                                  int sim) {
    StepParams sp = sd->sp;
    sp.dt = ss.dt;
    // obstacles are reset every step: no shapes this step, empty mask
    sp.mask_zero = ss.sh_count[sim] == 0 ? 1 : 0;
    return sp;
}

// Completion signals of finished items, held back so that one release fence
// covers several (the fence waits for the CTA's stores to reach L2, about a
// microsecond).  Owned by thread 0.  Flushed when kPending items are held,
// before thread 0 waits on a counter that is not yet satisfied, and at the
// end: a CTA never spins while it holds a signal, so holding them cannot
// deadlock two CTAs that wait on each other's counters.
constexpr int kPending = 4;

struct PendingSignals {
    int idx[kPending];
    int n = 0;
    __device__ __forceinline__ void flush(unsigned long long* counters) {
        if (n == 0) return;
        // release pattern: every write of the held items (ordered before this
        // thread by the barrier that ended each of them), then the counts
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        for (int i = 0; i < n; ++i)
            asm volatile("red.relaxed.gpu.global.add.u64 [%0], 1;" ::"l"(counters + idx[i])
                         : "memory");
        n = 0;
    }
};

__global__ void __launch_bounds__(32 * kStepThreadsY, 1) k_batch_step(const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_item, s_pref;
    __shared__ long long s_next;
    __shared__ uint32_t s_parity;
    __shared__ StepShared ss;
    // the current item's descriptor and the next one's, copied ahead by
    // thread 0 (cp.async) while the current item runs
    __shared__ __align__(16) StepItem s_w[2];
    const int tid = threadIdx.x + 32 * threadIdx.y;
    if (tid == 0) {
        const StepHeader* hdr = reinterpret_cast<const StepHeader*>(a.step);
        ss.epoch = hdr->epoch;
        ss.rc = hdr->rho_cur;
        ss.dt = hdr->dt;
        ss.op_begin = reinterpret_cast<const int*>(a.step + sizeof(StepHeader));
        ss.op_count = ss.op_begin + a.n_sims;
        ss.sh_begin = ss.op_count + a.n_sims;
        ss.sh_count = ss.sh_begin + a.n_sims;
        ss.ops = reinterpret_cast<const ForceOp*>(a.step + a.ops_off);
        ss.shapes = reinterpret_cast<const ShapeOp*>(a.step + a.shapes_off);
        // every CTA claims until it draws an index past the list: n_items +
        // gridDim.x claims per step
        ss.base = ss.epoch * (unsigned long long)(a.n_items + gridDim.x);
        mbar_init(&s_bar, 1);
        fence_barrier_init();
        s_item = (int)(atomicAdd(a.claim, 1ull) - ss.base);
        if (s_item < a.n_items) s_w[0] = a.items[s_item];
        s_pref = 0;
        s_parity = 0;
    }
    __syncthreads();
    PendingSignals pend;  // thread 0's
    for (int cur = 0;; cur ^= 1) {
        const int k = s_item;
        if (k >= a.n_items) break;
        const StepItem& w = s_w[cur];
        unsigned long long next = 0;
        if (tid == 0) next = atomicAdd(a.claim, 1ull);  // in flight during the wait
        if (tid == 0) {
            if (w.wait >= 0) {
                const unsigned long long target = (ss.epoch + 1) * (unsigned long long)w.need;
                if (ld_acquire_u64(a.counters + w.wait) < target) {
                    pend.flush(a.counters);
                    if (!wait_counter(a.counters + w.wait, target)) atomicOr(a.status, 2);
                }
            }
            s_next = (long long)(next - ss.base);
            if (s_next < a.n_items) {
                const char* src = reinterpret_cast<const char*>(a.items + s_next);
                const unsigned dst = (unsigned)__cvta_generic_to_shared(&s_w[cur ^ 1]);
#pragma unroll
                for (int i = 0; i < (int)(sizeof(StepItem) / 16); ++i)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst + 16 * i),
                                 "l"(src + 16 * i)
                                 : "memory");
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        __syncthreads();  // s_item read by all; dependency satisfied
        const int kind = w.kind;
        const int sim = w.sim;
        const BatchSimDesc* sd = a.desc + sim;
        switch (kind) {
            case ITEM_FORCE:
                band_force(sd, w.a, w.b, ss.shapes + ss.sh_begin[sim],
                           ss.sh_count[sim], ss.ops + ss.op_begin[sim], ss.op_count[sim], ss.rc,
                           smem, &s_bar, &s_parity, a.status);
                break;
            case ITEM_ADVECT:
                band_advect(sd, ss.dt, ss.sh_count[sim] == 0 ? 1 : 0, w.a,
                            w.b, smem, &s_bar, &s_parity, a.status);
                break;
            case ITEM_CALC_VORT: {
                const Grid g = sd->g;
                band_cells(w.a, w.b, g.W, [&](int x, int y) {
                    cell_calc_vorticity<true>(sd->vel[sd->vort_in], sd->vort, g, x, y);
                });
                break;
            }
            case ITEM_APPLY_VORT: {
                const Grid g = sd->g;
                const StepParams sp = step_params(sd, ss, sim);
                band_cells(w.a, w.b, g.W, [&](int x, int y) {
                    cell_apply_vorticity<true>(sd->vel[sd->vort_in], sd->vel[sd->vort_out],
                                               sd->vort, g, &sp, x, y);
                });
                break;
            }
            case ITEM_VISC: {
                const Grid g = sd->g;
                const StepParams sp = step_params(sd, ss, sim);
                band_cells(w.a, w.b, g.W, [&](int x, int y) {
                    cell_viscosity<true>(sd->vel[sd->visc_in], sd->vel[sd->visc_out], g, &sp, x,
                                         y);
                });
                break;
            }
            case ITEM_DIV:
                band_divergence(sd, ss.sh_count[sim] == 0 ? 1 : 0, w.a, w.b,
                                smem, &s_bar, &s_parity, a.status);
                break;
            case ITEM_JACOBI: {
                const int config = w.config;
                const long long nk = s_next;
                if (config == JACOBI_RT_B)
                    jacobi_item<RtB>(k, nk, a.items, a.n_items, a.jsims, a.counters,
                                     ss.epoch + 1, smem, &s_bar, &s_parity, a.status, &s_pref);
                else if (config == JACOBI_RT_A)
                    jacobi_item<RtA>(k, nk, a.items, a.n_items, a.jsims, a.counters,
                                     ss.epoch + 1, smem, &s_bar, &s_parity, a.status, &s_pref);
                else
                    jacobi_tb_item(k, a.items, a.jsims, smem, &s_bar, &s_parity, a.status);
                break;
            }
            case ITEM_SUBGRAD:
                band_subgrad(sd, w.a, w.b, smem, &s_bar, &s_parity, a.status);
                break;
            case ITEM_DENSITY:
                // the fluid update resets the obstacles before the density
                // update runs (natrix/core/fluid_simulator.py:267-280): no
                // mask test
                band_density(sd, ss.dt, ss.rc, w.a, w.b, smem, &s_bar,
                             &s_parity, a.status);
                break;
            default: break;
        }
        __syncthreads();  // the item's writes are done
        if (tid == 0) {
            pend.idx[pend.n++] = w.done;
            if (pend.n == kPending) pend.flush(a.counters);
            asm volatile("cp.async.wait_all;" ::: "memory");  // the next descriptor
            s_item = (int)s_next;
        }
        __syncthreads();
    }
    if (tid == 0) pend.flush(a.counters);
}

constexpr int step_smem_bytes() {
    return RtB::SMEM > RtA::SMEM ? (RtB::SMEM > TbStep::SMEM ? RtB::SMEM : TbStep::SMEM)
                                 : (RtA::SMEM > TbStep::SMEM ? RtA::SMEM : TbStep::SMEM);
}

int round_up(int v, int m) { return (v + m - 1) / m * m; }

int fail(int code, const char* msg) { return set_last_error(code, msg); }

template <class T>
cudaError_t upload_vec(T** dev, size_t* cap, const std::vector<T>& v) {
    const size_t n = std::max<size_t>(v.size(), 1);
    if (*cap < n) {
        cudaFree(*dev);
        *dev = nullptr;
        cudaError_t e = cudaMalloc(dev, n * sizeof(T));
        if (e != cudaSuccess) return e;
        *cap = n;
    }
    if (v.empty()) return cudaSuccess;
    return cudaMemcpy(*dev, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

struct DevList {
    int4* ptr = nullptr;
    size_t cap = 0;
    int n = 0;
};

struct JacobiLaunch {
    int config;
    JacobiBatchItem* items = nullptr;
    int n = 0;
};

}  // namespace

struct natrix_batch {
    int device = 0;
    int n = 0;
    std::vector<Grid> grids;
    std::vector<natrix_params> prm;
    std::vector<float> d_speed, d_diss;
    int tune_config[kClasses] = {JACOBI_TB, JACOBI_RT_A, JACOBI_RT_B};
    int tune_sweeps[kClasses] = {8, 8, 8};
    unsigned char* arena = nullptr;
    std::vector<BatchSimDesc> desc;
    BatchSimDesc* d_desc = nullptr;
    std::vector<JacobiBatchSim> jsims;
    JacobiBatchSim* d_jsims = nullptr;
    DevList items_all, items_vort, items_visc;
    std::vector<JacobiLaunch> jl;
    // per-step upload
    unsigned char* d_step = nullptr;
    unsigned char* h_step = nullptr;  // pinned, double-buffered
    size_t step_cap = 0;
    cudaEvent_t step_ev[2] = {};
    int step_slot = 0;
    std::vector<std::vector<ForceOp>> fq;
    std::vector<std::vector<ShapeOp>> sq;
    int rho_cur = 0;
    bool dirty = true;  // tables / graphs need rebuilding
    bool use_graph = true;
    cudaGraphExec_t graph[2] = {};
    cudaStream_t capture = nullptr;
    int* d_status = nullptr;
    int64_t launches = 0;
    int launches_per_step = 0;
    // persistent step kernel (one launch per step, the default) or one
    // launch per phase
    bool persistent = true;
    StepItem* d_items = nullptr;
    size_t items_cap = 0;
    int n_items = 0;
    unsigned long long* d_counters = nullptr;  // [n_sims][phases] completions
    size_t counters_cap = 0;
    unsigned long long* d_claim = nullptr;
    unsigned long long epoch = 0;
    int step_grid = 0;
};

namespace {

// The persistent kernel's work list: phases in order, within a phase the
// simulations by decreasing sweep work (the longest dependency chains start
// first), per simulation its bands of rows (see band_rows) or its sweep
// tiles.  Each item waits for all
// items of its simulation's previous phase.
int build_step_items(natrix_batch* b, const std::vector<int>& cfg_of,
                     const std::vector<int>& per_of, const std::vector<int>& launches_of,
                     int max_launches) {
    const int n = b->n;
    for (int i = 0; i < n; ++i)
        if (b->grids[i].P > kMaxStagedPitch)
            return fail(NATRIX_ERANGE,
                        "the persistent batch step stages rows of at most 3008 cells in shared "
                        "memory; use the per-phase mode for wider simulations");
    const int kF = 0, kA = 1, kCV = 2, kAV = 3, kVS = 4, kD = 5, kJ = 6;
    const int kS = kJ + max_launches, kR = kS + 1, phases = kR + 1;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const double wx = (double)b->grids[x].W * b->grids[x].H * b->prm[x].iterations;
        const double wy = (double)b->grids[y].W * b->grids[y].H * b->prm[y].iterations;
        return wx > wy;
    });
    // forcing, vorticity and viscosity bands: a multiple of 32 rows (the
    // forcing item's block height), about 16k cells and within the staging
    // space where that allows; the staged phases' bands fit their rows (and
    // halos) in the staging space
    auto staged = [&](int ph) { return ph == kA || ph == kD || ph == kS || ph == kR; };
    auto band_rows = [&](const Grid& g, int ph) {
        if (staged(ph)) return staged_band_rows(g.P);
        // forcing stages 12 B per cell (velocity, density) in 32-row blocks
        const int r = std::min(16384 / g.W, kStageBytes / (12 * g.P)) / kForceRows * kForceRows;
        return r < kForceRows ? kForceRows : r;
    };
    auto bands = [&](const Grid& g, int ph) {
        return (g.H + band_rows(g, ph) - 1) / band_rows(g, ph);
    };
    auto tiles = [&](int i) {
        int tx, ty;
        jacobi_tile(cfg_of[i], &tx, &ty);
        const Grid& g = b->grids[i];
        return ((g.W + tx - 1) / tx) * ((g.H + ty - 1) / ty);
    };
    // the phases each simulation runs, in order
    std::vector<std::vector<int>> seq(n);
    for (int i = 0; i < n; ++i) {
        seq[i].push_back(kF);
        seq[i].push_back(kA);
        if (b->prm[i].vorticity > 0.0f) {
            seq[i].push_back(kCV);
            seq[i].push_back(kAV);
        }
        if (b->prm[i].viscosity > 0.0f) seq[i].push_back(kVS);
        seq[i].push_back(kD);
        for (int m = 0; m < launches_of[i]; ++m) seq[i].push_back(kJ + m);
        seq[i].push_back(kS);
        seq[i].push_back(kR);
    }
    auto count_of = [&](int i, int ph) {
        return (ph >= kJ && ph < kS) ? tiles(i) : bands(b->grids[i], ph);
    };
    // Phase-major over all simulations: every phase offers many ready items.
    // (Cutting the list into waves that fit in L2, all phases of a wave
    // before the next, was measured: 5.2 ms per step instead of 2.8 on the
    // 512-simulation workload, the CTAs idling on the chain inside a wave.)
    std::vector<StepItem> items;
    for (int ph = 0; ph < phases; ++ph) {
        for (int i : order) {
            const auto& q = seq[i];
            const auto pos = std::find(q.begin(), q.end(), ph);
            if (pos == q.end()) continue;
            StepItem base{};
            base.sim = i;
            base.done = i * phases + ph;
            if (pos == q.begin()) {
                base.wait = -1;
            } else {
                const int prev = *(pos - 1);
                base.wait = i * phases + prev;
                base.need = count_of(i, prev);
            }
            const Grid& g = b->grids[i];
            if (ph >= kJ && ph < kS) {
                const int m = ph - kJ;
                int tx, ty;
                jacobi_tile(cfg_of[i], &tx, &ty);
                base.kind = ITEM_JACOBI;
                base.config = cfg_of[i];
                base.src = m & 1;
                base.sweeps = std::min(b->prm[i].iterations - 1 - m * per_of[i], per_of[i]);
                for (int y = 0; y < g.H; y += ty)
                    for (int x = 0; x < g.W; x += tx) {
                        StepItem t = base;
                        t.a = x;
                        t.b = y;
                        items.push_back(t);
                    }
                continue;
            }
            base.kind = ph == kF    ? ITEM_FORCE
                        : ph == kA  ? ITEM_ADVECT
                        : ph == kCV ? ITEM_CALC_VORT
                        : ph == kAV ? ITEM_APPLY_VORT
                        : ph == kVS ? ITEM_VISC
                        : ph == kD  ? ITEM_DIV
                        : ph == kS  ? ITEM_SUBGRAD
                                    : ITEM_DENSITY;
            const int rows = band_rows(g, ph);
            for (int y = 0; y < g.H; y += rows) {
                StepItem t = base;
                t.a = y;
                t.b = std::min(y + rows, g.H);
                items.push_back(t);
            }
        }
    }
    cudaError_t e = upload_vec(&b->d_items, &b->items_cap, items);
    b->n_items = (int)items.size();
    const size_t nc = (size_t)n * phases;
    if (e == cudaSuccess && b->counters_cap < nc) {
        cudaFree(b->d_counters);
        b->d_counters = nullptr;
        e = cudaMalloc(&b->d_counters, nc * sizeof(unsigned long long));
        if (e == cudaSuccess) b->counters_cap = nc;
    }
    if (e == cudaSuccess && !b->d_claim) e = cudaMalloc(&b->d_claim, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->d_counters, 0, nc * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->d_claim, 0, sizeof(unsigned long long));
    if (e == cudaSuccess && b->step_grid == 0) {
        e = cudaFuncSetAttribute(k_batch_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 step_smem_bytes());
        int per_sm = 0, sms = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_step,
                                                              32 * kStepThreadsY,
                                                              step_smem_bytes());
        if (e == cudaSuccess)
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
        if (e == cudaSuccess) b->step_grid = std::max(1, per_sm) * std::max(1, sms);
    }
    if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
    b->epoch = 0;
    return NATRIX_OK;
}

// Rebuild descriptors, item lists and Jacobi launch lists (host -> device).
int rebuild(natrix_batch* b) {
    const int n = b->n;
    std::vector<int4> all, vort, visc;
    for (int i = 0; i < n; ++i) {
        BatchSimDesc& s = b->desc[i];
        const natrix_params& p = b->prm[i];
        s.sp = StepParams{};
        s.sp.speed = p.speed;
        s.sp.dissipation = p.dissipation;
        s.sp.vorticity = p.vorticity;
        if (p.viscosity > 0.0f) {
            const double alpha = 1.0 / (double)p.viscosity;
            s.sp.alpha = (float)alpha;
            s.sp.rbeta = (float)(1.0 / (4.0 + alpha));
        }
        s.sp.has_borders = p.has_borders ? 1 : 0;
        s.sp.mask_zero = 1;
        s.sp.d_speed = b->d_speed[i];
        s.sp.d_dissipation = b->d_diss[i];
        int cur = 1;
        s.vort_in = s.vort_out = s.visc_in = s.visc_out = 1;
        if (p.vorticity > 0.0f) {
            s.vort_in = cur;
            s.vort_out = 3 - cur;
            cur = 3 - cur;
        }
        if (p.viscosity > 0.0f) {
            s.visc_in = cur;
            s.visc_out = 3 - cur;
            cur = 3 - cur;
        }
        s.last = cur;
        const Grid& g = s.g;
        for (int by = 0; by < g.H; by += BY)
            for (int bx = 0; bx < g.W; bx += BX) {
                const int4 it = make_int4(i, bx, by, 0);
                all.push_back(it);
                if (p.vorticity > 0.0f) vort.push_back(it);
                if (p.viscosity > 0.0f) visc.push_back(it);
            }
    }
    // Jacobi: per simulation, configuration of its size class; encode maps
    std::vector<int> launches_of(n, 0), cfg_of(n, 0), per_of(n, 8);
    int max_launches = 0;
    for (int i = 0; i < n; ++i) {
        const int c = size_class(b->grids[i]);
        cfg_of[i] = b->tune_config[c];
        per_of[i] = std::max(1, std::min(b->tune_sweeps[c], jacobi_max_sweeps_per_launch()));
        const int rem = b->prm[i].iterations - 1;
        launches_of[i] = rem > 0 ? (rem + per_of[i] - 1) / per_of[i] : 0;
        max_launches = std::max(max_launches, launches_of[i]);
        b->desc[i].p_final = launches_of[i] & 1;
        const char* err = nullptr;
        JacobiBatchSim& js = b->jsims[i];
        if (!jacobi_encode_maps_for(&js.maps, cfg_of[i], b->desc[i].p[0], b->desc[i].p[1],
                                    b->desc[i].div, b->desc[i].flags, b->grids[i], &err))
            return fail(NATRIX_ECUDA, err);
        js.p[0] = b->desc[i].p[0];
        js.p[1] = b->desc[i].p[1];
        js.g = b->grids[i];
    }
    if (b->persistent) {
        const int rc = build_step_items(b, cfg_of, per_of, launches_of, max_launches);
        if (rc) return rc;
    }
    for (auto& l : b->jl) cudaFree(l.items);
    b->jl.clear();
    for (int m = 0; m < max_launches; ++m) {
        for (int c : {JACOBI_TB, JACOBI_RT_A, JACOBI_RT_B}) {
            std::vector<JacobiBatchItem> its;
            for (int i = 0; i < n; ++i) {
                if (cfg_of[i] != c || m >= launches_of[i]) continue;
                const int rem = b->prm[i].iterations - 1 - m * per_of[i];
                const int sw = std::min(rem, per_of[i]);
                int tx, ty;
                jacobi_tile(c, &tx, &ty);
                const Grid& g = b->grids[i];
                for (int y = 0; y < g.H; y += ty)
                    for (int x = 0; x < g.W; x += tx)
                        its.push_back(JacobiBatchItem{i, m & 1, sw, x, y});
            }
            if (its.empty()) continue;
            JacobiLaunch l;
            l.config = c;
            l.n = (int)its.size();
            size_t cap = 0;
            cudaError_t e = upload_vec(&l.items, &cap, its);
            if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
            b->jl.push_back(l);
        }
    }
    size_t cap;
    cudaError_t e = cudaSuccess;
    cap = b->items_all.cap;
    e = upload_vec(&b->items_all.ptr, &cap, all);
    b->items_all.cap = cap;
    b->items_all.n = (int)all.size();
    if (e == cudaSuccess) {
        cap = b->items_vort.cap;
        e = upload_vec(&b->items_vort.ptr, &cap, vort);
        b->items_vort.cap = cap;
        b->items_vort.n = (int)vort.size();
    }
    if (e == cudaSuccess) {
        cap = b->items_visc.cap;
        e = upload_vec(&b->items_visc.ptr, &cap, visc);
        b->items_visc.cap = cap;
        b->items_visc.n = (int)visc.size();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_desc, b->desc.data(), n * sizeof(BatchSimDesc),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_jsims, b->jsims.data(), n * sizeof(JacobiBatchSim),
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
    for (auto& g : b->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    b->dirty = false;
    return NATRIX_OK;
}

// The kernel sequence of one step, reading the step block at b->d_step.
cudaError_t enqueue_step(natrix_batch* b, int rho_cur, cudaStream_t st, int* launches) {
    const int n = b->n;
    const StepHeader* hdr = reinterpret_cast<const StepHeader*>(b->d_step);
    const int* op_begin = reinterpret_cast<const int*>(b->d_step + sizeof(StepHeader));
    const int* op_count = op_begin + n;
    const int* sh_begin = op_count + n;
    const int* sh_count = sh_begin + n;
    // op and shape arrays follow at offsets recorded in the header block
    const size_t ops_off = sizeof(StepHeader) + 4 * (size_t)n * sizeof(int);
    const ForceOp* ops = reinterpret_cast<const ForceOp*>(b->d_step + ops_off);
    // shapes start after the op capacity (fixed layout so a graph can replay)
    const size_t shapes_off = ops_off + (size_t)kMaxOpsPerLaunch * n * sizeof(ForceOp);
    const ShapeOp* shapes = reinterpret_cast<const ShapeOp*>(b->d_step + shapes_off);
    int count = 0;
    if (b->persistent) {
        const StepArgs a{b->d_items, b->n_items, n, b->d_desc, b->d_jsims, b->d_counters,
                         b->d_claim, b->d_step, ops_off, shapes_off, b->d_status};
        k_batch_step<<<b->step_grid, dim3(BX, kStepThreadsY), step_smem_bytes(), st>>>(a);
        *launches = 1;
        return cudaGetLastError();
    }
    k_batch_prepare<<<(n + 127) / 128, 128, 0, st>>>(b->d_desc, hdr, sh_count);
    ++count;
    const int na = b->items_all.n;
    const int4* all = b->items_all.ptr;
    k_batch_obstacles<<<na, dim3(BX, BY), 0, st>>>(all, b->d_desc, shapes, sh_begin, sh_count);
    k_batch_forcing<<<na, dim3(BX, BY), 0, st>>>(all, b->d_desc, rho_cur, ops, op_begin,
                                                 op_count);
    k_batch_advect<<<na, dim3(BX, BY), 0, st>>>(all, b->d_desc, rho_cur);
    count += 3;
    if (b->items_vort.n) {
        k_batch_calc_vort<<<b->items_vort.n, dim3(BX, BY), 0, st>>>(b->items_vort.ptr,
                                                                    b->d_desc, rho_cur);
        k_batch_apply_vort<<<b->items_vort.n, dim3(BX, BY), 0, st>>>(b->items_vort.ptr,
                                                                     b->d_desc, rho_cur);
        count += 2;
    }
    if (b->items_visc.n) {
        k_batch_visc<<<b->items_visc.n, dim3(BX, BY), 0, st>>>(b->items_visc.ptr, b->d_desc,
                                                               rho_cur);
        ++count;
    }
    k_batch_divergence<<<na, dim3(BX, BY), 0, st>>>(all, b->d_desc, rho_cur);
    ++count;
    for (const JacobiLaunch& l : b->jl) {
        cudaError_t e = launch_jacobi_batch(l.config, l.items, l.n, b->d_jsims, b->d_status, st);
        if (e != cudaSuccess) return e;
        ++count;
    }
    k_batch_subgrad<<<na, dim3(BX, BY), 0, st>>>(all, b->d_desc, rho_cur);
    k_batch_density<<<na, dim3(BX, BY), 0, st>>>(all, b->d_desc, rho_cur);
    count += 2;
    *launches = count;
    return cudaGetLastError();
}

size_t step_capacity(int n) {
    return sizeof(StepHeader) + 4 * (size_t)n * sizeof(int) +
           (size_t)kMaxOpsPerLaunch * n * (sizeof(ForceOp) + sizeof(ShapeOp));
}

void free_batch(natrix_batch* b) {
    for (auto& g : b->graph)
        if (g) cudaGraphExecDestroy(g);
    if (b->capture) cudaStreamDestroy(b->capture);
    for (auto& e : b->step_ev)
        if (e) cudaEventDestroy(e);
    for (auto& l : b->jl) cudaFree(l.items);
    cudaFree(b->items_all.ptr);
    cudaFree(b->items_vort.ptr);
    cudaFree(b->items_visc.ptr);
    cudaFree(b->d_desc);
    cudaFree(b->d_jsims);
    cudaFree(b->d_step);
    cudaFree(b->d_status);
    cudaFree(b->d_items);
    cudaFree(b->d_counters);
    cudaFree(b->d_claim);
    cudaFree(b->arena);
    if (b->h_step) cudaFreeHost(b->h_step);
    delete b;
}

}  // namespace

extern "C" {

int natrix_batch_create(int32_t n, const int32_t* widths, const int32_t* heights,
                        natrix_batch** out) {
    if (!out || n < 1 || !widths || !heights) return fail(NATRIX_EINVAL, "bad batch arguments");
    *out = nullptr;
    natrix_batch* b = new natrix_batch();
    cudaGetDevice(&b->device);
    b->n = n;
    size_t total = 0;
    for (int i = 0; i < n; ++i) {
        if (widths[i] < 1 || heights[i] < 1 || widths[i] > 32768 || heights[i] > 32768) {
            delete b;
            return fail(NATRIX_EINVAL, "bad grid size in batch");
        }
        const Grid g{widths[i], heights[i], round_up(widths[i], 32)};
        b->grids.push_back(g);
        // vel x3 (8 B), p x2, div, vort, rho x2 (4 B), mask, flags (1 B); each
        // buffer starts 256-byte aligned
        total += (size_t)g.P * g.H * (24 + 24) + (size_t)round_up(g.P * g.H, 256) * 2 + 16 * 256;
    }
    cudaError_t e = cudaMalloc(&b->arena, total);
    if (e == cudaSuccess) e = cudaMemset(b->arena, 0, total);
    if (e != cudaSuccess) {
        free_batch(b);
        return fail(NATRIX_ENOMEM, cudaGetErrorString(e));
    }
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = b->arena + off;
        off += (bytes + 255) / 256 * 256;
        return p;
    };
    b->desc.resize(n);
    b->jsims.resize(n);
    b->prm.assign(n, natrix_params{500.0f, 50, 1.0f, 0.0f, 0.1f, 1, 1, 0});
    b->d_speed.assign(n, 500.0f);
    b->d_diss.assign(n, 1.0f);
    b->fq.resize(n);
    b->sq.resize(n);
    for (int i = 0; i < n; ++i) {
        BatchSimDesc& s = b->desc[i];
        const Grid& g = b->grids[i];
        const size_t cells = (size_t)g.P * g.H;
        s.g = g;
        for (auto& v : s.vel) v = reinterpret_cast<float2*>(take(cells * 8));
        for (auto& q : s.p) q = reinterpret_cast<float*>(take(cells * 4));
        s.div = reinterpret_cast<float*>(take(cells * 4));
        s.vort = reinterpret_cast<float*>(take(cells * 4));
        for (auto& r : s.rho) r = reinterpret_cast<float*>(take(cells * 4));
        s.mask = take(cells);
        s.flags = take(cells);
    }
    e = cudaMalloc(&b->d_desc, n * sizeof(BatchSimDesc));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_jsims, n * sizeof(JacobiBatchSim));
    b->step_cap = step_capacity(n);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_step, b->step_cap);
    if (e == cudaSuccess) e = cudaMemset(b->d_step, 0, b->step_cap);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_step, 2 * b->step_cap);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(int));
    for (int k = 0; k < 2 && e == cudaSuccess; ++k)
        e = cudaEventCreateWithFlags(&b->step_ev[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_batch(b);
        return fail(NATRIX_ENOMEM, cudaGetErrorString(e));
    }
    *out = b;
    return NATRIX_OK;
}

int natrix_batch_destroy(natrix_batch* b) {
    if (!b) return NATRIX_OK;
    DeviceGuard dg(b->device);
    cudaDeviceSynchronize();
    free_batch(b);
    return NATRIX_OK;
}

int natrix_batch_set_params(natrix_batch* b, int32_t sim, const natrix_params* p) {
    if (!b || !p || sim < -1 || sim >= b->n) return fail(NATRIX_EINVAL, "bad arguments");
    if (!(p->speed > 0.0f) || p->iterations < 1 || !(p->dissipation > 0.0f) ||
        !(p->vorticity >= 0.0f) || !(p->viscosity >= 0.0f))
        return fail(NATRIX_EINVAL, "invalid parameters: speed, iterations and dissipation must "
                                   "be > 0, vorticity and viscosity >= 0");
    for (int i = (sim < 0 ? 0 : sim); i < (sim < 0 ? b->n : sim + 1); ++i) b->prm[i] = *p;
    b->dirty = true;
    return NATRIX_OK;
}

int natrix_batch_set_density_params(natrix_batch* b, int32_t sim, float speed,
                                    float dissipation) {
    if (!b || sim < -1 || sim >= b->n) return fail(NATRIX_EINVAL, "bad arguments");
    if (!(speed > 0.0f) || !(dissipation > 0.0f))
        return fail(NATRIX_EINVAL, "speed and dissipation must be > 0");
    for (int i = (sim < 0 ? 0 : sim); i < (sim < 0 ? b->n : sim + 1); ++i) {
        b->d_speed[i] = speed;
        b->d_diss[i] = dissipation;
    }
    b->dirty = true;
    return NATRIX_OK;
}

int natrix_batch_set_tuning(natrix_batch* b, int32_t size_class, int32_t config,
                            int32_t sweeps_per_launch) {
    if (!b || size_class < 0 || size_class >= kClasses || config < JACOBI_TB ||
        config > JACOBI_RT_B || sweeps_per_launch < 1 ||
        sweeps_per_launch > jacobi_max_sweeps_per_launch())
        return fail(NATRIX_EINVAL, "bad tuning");
    b->tune_config[size_class] = config;
    b->tune_sweeps[size_class] = sweeps_per_launch;
    b->dirty = true;
    return NATRIX_OK;
}

int natrix_batch_set_graph(natrix_batch* b, int32_t enable) {
    if (!b) return fail(NATRIX_EINVAL, "NULL handle");
    b->use_graph = enable != 0;
    return NATRIX_OK;
}

int natrix_batch_set_persistent(natrix_batch* b, int32_t enable) {
    if (!b) return fail(NATRIX_EINVAL, "NULL handle");
    if (b->persistent != (enable != 0)) {
        b->persistent = enable != 0;
        b->dirty = true;
    }
    return NATRIX_OK;
}

int natrix_batch_add_velocity(natrix_batch* b, int32_t sim, float px, float py, float vx,
                              float vy, float radius) {
    if (!b || sim < 0 || sim >= b->n) return fail(NATRIX_EINVAL, "bad arguments");
    if ((int)b->fq[sim].size() >= kMaxOpsPerLaunch)
        return fail(NATRIX_ERANGE, "more than 256 forcing ops for one simulation in one step");
    b->fq[sim].push_back(ForceOp{FORCE_CONE_VELOCITY, px, py, radius, vx, vy, 0.0f, 0});
    return NATRIX_OK;
}

int natrix_batch_add_splats(natrix_batch* b, int32_t sim, const float* splats, int32_t n) {
    if (!b || sim < 0 || sim >= b->n || n < 0 || (n && !splats))
        return fail(NATRIX_EINVAL, "bad arguments");
    if ((int)b->fq[sim].size() + n > kMaxOpsPerLaunch)
        return fail(NATRIX_ERANGE, "more than 256 forcing ops for one simulation in one step");
    for (int i = 0; i < n; ++i)
        if (!(splats[(size_t)i * NATRIX_SPLAT_FLOATS + 2] > 0.0f))
            return fail(NATRIX_EINVAL, "splat radius must be > 0");
    for (int i = 0; i < n; ++i) {
        const float* r = splats + (size_t)i * NATRIX_SPLAT_FLOATS;
        b->fq[sim].push_back(ForceOp{FORCE_GAUSS, r[0], r[1], r[2], r[3], r[4], r[5], 0});
    }
    return NATRIX_OK;
}

int natrix_batch_add_circle_obstacle(natrix_batch* b, int32_t sim, float px, float py,
                                     float radius, int32_t is_static) {
    if (!b || sim < 0 || sim >= b->n) return fail(NATRIX_EINVAL, "bad arguments");
    if ((int)b->sq[sim].size() >= kMaxOpsPerLaunch)
        return fail(NATRIX_ERANGE, "more than 256 obstacle shapes for one simulation in one step");
    b->sq[sim].push_back(ShapeOp{SHAPE_CIRCLE, is_static ? 1 : 0, {px, py, radius, 0, 0, 0}});
    return NATRIX_OK;
}

int natrix_batch_add_splats_bulk(natrix_batch* b, const int32_t* counts, const float* splats) {
    if (!b || !counts) return fail(NATRIX_EINVAL, "bad arguments");
    size_t off = 0;
    for (int i = 0; i < b->n; ++i) {
        int rc = natrix_batch_add_splats(b, i, splats + off * NATRIX_SPLAT_FLOATS, counts[i]);
        if (rc) return rc;
        off += (size_t)counts[i];
    }
    return NATRIX_OK;
}

int natrix_batch_add_circles_bulk(natrix_batch* b, const int32_t* counts, const float* circles) {
    if (!b || !counts) return fail(NATRIX_EINVAL, "bad arguments");
    size_t off = 0;
    for (int i = 0; i < b->n; ++i) {
        for (int k = 0; k < counts[i]; ++k, ++off) {
            const float* c = circles + off * 3;
            int rc = natrix_batch_add_circle_obstacle(b, i, c[0], c[1], c[2], 0);
            if (rc) return rc;
        }
    }
    return NATRIX_OK;
}

int natrix_batch_step(natrix_batch* b, float dt, void* stream) {
    if (!b) return fail(NATRIX_EINVAL, "NULL handle");
    DeviceGuard dg(b->device);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (b->dirty) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
        int rc = rebuild(b);
        if (rc) return rc;
    }
    // pack the step block: header, op / shape ranges, ops, shapes (fixed offsets)
    const int n = b->n;
    const int slot = b->step_slot;
    b->step_slot ^= 1;
    cudaError_t e = cudaEventSynchronize(b->step_ev[slot]);
    if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
    unsigned char* h = b->h_step + slot * b->step_cap;
    StepHeader hdr{dt, n, b->rho_cur, 0, b->epoch, 0};
    std::memcpy(h, &hdr, sizeof hdr);
    int* ranges = reinterpret_cast<int*>(h + sizeof(StepHeader));
    const size_t ops_off = sizeof(StepHeader) + 4 * (size_t)n * sizeof(int);
    const size_t shapes_off = ops_off + (size_t)kMaxOpsPerLaunch * n * sizeof(ForceOp);
    ForceOp* ops = reinterpret_cast<ForceOp*>(h + ops_off);
    ShapeOp* shapes = reinterpret_cast<ShapeOp*>(h + shapes_off);
    int no = 0, ns = 0;
    for (int i = 0; i < n; ++i) {
        ranges[i] = no;
        ranges[n + i] = (int)b->fq[i].size();
        ranges[2 * n + i] = ns;
        ranges[3 * n + i] = (int)b->sq[i].size();
        std::copy(b->fq[i].begin(), b->fq[i].end(), ops + no);
        std::copy(b->sq[i].begin(), b->sq[i].end(), shapes + ns);
        no += (int)b->fq[i].size();
        ns += (int)b->sq[i].size();
        b->fq[i].clear();
        b->sq[i].clear();
    }
    // copy the used parts (the layout keeps fixed offsets)
    e = cudaMemcpyAsync(b->d_step, h, ops_off + no * sizeof(ForceOp), cudaMemcpyHostToDevice,
                        st);
    if (e == cudaSuccess && ns)
        e = cudaMemcpyAsync(b->d_step + shapes_off, h + shapes_off, ns * sizeof(ShapeOp),
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->step_ev[slot], st);
    if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));

    const int rc = b->rho_cur;
    int launches = 0;
    if (b->use_graph && b->graph[rc]) {
        e = cudaGraphLaunch(b->graph[rc], st);
        launches = b->launches_per_step;
    } else {
        // run this step directly; with graphs on, also record the same
        // sequence (not executed) as the graph of this density parity
        e = enqueue_step(b, rc, st, &launches);
        b->launches_per_step = launches;
        if (e == cudaSuccess && b->use_graph) {
            cudaGraph_t g = nullptr;
            int unused = 0;
            e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                const cudaError_t e2 = enqueue_step(b, rc, b->capture, &unused);
                e = cudaStreamEndCapture(b->capture, &g);
                if (e == cudaSuccess) e = e2;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph[rc], g, 0);
            if (g) cudaGraphDestroy(g);
        }
    }
    if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
    b->launches += launches;
    b->rho_cur ^= 1;
    ++b->epoch;
    return NATRIX_OK;
}

int natrix_batch_field(natrix_batch* b, int32_t sim, int32_t field, void** ptr, int64_t* pitch) {
    if (!b || sim < 0 || sim >= b->n || !ptr || !pitch) return fail(NATRIX_EINVAL, "bad arguments");
    const BatchSimDesc& s = b->desc[sim];
    *pitch = s.g.P;
    switch (field) {
        case NATRIX_FIELD_VELOCITY: *ptr = s.vel[0]; break;
        case NATRIX_FIELD_PRESSURE: *ptr = s.p[s.p_final]; break;
        case NATRIX_FIELD_DIVERGENCE: *ptr = s.div; break;
        case NATRIX_FIELD_VORTICITY: *ptr = s.vort; break;
        case NATRIX_FIELD_DENSITY: *ptr = s.rho[b->rho_cur]; break;
        default: return fail(NATRIX_EINVAL, "unknown field");
    }
    return NATRIX_OK;
}

int natrix_batch_download(natrix_batch* b, int32_t sim, int32_t field, void* host, void* stream) {
    void* ptr = nullptr;
    int64_t pitch = 0;
    int rc = natrix_batch_field(b, sim, field, &ptr, &pitch);
    if (rc) return rc;
    if (!host) return fail(NATRIX_EINVAL, "NULL host buffer");
    const Grid& g = b->grids[sim];
    const size_t esz = field == NATRIX_FIELD_VELOCITY ? 8 : 4;
    DeviceGuard dg(b->device);
    cudaError_t e = cudaMemcpy2DAsync(host, g.W * esz, ptr, (size_t)pitch * esz, g.W * esz, g.H,
                                      cudaMemcpyDeviceToHost, reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? NATRIX_OK : fail(NATRIX_ECUDA, cudaGetErrorString(e));
}

int natrix_batch_launches(natrix_batch* b, int64_t* total, int32_t* per_step) {
    if (!b || !total || !per_step) return fail(NATRIX_EINVAL, "NULL argument");
    *total = b->launches;
    *per_step = b->launches_per_step;
    return NATRIX_OK;
}

int natrix_batch_sync(natrix_batch* b, void* stream) {
    if (!b) return fail(NATRIX_EINVAL, "NULL handle");
    DeviceGuard dg(b->device);
    cudaError_t e = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
    int status = 0;
    e = cudaMemcpy(&status, b->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(NATRIX_ECUDA, cudaGetErrorString(e));
    if (status) {
        cudaMemset(b->d_status, 0, sizeof(int));
        return fail(NATRIX_EDEVICE, "a batched kernel reported a bounded wait that ran out");
    }
    return NATRIX_OK;
}

}  // extern "C"
