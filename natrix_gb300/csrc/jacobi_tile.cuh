// Jacobi pressure-sweep tiles (shader.Poisson.comp:17-38): the TMA and
// mbarrier helpers, the two tile configurations and the per-tile bodies,
// shared by the sweep kernels (jacobi_tma.cu) and the batch step kernel
// (batch.cu).  Every sweep evaluates exactly the reference's expression
//     p' = (pL + pR + pB + pT - b) * 0.25
// with a neighbour replaced by the centre when it is an obstacle or beyond a
// wall, so k fused sweeps on a tile with a k-cell halo equal k single sweeps
// bit for bit.
#pragma once

#include <cudaTypedefs.h>

#include <type_traits>

#include "kernels.cuh"

namespace natrix {

constexpr int align128(int b) { return (b + 127) / 128 * 128; }

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// Bounded wait for the given phase parity of a tile barrier (about 4M polls).
__device__ __forceinline__ bool wait_phase(uint64_t* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Completion counters of persistent kernels whose CTAs wait on each other's
// items (batch.cu, the sweep chain of jacobi_tma.cu).
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Bounded wait (about 2^24 polls with back-off) for *c >= target.
__device__ __forceinline__ bool wait_counter(const unsigned long long* c,
                                             unsigned long long target) {
    for (int it = 0; it < (1 << 24); ++it) {
        if (ld_acquire_u64(c) >= target) return true;
        __nanosleep(64);
    }
    return false;
}

// Order generic-proxy writes (other CTAs' stores released through a
// completion counter; this CTA's use of the staging memory) before the
// async-proxy copies the calling thread issues next.
__device__ __forceinline__ void fence_before_tma() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
    fence_proxy_async();
}

// One tile of work: where to load it from, where to write it, how far to go.
struct TileJob {
    const CUtensorMap* p;
    const CUtensorMap* d;
    const CUtensorMap* f;
    float* pout;
    Grid g;
    int sweeps;
    int tile_x, tile_y;
    // Gradient subtraction fused after the sweeps (shader.SubtractGradient.comp
    // on the output tile, from the register-resident pressure): vout = vin -
    // grad p.  Null: not fused.  Needs sweeps < HALO, so the pressure one cell
    // beyond the output tile is still exact.
    const float2* vin;
    float2* vout;
};

// ---------------------------------------------------------------------------
// Shared-memory variant: TX x TY output tile, region shrinking one cell per
// sweep, ping-pong between two pressure buffers in shared memory.
template <int TX_, int TY_, int HALO_, int THREADS_Y_ = 8>
struct TbCfg {
    static constexpr int TX = TX_, TY = TY_, HALO = HALO_;
    static constexpr int HXP = (HALO + 3) / 4 * 4;  // x-halo of the float boxes
    static constexpr int HXF = 16;                    // x-halo of the uint8 box
    static constexpr int RX = TX + 2 * HXP, RY = TY + 2 * HALO, RXF = TX + 2 * HXF;
    static constexpr int P_BYTES = RX * RY * 4, F_BYTES = RXF * RY;
    static constexpr int OFF_A = 0;
    static constexpr int OFF_B = OFF_A + align128(P_BYTES);
    static constexpr int OFF_D = OFF_B + align128(P_BYTES);
    static constexpr int OFF_F = OFF_D + align128(P_BYTES);
    static constexpr int OFF_BAR = OFF_F + align128(F_BYTES);
    static constexpr int SMEM = OFF_BAR + 128;
    static constexpr int THREADS_X = 32, THREADS_Y = THREADS_Y_;
    static_assert(TX % 16 == 0, "tile width must keep the uint8 box 16-byte aligned");
    static_assert(RX <= 256 && RY <= 256 && RXF <= 256, "TMA box dimensions are <= 256");
};

using Tb = TbCfg<64, 32, 8>;

// Sweeps and output of one shared-memory tile whose staging copies (pressure
// into buffer A, divergence, flags) have landed; blockDim = (THREADS_X,
// THREADS_Y).
template <class C>
__device__ __forceinline__ void tb_tile_body(const TileJob& job, unsigned char* smem) {
    float* A = reinterpret_cast<float*>(smem + C::OFF_A);
    float* B = reinterpret_cast<float*>(smem + C::OFF_B);
    const float* D = reinterpret_cast<const float*>(smem + C::OFF_D);
    const uint8_t* F = reinterpret_cast<const uint8_t*>(smem + C::OFF_F);
    const int tile_x = job.tile_x, tile_y = job.tile_y, sweeps = job.sweeps;
    const int tx = threadIdx.x, ty = threadIdx.y;
    constexpr int RX = C::RX, RXF = C::RXF, FOFF = C::HXF - C::HXP;
    for (int s = 1; s <= sweeps; ++s) {
        const float* src = (s & 1) ? A : B;
        float* dst = (s & 1) ? B : A;
        const int m = sweeps - s;
        const int x0 = C::HXP - m, x1 = C::HXP + C::TX + m;
        const int y0 = C::HALO - m, y1 = C::HALO + C::TY + m;
        for (int yy = y0 + ty; yy < y1; yy += C::THREADS_Y) {
            for (int xx = x0 + tx; xx < x1; xx += C::THREADS_X) {
                const int i = yy * RX + xx;
                const float pc = src[i];
                const uint8_t f = F[yy * RXF + xx + FOFF];
                const float l = (f & NB_L) ? pc : src[i - 1];
                const float r = (f & NB_R) ? pc : src[i + 1];
                const float b = (f & NB_B) ? pc : src[i - RX];
                const float t = (f & NB_T) ? pc : src[i + RX];
                dst[i] = (l + r + b + t - D[i]) * 0.25f;
            }
        }
        __syncthreads();
    }
    const float* res = (sweeps & 1) ? B : A;

    // tile interior -> global, 16-byte stores; a float4 group starting inside
    // the row stays inside the padded pitch (pitch and tile_x are multiples of 4)
    constexpr int GROUPS = C::TX / 4;
    const Grid& g = job.g;
    for (int k = ty * C::THREADS_X + tx; k < C::TY * GROUPS; k += C::THREADS_X * C::THREADS_Y) {
        const int row = k / GROUPS, grp = k % GROUPS;
        const int gy = tile_y + row, gx = tile_x + grp * 4;
        if (gy >= g.H || gx >= g.W) continue;
        const float4 v =
            *reinterpret_cast<const float4*>(res + (C::HALO + row) * RX + C::HXP + grp * 4);
        *reinterpret_cast<float4*>(job.pout + (size_t)gy * g.P + gx) = v;
    }
}

// ---------------------------------------------------------------------------
// Register-tiled, persistent variant.  The CTA region is 128 columns x NW*R
// rows; warp w owns rows [w*R, w*R + R), lane l owns columns [4l, 4l + 4), so
// each cell of the region lives in one thread's registers (pressure,
// divergence, flags) for all the launch's sweeps.  Per sweep a thread needs,
// per row, its left/right neighbours (warp shuffles of the adjacent lanes'
// edge columns) and the rows above/below (its own registers, or the
// neighbouring warps' edge rows exchanged through a double-buffered
// shared-memory slot: one barrier per sweep).  Rows whose warp holds no wall
// or obstacle neighbour take a substitution-free path (warp-uniform branch).
// Cells near the region edge compute from missing neighbours; after s sweeps
// the outer s rows / columns are invalid and the output tile (HALO rows and
// HXP columns in) stays exact for s <= HALO.
//
// The grid is persistent (one CTA per SM, jobs assigned round-robin): once
// every thread has copied the current tile's staging buffers into registers,
// the elected thread issues the TMA loads of the CTA's next job into the same
// staging buffers, so the copy overlaps this tile's sweeps.
template <int R_, int NW_, int HALO_>
struct RtCfg {
    static constexpr int R = R_, NW = NW_, HALO = HALO_;
    static constexpr int RX = 128, RY = NW * R;
    static constexpr int HXP = (HALO + 3) / 4 * 4;
    static constexpr int TX = RX - 2 * HXP, TY = RY - 2 * HALO;
    static constexpr int HXF = 16, RXF = TX + 2 * HXF;
    static constexpr int P_BYTES = RX * RY * 4, F_BYTES = RXF * RY;
    static constexpr int X_FLOATS = 2 * NW * 2 * RX;  // [slot][warp][top,bottom][RX]
    static constexpr int OFF_P = 0;
    static constexpr int OFF_D = OFF_P + align128(P_BYTES);
    static constexpr int OFF_F = OFF_D + align128(P_BYTES);
    static constexpr int OFF_X = OFF_F + align128(F_BYTES);
    static constexpr int OFF_BAR = OFF_X + align128(X_FLOATS * 4);
    static constexpr int SMEM = OFF_BAR + 128;
    static constexpr int THREADS = NW * 32;
    // resident CTAs per SM: two of 8 warps each, else one
    static constexpr int CTAS = THREADS <= 256 ? 2 : 1;
    static_assert(TX % 16 == 0, "tile width must keep the uint8 box 16-byte aligned");
    static_assert(RY <= 256 && RXF <= 256, "TMA box dimensions are <= 256");
    static_assert(TY > 0, "region too short for the halo");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
    static_assert(CTAS == 1 || SMEM + 8 * 1024 <= 113 * 1024, "two CTAs per SM");
};

// 16 warps x 8 rows: 128x128 region, 112x112 output tile
using RtA = RtCfg<8, 16, 8>;
// 16 warps x 9 rows: 128x144 region, 112x128 output tile
using RtB = RtCfg<9, 16, 8>;
// 16 warps x 2 rows: 128x32 region, 112x16 output tile.  For grids with
// fewer tall tiles than SMs: a sweep of a tile costs time in proportion to
// the rows each warp holds, so more, shorter tiles finish a launch sooner
// although each recomputes a larger share of halo cells.
using RtC = RtCfg<2, 16, 8>;
// 8 warps x 9 rows: 128x72 region, 112x56 output tile, two CTAs per SM, so
// one CTA's sweep barrier waits are covered by the other's warps.
using RtD = RtCfg<9, 8, 8>;

// The three copies of a tile on one mbarrier phase: the expected bytes are
// registered first, so the phase cannot complete before the last copy lands
// even when the pressure copy is issued later (issue_pressure_load).
template <class C>
__device__ __forceinline__ void issue_static_loads(unsigned char* smem, uint64_t* bar,
                                                   const TileJob& job) {
    mbar_expect_tx(bar, 2 * C::P_BYTES + C::F_BYTES);
    tma_load_2d(smem + C::OFF_D, job.d, job.tile_x - C::HXP, job.tile_y - C::HALO, bar);
    tma_load_2d(smem + C::OFF_F, job.f, job.tile_x - C::HXF, job.tile_y - C::HALO, bar);
}

template <class C>
__device__ __forceinline__ void issue_pressure_load(unsigned char* smem, uint64_t* bar,
                                                    const TileJob& job) {
    tma_load_2d(smem + C::OFF_P, job.p, job.tile_x - C::HXP, job.tile_y - C::HALO, bar);
}

template <class C>
__device__ __forceinline__ void issue_tile_loads(unsigned char* smem, uint64_t* bar,
                                                 const TileJob& job) {
    issue_static_loads<C>(smem, bar, job);
    issue_pressure_load<C>(smem, bar, job);
}

// One register tile whose staging copies (pressure, divergence, flags) have
// landed in shared memory: load the thread's cells into registers, call
// after_load() once every thread has (the staging buffers are then free),
// run job.sweeps sweeps, subtract the gradient when job.vin is set, write
// the output tile.  Threads are numbered linearly (x fastest), C::THREADS
// of them.
template <class C, class AfterLoad>
__device__ __forceinline__ void rt_tile_body(const TileJob& job, unsigned char* smem,
                                             AfterLoad after_load) {
    const float* Ps = reinterpret_cast<const float*>(smem + C::OFF_P);
    const float* Ds = reinterpret_cast<const float*>(smem + C::OFF_D);
    const uint8_t* Fs = reinterpret_cast<const uint8_t*>(smem + C::OFF_F);
    float* X = reinterpret_cast<float*>(smem + C::OFF_X);
    constexpr int R = C::R, RX = C::RX;
    constexpr unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int lane = tid & 31, w = tid >> 5;
    const int c0 = lane * 4, r0 = w * R;

    // Side walls on the fast path: the left wall's cell is always this
    // lane's cell 0 (the region starts HXP = 0 mod 4 columns left of a
    // tile that starts at a multiple of 4), the right wall's is cell 3
    // when W = 0 mod 4; the clamped neighbour is the cell itself, so one
    // lane-uniform select per row replaces the per-cell flag tests and
    // those wall bits do not make a row slow.
    const int gx0 = job.tile_x - C::HXP + c0;
    const bool wall_l = gx0 == 0;
    const bool wall_r = gx0 + 3 == job.g.W - 1;
    const uint32_t side = (wall_l ? (uint32_t)NB_L : 0u) | (wall_r ? (uint32_t)NB_R << 24 : 0u);
    float p[R][4], d[R][4];
    uint32_t f[R];
    uint32_t slow = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float4 v = *reinterpret_cast<const float4*>(Ps + (r0 + r) * RX + c0);
        const float4 b = *reinterpret_cast<const float4*>(Ds + (r0 + r) * RX + c0);
        p[r][0] = v.x; p[r][1] = v.y; p[r][2] = v.z; p[r][3] = v.w;
        d[r][0] = b.x; d[r][1] = b.y; d[r][2] = b.z; d[r][3] = b.w;
        f[r] = *reinterpret_cast<const uint32_t*>(Fs + (r0 + r) * C::RXF + c0 +
                                                  (C::HXF - C::HXP));
        if (__any_sync(FULL, (f[r] & ~side) != 0u)) slow |= 1u << r;
    }
    __syncthreads();  // staging consumed: the caller may refill it
    after_load();

    // One sweep of row r from the old values of the rows above (up) and
    // below (dn); left / right neighbours by shuffle.
    // SIDE_: the tile touches a side wall (else the wall selects are dropped)
    auto sweep_row = [&](auto SIDE_, int r, const float* up, const float* dn) {
        float cur[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) cur[j] = p[r][j];
        float lft = __shfl_up_sync(FULL, cur[3], 1);
        float rgt = __shfl_down_sync(FULL, cur[0], 1);
        if (decltype(SIDE_)::value) {
            lft = wall_l ? cur[0] : lft;
            rgt = wall_r ? cur[3] : rgt;
        }
        const float L[4] = {lft, cur[0], cur[1], cur[2]};
        const float Rn[4] = {cur[1], cur[2], cur[3], rgt};
        if (slow & (1u << r)) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t fb = f[r] >> (8 * j);
                const float l = (fb & NB_L) ? cur[j] : L[j];
                const float rr = (fb & NB_R) ? cur[j] : Rn[j];
                const float b = (fb & NB_B) ? cur[j] : up[j];
                const float tt = (fb & NB_T) ? cur[j] : dn[j];
                p[r][j] = (l + rr + b + tt - d[r][j]) * 0.25f;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                p[r][j] = (L[j] + Rn[j] + up[j] + dn[j] - d[r][j]) * 0.25f;
        }
    };
    // Each sweep: publish the warp's edge rows, sweep the interior rows
    // (their neighbours are this warp's own), then the CTA barrier, then
    // the two edge rows with the neighbouring warps' rows.  Warps reach
    // the barrier after the bulk of their work, so arrival skew costs
    // less; rows 1 and R-2 keep their old values for the edge rows.
    auto sweep_all = [&](auto SIDE_) {
    for (int s = 0; s < job.sweeps; ++s) {
        float* xs = X + (s & 1) * (C::NW * 2 * RX);
        *reinterpret_cast<float4*>(xs + (w * 2 + 0) * RX + c0) =
            make_float4(p[0][0], p[0][1], p[0][2], p[0][3]);
        *reinterpret_cast<float4*>(xs + (w * 2 + 1) * RX + c0) =
            make_float4(p[R - 1][0], p[R - 1][1], p[R - 1][2], p[R - 1][3]);
        float old1[4], oldm[4];  // rows 1 and R-2 before this sweep
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            old1[j] = p[1][j];
            oldm[j] = p[R - 2][j];
        }
        {
            float up[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) up[j] = p[0][j];
#pragma unroll
            for (int r = 1; r < R - 1; ++r) {
                float cur[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) cur[j] = p[r][j];
                sweep_row(SIDE_, r, up, p[r + 1]);
#pragma unroll
                for (int j = 0; j < 4; ++j) up[j] = cur[j];
            }
        }
        __syncthreads();
        float up0[4], belowR[4];
        {
            const float4 a =
                w > 0 ? *reinterpret_cast<const float4*>(xs + ((w - 1) * 2 + 1) * RX + c0)
                      : make_float4(p[0][0], p[0][1], p[0][2], p[0][3]);
            const float4 b =
                w < C::NW - 1
                    ? *reinterpret_cast<const float4*>(xs + ((w + 1) * 2 + 0) * RX + c0)
                    : make_float4(p[R - 1][0], p[R - 1][1], p[R - 1][2], p[R - 1][3]);
            up0[0] = a.x; up0[1] = a.y; up0[2] = a.z; up0[3] = a.w;
            belowR[0] = b.x; belowR[1] = b.y; belowR[2] = b.z; belowR[3] = b.w;
        }
        sweep_row(SIDE_, 0, up0, old1);
        sweep_row(SIDE_, R - 1, oldm, belowR);
    }
    };
    // the side-wall lanes are the same in every warp of a tile
    if (__any_sync(FULL, wall_l || wall_r))
        sweep_all(std::true_type{});
    else
        sweep_all(std::false_type{});
    const Grid& g = job.g;
    if (job.vin) {
        // Gradient subtraction on the output tile (cell_subtract_gradient's
        // arithmetic): one more exchange of the warps' edge rows, then each
        // output cell reads its four neighbours from registers.
        float* xs = X + (job.sweeps & 1) * (C::NW * 2 * RX);
        *reinterpret_cast<float4*>(xs + (w * 2 + 0) * RX + c0) =
            make_float4(p[0][0], p[0][1], p[0][2], p[0][3]);
        *reinterpret_cast<float4*>(xs + (w * 2 + 1) * RX + c0) =
            make_float4(p[R - 1][0], p[R - 1][1], p[R - 1][2], p[R - 1][3]);
        __syncthreads();
        float up[4], below[4];
        {
            const float4 a =
                w > 0 ? *reinterpret_cast<const float4*>(xs + ((w - 1) * 2 + 1) * RX + c0)
                      : make_float4(p[0][0], p[0][1], p[0][2], p[0][3]);
            const float4 b =
                w < C::NW - 1
                    ? *reinterpret_cast<const float4*>(xs + ((w + 1) * 2 + 0) * RX + c0)
                    : make_float4(p[R - 1][0], p[R - 1][1], p[R - 1][2], p[R - 1][3]);
            up[0] = a.x; up[1] = a.y; up[2] = a.z; up[3] = a.w;
            below[0] = b.x; below[1] = b.y; below[2] = b.z; below[3] = b.w;
        }
        const bool out_col = c0 >= C::HXP && c0 < C::HXP + C::TX;
        const int gx = job.tile_x + c0 - C::HXP;
        auto in_tile = [&](int r) {
            const int rr = r0 + r;
            const int gy = job.tile_y + rr - C::HALO;
            return out_col && rr >= C::HALO && rr < C::HALO + C::TY && gy < g.H && gx < g.W;
        };
        // the velocity of three rows in flight at once (vin is only read in
        // this launch; the rows' stores would otherwise order each load after
        // the previous row's stores)
        constexpr int kRows = 3;
        float4 va[kRows], vb[kRows];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (r % kRows == 0) {
#pragma unroll
                for (int i = 0; i < kRows; ++i) {
                    va[i] = vb[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (r + i < R && in_tile(r + i)) {
                        const size_t o =
                            (size_t)(job.tile_y + r0 + r + i - C::HALO) * g.P + gx;
                        va[i] = __ldg(reinterpret_cast<const float4*>(job.vin + o));
                        vb[i] = __ldg(reinterpret_cast<const float4*>(job.vin + o + 2));
                    }
                }
            }
            float cur[4], dn[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                cur[j] = p[r][j];
                dn[j] = r < R - 1 ? p[r + 1][j] : below[j];
            }
            const float lft = __shfl_up_sync(FULL, cur[3], 1);
            const float rgt = __shfl_down_sync(FULL, cur[0], 1);
            const int rr = r0 + r;
            const int gy = job.tile_y + rr - C::HALO;
            if (in_tile(r)) {
                const float L[4] = {lft, cur[0], cur[1], cur[2]};
                const float Rn[4] = {cur[1], cur[2], cur[3], rgt};
                const size_t o = (size_t)gy * g.P + gx;
                const float4 a4 = va[r % kRows], b4 = vb[r % kRows];
                float2 v[4] = {make_float2(a4.x, a4.y), make_float2(a4.z, a4.w),
                               make_float2(b4.x, b4.y), make_float2(b4.z, b4.w)};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t fb = f[r] >> (8 * j);
                    const float pc = cur[j];
                    const float x1 = (fb & NB_L) ? pc : L[j];
                    const float x2 = (fb & NB_R) ? pc : Rn[j];
                    const float y1 = (fb & NB_B) ? pc : up[j];
                    const float y2 = (fb & NB_T) ? pc : dn[j];
                    v[j].x -= 0.5f * (x2 - x1);
                    v[j].y -= 0.5f * (y2 - y1);
                }
                if (gx + 3 < g.W) {
                    *reinterpret_cast<float4*>(job.vout + o) = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
                    *reinterpret_cast<float4*>(job.vout + o + 2) = make_float4(v[2].x, v[2].y, v[3].x, v[3].y);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (gx + j < g.W) job.vout[o + j] = v[j];
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) up[j] = cur[j];
        }
    }

    // output tile: region rows [HALO, HALO + TY), columns [HXP, HXP + TX)
    if (c0 >= C::HXP && c0 < C::HXP + C::TX) {
        const int gx = job.tile_x + c0 - C::HXP;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int rr = r0 + r;
            const int gy = job.tile_y + rr - C::HALO;
            if (rr >= C::HALO && rr < C::HALO + C::TY && gy < g.H && gx < g.W)
                *reinterpret_cast<float4*>(job.pout + (size_t)gy * g.P + gx) =
                    make_float4(p[r][0], p[r][1], p[r][2], p[r][3]);
        }
    }
}

}  // namespace natrix
