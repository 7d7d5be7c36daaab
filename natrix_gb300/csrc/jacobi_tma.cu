// Plain Jacobi pressure sweeps (shader.Poisson.comp:17-38, looped K times by
// natrix/core/fluid_simulator.py:251-255), temporally blocked.
//
// One CTA owns a TX x TY output tile.  A single elected thread issues three
// TMA tile loads (cp.async.bulk.tensor.2d) of the tile plus a halo of HALO
// cells: pressure and divergence (float, x-halo rounded up to 4 cells so the
// box starts on a 16-byte boundary) and the neighbour-substitution flags
// (uint8, x-halo 16 for the same reason), completing on one mbarrier.  The
// CTA then runs `sweeps` <= HALO sweeps in shared memory, ping-ponging
// between two pressure buffers on a region that shrinks by one cell per
// sweep, and writes the tile interior back with 16-byte stores.  Every sweep
// evaluates exactly the reference's expression
//     p' = (pL + pR + pB + pT - b) * 0.25
// on the same inputs, so k fused sweeps equal k single sweeps bit for bit.
//
// TMA fills out-of-grid cells with zeros.  No in-grid cell ever reads them:
// a cell on a wall has the wall bit in its flags and substitutes its own
// pressure (the clamped neighbour index of common.sh:9-19 is the cell).
// Out-of-grid halo cells compute values nobody reads.
//
// The mbarrier wait is bounded; on time-out the kernel records status bit 1,
// waits once more (bounded) for its copies, and returns without writing.
#include <cudaTypedefs.h>

#include <cstdlib>

#include "kernels.cuh"

namespace natrix {

namespace {

constexpr int align128(int b) { return (b + 127) / 128 * 128; }

template <int TX_, int TY_, int HALO_>
struct JacCfg {
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
    static constexpr int THREADS_X = 32, THREADS_Y = 8;
    static_assert(TX % 16 == 0, "tile width must keep the uint8 box 16-byte aligned");
    static_assert(RX <= 256 && RY <= 256 && RXF <= 256, "TMA box dimensions are <= 256");
};

using Cfg = JacCfg<64, 32, 8>;

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

// Bounded wait for phase 0 of the tile barrier (about 4M polls).
__device__ __forceinline__ bool wait_tile(uint64_t* bar) {
    for (int it = 0; it < (1 << 22); ++it)
        if (mbar_try_wait(bar, 0)) return true;
    return false;
}

__global__ void __launch_bounds__(Cfg::THREADS_X* Cfg::THREADS_Y)
    k_jacobi_tb(const __grid_constant__ CUtensorMap tm_p, const __grid_constant__ CUtensorMap tm_div,
                const __grid_constant__ CUtensorMap tm_flags, float* __restrict__ pout, Grid g,
                int sweeps, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    float* A = reinterpret_cast<float*>(smem + Cfg::OFF_A);
    float* B = reinterpret_cast<float*>(smem + Cfg::OFF_B);
    const float* D = reinterpret_cast<const float*>(smem + Cfg::OFF_D);
    const uint8_t* F = reinterpret_cast<const uint8_t*>(smem + Cfg::OFF_F);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + Cfg::OFF_BAR);
    __shared__ int s_ok;

    const int tile_x = blockIdx.x * Cfg::TX, tile_y = blockIdx.y * Cfg::TY;
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (tx == 0 && ty == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
        mbar_expect_tx(bar, 2 * Cfg::P_BYTES + Cfg::F_BYTES);
        tma_load_2d(A, &tm_p, tile_x - Cfg::HXP, tile_y - Cfg::HALO, bar);
        tma_load_2d(smem + Cfg::OFF_D, &tm_div, tile_x - Cfg::HXP, tile_y - Cfg::HALO, bar);
        tma_load_2d(smem + Cfg::OFF_F, &tm_flags, tile_x - Cfg::HXF, tile_y - Cfg::HALO, bar);
        bool ok = wait_tile(bar);
        if (!ok) {
            atomicOr(status, 1);
            wait_tile(bar);  // let the copies land before the CTA exits
        }
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) return;

    constexpr int RX = Cfg::RX, RXF = Cfg::RXF, FOFF = Cfg::HXF - Cfg::HXP;
    for (int s = 1; s <= sweeps; ++s) {
        const float* src = (s & 1) ? A : B;
        float* dst = (s & 1) ? B : A;
        const int m = sweeps - s;
        const int x0 = Cfg::HXP - m, x1 = Cfg::HXP + Cfg::TX + m;
        const int y0 = Cfg::HALO - m, y1 = Cfg::HALO + Cfg::TY + m;
        for (int yy = y0 + ty; yy < y1; yy += Cfg::THREADS_Y) {
            for (int xx = x0 + tx; xx < x1; xx += Cfg::THREADS_X) {
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
    constexpr int GROUPS = Cfg::TX / 4;
    for (int k = ty * Cfg::THREADS_X + tx; k < Cfg::TY * GROUPS;
         k += Cfg::THREADS_X * Cfg::THREADS_Y) {
        const int row = k / GROUPS, grp = k % GROUPS;
        const int gy = tile_y + row, gx = tile_x + grp * 4;
        if (gy >= g.H || gx >= g.W) continue;
        const float4 v =
            *reinterpret_cast<const float4*>(res + (Cfg::HALO + row) * RX + Cfg::HXP + grp * 4);
        *reinterpret_cast<float4*>(pout + (size_t)gy * g.P + gx) = v;
    }
}

// ---------------------------------------------------------------------------
// Register-tiled, persistent variant (the default).  The CTA region is 128
// columns x NW*R rows; warp w owns rows [w*R, w*R + R), lane l owns columns
// [4l, 4l + 4), so each cell of the region lives in one thread's registers
// (pressure, divergence, flags) for all the launch's sweeps.  Per sweep a
// thread needs, per row, its left/right neighbours (warp shuffles of the
// adjacent lanes' edge columns) and the rows above/below (its own registers,
// or the neighbouring warps' edge rows exchanged through a double-buffered
// shared-memory slot: one barrier per sweep).  Rows whose warp holds no wall
// or obstacle neighbour take a substitution-free path (warp-uniform branch).
// Cells near the region edge compute from missing neighbours; after s sweeps
// the outer s rows / columns are invalid and the output tile (HALO rows and
// HXP columns in) stays exact for s <= HALO.
//
// The grid is persistent (one CTA per SM, tiles assigned round-robin): once
// every thread has copied the current tile's staging buffers into registers,
// the elected thread issues the TMA loads of the CTA's next tile into the
// same staging buffers, so the copy overlaps this tile's sweeps.
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
    static_assert(TX % 16 == 0, "tile width must keep the uint8 box 16-byte aligned");
    static_assert(RY <= 256 && RXF <= 256, "TMA box dimensions are <= 256");
    static_assert(TY > 0, "region too short for the halo");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};

// 16 warps x 8 rows: 128x128 region, 112x112 output tile
using RtA = RtCfg<8, 16, 8>;
// 16 warps x 9 rows: 128x144 region, 112x128 output tile
using RtB = RtCfg<9, 16, 8>;

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bounded wait for the given phase parity of the tile barrier.
__device__ __forceinline__ bool wait_phase(uint64_t* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

template <class C>
__device__ __forceinline__ void issue_tile_loads(unsigned char* smem, uint64_t* bar,
                                                 const CUtensorMap* tm_p,
                                                 const CUtensorMap* tm_div,
                                                 const CUtensorMap* tm_flags, int tile_x,
                                                 int tile_y) {
    mbar_expect_tx(bar, 2 * C::P_BYTES + C::F_BYTES);
    tma_load_2d(smem + C::OFF_P, tm_p, tile_x - C::HXP, tile_y - C::HALO, bar);
    tma_load_2d(smem + C::OFF_D, tm_div, tile_x - C::HXP, tile_y - C::HALO, bar);
    tma_load_2d(smem + C::OFF_F, tm_flags, tile_x - C::HXF, tile_y - C::HALO, bar);
}

template <class C>
__global__ void __launch_bounds__(C::THREADS, 1)
    k_jacobi_rt(const __grid_constant__ CUtensorMap tm_p, const __grid_constant__ CUtensorMap tm_div,
                const __grid_constant__ CUtensorMap tm_flags, float* __restrict__ pout, Grid g,
                int sweeps, int tiles_x, int n_tiles, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    const float* Ps = reinterpret_cast<const float*>(smem + C::OFF_P);
    const float* Ds = reinterpret_cast<const float*>(smem + C::OFF_D);
    const uint8_t* Fs = reinterpret_cast<const uint8_t*>(smem + C::OFF_F);
    float* X = reinterpret_cast<float*>(smem + C::OFF_X);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
    __shared__ int s_ok;

    constexpr int R = C::R, RX = C::RX;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int c0 = lane * 4, r0 = w * R;

    int tile = blockIdx.x;
    if (tile >= n_tiles) return;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
        issue_tile_loads<C>(smem, bar, &tm_p, &tm_div, &tm_flags, (tile % tiles_x) * C::TX,
                            (tile / tiles_x) * C::TY);
    }
    uint32_t parity = 0;
    for (; tile < n_tiles; tile += gridDim.x, parity ^= 1u) {
        const int tile_x = (tile % tiles_x) * C::TX, tile_y = (tile / tiles_x) * C::TY;
        if (threadIdx.x == 0) {
            bool ok = wait_phase(bar, parity);
            if (!ok) {
                atomicOr(status, 1);
                wait_phase(bar, parity);  // let the copies land before the CTA exits
            }
            s_ok = ok ? 1 : 0;
        }
        __syncthreads();
        if (!s_ok) return;

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
            if (__any_sync(FULL, f[r] != 0u)) slow |= 1u << r;
        }
        __syncthreads();  // staging consumed: prefetch the next tile into it
        const int next = tile + gridDim.x;
        if (threadIdx.x == 0 && next < n_tiles) {
            fence_proxy_async();
            issue_tile_loads<C>(smem, bar, &tm_p, &tm_div, &tm_flags, (next % tiles_x) * C::TX,
                                (next / tiles_x) * C::TY);
        }

        for (int s = 0; s < sweeps; ++s) {
            float* xs = X + (s & 1) * (C::NW * 2 * RX);
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
#pragma unroll
            for (int r = 0; r < R; ++r) {
                float cur[4], dn[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    cur[j] = p[r][j];
                    dn[j] = r < R - 1 ? p[r + 1][j] : below[j];
                }
                const float lft = __shfl_up_sync(FULL, cur[3], 1);
                const float rgt = __shfl_down_sync(FULL, cur[0], 1);
                const float L[4] = {lft, cur[0], cur[1], cur[2]};
                const float Rn[4] = {cur[1], cur[2], cur[3], rgt};
                if (slow & (1u << r)) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const uint32_t fb = f[r] >> (8 * j);
                        const float l = (fb & NB_L) ? cur[j] : L[j];
                        const float rr = (fb & NB_R) ? cur[j] : Rn[j];
                        const float b = (fb & NB_B) ? cur[j] : up[j];
                        const float t = (fb & NB_T) ? cur[j] : dn[j];
                        p[r][j] = (l + rr + b + t - d[r][j]) * 0.25f;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        p[r][j] = (L[j] + Rn[j] + up[j] + dn[j] - d[r][j]) * 0.25f;
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) up[j] = cur[j];
            }
        }

        // output tile: region rows [HALO, HALO + TY), columns [HXP, HXP + TX)
        if (c0 >= C::HXP && c0 < C::HXP + C::TX) {
            const int gx = tile_x + c0 - C::HXP;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int rr = r0 + r;
                const int gy = tile_y + rr - C::HALO;
                if (rr >= C::HALO && rr < C::HALO + C::TY && gy < g.H && gx < g.W)
                    *reinterpret_cast<float4*>(pout + (size_t)gy * g.P + gx) =
                        make_float4(p[r][0], p[r][1], p[r][2], p[r][3]);
            }
        }
    }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

bool encode_2d(CUtensorMap* map, CUtensorMapDataType dt, int elem_bytes, void* base, Grid g,
               int box_x, int box_y, const char** err) {
    auto fn = get_encode();
    if (!fn) {
        *err = "cuTensorMapEncodeTiled is unavailable from the driver";
        return false;
    }
    cuuint64_t dims[2] = {(cuuint64_t)g.W, (cuuint64_t)g.H};
    cuuint64_t strides[1] = {(cuuint64_t)g.P * (cuuint64_t)elem_bytes};
    cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_y};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, dt, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        *err = "cuTensorMapEncodeTiled failed";
        return false;
    }
    return true;
}

// Kernel variant: 0 = shared-memory sweeps (k_jacobi_tb), 1 = register tiled
// persistent (k_jacobi_rt, default).  NATRIX_JACOBI_VARIANT selects one for
// comparison.
int variant() {
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("NATRIX_JACOBI_VARIANT");
        v = (e && e[0] == '0') ? 0 : 1;
    }
    return v;
}

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
            n = 1;
    }
    return n;
}

// Cost of a register-tiled configuration on a grid: rounds of persistent
// tiles times the region cells each tile computes (lower is better).
template <class C>
double rt_cost(Grid g) {
    const long tx = (g.W + C::TX - 1) / C::TX, ty = (g.H + C::TY - 1) / C::TY;
    const long tiles = tx * ty, sms = num_sms();
    const long rounds = (tiles + sms - 1) / sms;
    return (double)rounds * C::RX * C::RY * (tiles < sms ? (double)tiles / sms : 1.0);
}

template <class C>
cudaError_t launch_rt(const JacobiMaps& maps, float* const pbuf[2], int src, Grid g, int sweeps,
                      int* status, cudaStream_t st) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_jacobi_rt<C>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int tiles_x = (g.W + C::TX - 1) / C::TX, tiles_y = (g.H + C::TY - 1) / C::TY;
    const int n_tiles = tiles_x * tiles_y;
    const int grid = n_tiles < num_sms() ? n_tiles : num_sms();
    k_jacobi_rt<C><<<grid, C::THREADS, C::SMEM, st>>>(maps.p[src], maps.div, maps.flags,
                                                      pbuf[1 - src], g, sweeps, tiles_x, n_tiles,
                                                      status);
    return cudaGetLastError();
}

}  // namespace

int jacobi_max_sweeps_per_launch() { return Cfg::HALO < RtA::HALO ? Cfg::HALO : RtA::HALO; }

int jacobi_config(Grid g) {
    if (variant() == 0) return 0;
    return rt_cost<RtB>(g) < rt_cost<RtA>(g) ? 2 : 1;
}

bool jacobi_encode_maps(JacobiMaps* maps, float* p0, float* p1, float* div, uint8_t* flags,
                        Grid g, const char** err) {
    const int cfg = jacobi_config(g);
    int bx = Cfg::RX, by = Cfg::RY, bfx = Cfg::RXF;
    if (cfg == 1) bx = RtA::RX, by = RtA::RY, bfx = RtA::RXF;
    if (cfg == 2) bx = RtB::RX, by = RtB::RY, bfx = RtB::RXF;
    maps->config = cfg;
    return encode_2d(&maps->p[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p0, g, bx, by, err) &&
           encode_2d(&maps->p[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p1, g, bx, by, err) &&
           encode_2d(&maps->div, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, div, g, bx, by, err) &&
           encode_2d(&maps->flags, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, flags, g, bfx, by, err);
}

cudaError_t launch_jacobi(const JacobiMaps& maps, float* const pbuf[2], int src, Grid g,
                          int sweeps, int* status, cudaStream_t st) {
    if (sweeps < 1 || sweeps > jacobi_max_sweeps_per_launch()) return cudaErrorInvalidValue;
    if (maps.config == 1) return launch_rt<RtA>(maps, pbuf, src, g, sweeps, status, st);
    if (maps.config == 2) return launch_rt<RtB>(maps, pbuf, src, g, sweeps, status, st);
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_jacobi_tb,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             Cfg::SMEM);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    dim3 grid((g.W + Cfg::TX - 1) / Cfg::TX, (g.H + Cfg::TY - 1) / Cfg::TY);
    dim3 block(Cfg::THREADS_X, Cfg::THREADS_Y);
    k_jacobi_tb<<<grid, block, Cfg::SMEM, st>>>(maps.p[src], maps.div, maps.flags,
                                                pbuf[1 - src], g, sweeps, status);
    return cudaGetLastError();
}

}  // namespace natrix
