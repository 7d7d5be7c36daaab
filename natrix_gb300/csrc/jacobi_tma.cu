// Plain Jacobi pressure sweeps (shader.Poisson.comp:17-38, looped K times by
// natrix/core/fluid_simulator.py:251-255), temporally blocked: one launch runs
// up to HALO sweeps on tiles loaded with a HALO-cell halo by TMA
// (cp.async.bulk.tensor.2d) and writes only the tile interior.  Every sweep
// evaluates exactly the reference's expression
//     p' = (pL + pR + pB + pT - b) * 0.25
// (neighbour replaced by the centre when it is an obstacle or beyond a wall)
// on the same inputs, so k fused sweeps equal k single sweeps bit for bit.
//
// TMA boxes: pressure and divergence (float) start HXP = round_up(HALO, 4)
// cells left of the tile so the box starts on a 16-byte boundary; the uint8
// neighbour flags start 16 cells left for the same reason.  TMA fills
// out-of-grid cells with zeros.  No in-grid cell ever reads them: a cell on a
// wall has the wall bit in its flags and substitutes its own pressure (the
// clamped neighbour index of common.sh:9-19 is the cell itself).
//
// Two tile kernels, each templated on a job source so the same body serves
// one grid and a batch of simulations (one work item per tile); tensor maps
// live in device memory:
//   * k_jacobi_rt: register tiled, persistent, next tile prefetched by TMA
//     while the current one sweeps (grids wider than ~100 cells);
//   * k_jacobi_tb: shared-memory sweeps on a shrinking region, one tile per
//     CTA, several CTAs per SM (narrow grids).
// Every mbarrier wait is bounded; on time-out the kernel records status bit 1,
// waits once more (bounded) for its copies, and returns without writing.
#include <cudaTypedefs.h>

#include <cstdlib>
#include <type_traits>

#include "jacobi_tile.cuh"

namespace natrix {

namespace {

// Jobs of one grid: tile t of a tiles_x-wide decomposition.
struct GridJobs {
    const CUtensorMap* p;
    const CUtensorMap* d;
    const CUtensorMap* f;
    float* pout;
    Grid g;
    int sweeps, tiles_x, n, tx, ty;
    const uint32_t* slow;  // tiles next to obstacles (TileMarks bits), or null
    const float2* vin;     // fused gradient subtraction (see TileJob), or null
    float2* vout;
    // Divergence, flags and marks were final before this launch's predecessor
    // grid started (it is a sweep launch of the same chain): the first tile's
    // divergence and flags may be fetched before the dependency wait.
    int static_ready;
    __device__ __forceinline__ TileJob operator()(int t) const {
        return TileJob{p, d, f, pout, g, sweeps, (t % tiles_x) * tx, (t / tiles_x) * ty,
                       vin, vout};
    }
};

// Most tiles one CTA of a balanced launch takes (kMaxBalancedTiles over the
// SM count, rounded up, with room to spare).
constexpr int kMaxCtaTiles = 16;

template <class Jobs>
__device__ __forceinline__ const uint32_t* slow_marks(const Jobs&) { return nullptr; }
__device__ __forceinline__ const uint32_t* slow_marks(const GridJobs& j) { return j.slow; }
template <class Jobs>
__device__ __forceinline__ bool static_ready(const Jobs&) { return false; }
__device__ __forceinline__ bool static_ready(const GridJobs& j) { return j.static_ready != 0; }

// Balanced deal of n tiles to G CTAs, computed by one warp for CTA b.  Order:
// the marked (slow) tiles, then the others, each in index order; position p
// of that order goes to CTA p mod G in even rounds and G - 1 - (p mod G) in
// odd rounds, so CTA b takes the positions b, 2G - 1 - b, 2G + b, ... and a
// slow tile dealt early is followed by a plain tile dealt late.  Writes the
// tiles to out[] and returns their count (a permutation of 0..n-1 over all
// CTAs).  Needs n <= 32 * 32.
__device__ int balanced_tiles(const uint32_t* slow, int n, int b, int G, int* out) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int base = lane * 32;
    const uint32_t valid = base >= n ? 0u : (n - base >= 32 ? FULL : (1u << (n - base)) - 1u);
    const uint32_t ws = (base < n ? slow[lane] : 0u) & valid;
    const uint32_t wz = ~ws & valid;
    int is = __popc(ws), iz = __popc(wz);  // inclusive prefix counts over lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(FULL, is, o), c = __shfl_up_sync(FULL, iz, o);
        if (lane >= o) {
            is += a;
            iz += c;
        }
    }
    const int n_slow = __shfl_sync(FULL, is, 31);
    int count = 0;
    for (int k = 0;; ++k) {
        const int p = (k & 1) ? (k + 1) * G - 1 - b : k * G + b;
        if (p >= n || count >= kMaxCtaTiles) break;
        const bool s = p < n_slow;
        const int q = s ? p : p - n_slow;
        const int incl = s ? is : iz;
        uint32_t w = s ? ws : wz;
        const unsigned hit = __ballot_sync(FULL, incl > q);
        const int src = __ffs(hit) - 1;  // lane holding the q-th tile of its kind
        if (lane == src) {
            for (int r = q - (incl - __popc(w)); r > 0; --r) w &= w - 1u;
            out[count] = base + __ffs(w) - 1;
        }
        ++count;
    }
    return count;
}

// Jobs of a batch: item t names a simulation, a tile origin, a sweep count
// and the source pressure buffer.
struct BatchJobs {
    const JacobiBatchItem* items;
    const JacobiBatchSim* sims;
    int n;
    __device__ __forceinline__ TileJob operator()(int t) const {
        const JacobiBatchItem it = items[t];
        const JacobiBatchSim& s = sims[it.sim];
        return TileJob{&s.maps.p[it.src], &s.maps.div, &s.maps.flags, s.p[1 - it.src], s.g,
                       it.sweeps, it.tile_x, it.tile_y, nullptr, nullptr};
    }
};

template <class C, class Jobs>
__global__ void __launch_bounds__(C::THREADS_X* C::THREADS_Y)
    k_jacobi_tb(const Jobs jobs, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
    __shared__ int s_ok;

    pdl_enter();
    const TileJob job = jobs(blockIdx.x);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
        mbar_expect_tx(bar, 2 * C::P_BYTES + C::F_BYTES);
        tma_load_2d(smem + C::OFF_A, job.p, job.tile_x - C::HXP, job.tile_y - C::HALO, bar);
        tma_load_2d(smem + C::OFF_D, job.d, job.tile_x - C::HXP, job.tile_y - C::HALO, bar);
        tma_load_2d(smem + C::OFF_F, job.f, job.tile_x - C::HXF, job.tile_y - C::HALO, bar);
        bool ok = wait_phase(bar, 0);
        if (!ok) {
            atomicOr(status, 1);
            wait_phase(bar, 0);  // let the copies land before the CTA exits
        }
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) return;
    tb_tile_body<C>(job, smem);
}


// ---------------------------------------------------------------------------
// Register-tiled, persistent variant (the per-tile work is rt_tile_body): one
// CTA of C::THREADS threads per SM walks its tiles; once every thread has
// copied the current tile's staging buffers into registers, the elected
// thread issues the TMA loads of the CTA's next job into the same staging
// buffers, so the copy overlaps this tile's sweeps.
template <class C, class Jobs>
__global__ void __launch_bounds__(C::THREADS, 1)
    k_jacobi_rt(const Jobs jobs, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
    __shared__ int s_ok;

    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    // Programmatic dependent launch: wait, then trigger (a successor starts
    // only after every CTA here has passed its wait).  When the static inputs
    // are final the deal and the first tile's divergence / flags copies run
    // before the wait.
    const bool early = static_ready(jobs);
    if (!early) pdl_wait();
    // this CTA's tiles: the balanced deal when the tiles are marked, else
    // blockIdx.x + k * gridDim.x
    __shared__ int s_tiles[kMaxCtaTiles];
    __shared__ int s_count;
    const uint32_t* slow = slow_marks(jobs);
    const bool balanced = slow != nullptr && jobs.n <= kMaxBalancedTiles &&
                          (jobs.n + (int)gridDim.x - 1) / (int)gridDim.x <= kMaxCtaTiles;
    if (balanced) {
        if (w == 0) {
            const int cnt = balanced_tiles(slow, jobs.n, blockIdx.x, gridDim.x, s_tiles);
            if (lane == 0) s_count = cnt;
        }
        __syncthreads();
    }
    const int n_mine = balanced ? s_count
                                : (jobs.n > (int)blockIdx.x
                                       ? (jobs.n - 1 - (int)blockIdx.x) / (int)gridDim.x + 1
                                       : 0);
    auto tile_of = [&](int k) {
        return balanced ? s_tiles[k] : (int)blockIdx.x + k * (int)gridDim.x;
    };
    if (n_mine == 0) {
        if (early) pdl_wait();
        pdl_trigger();
        return;
    }
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
        const TileJob first = jobs(tile_of(0));
        issue_static_loads<C>(smem, bar, first);
        if (early) pdl_wait();
        issue_pressure_load<C>(smem, bar, first);
    } else if (early) {
        pdl_wait();
    }
    pdl_trigger();
    uint32_t parity = 0;
    for (int k = 0; k < n_mine; ++k, parity ^= 1u) {
        const TileJob job = jobs(tile_of(k));
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

        rt_tile_body<C>(job, smem, [&] {
            // staging consumed: prefetch the next job into it
            if (threadIdx.x == 0 && k + 1 < n_mine) {
                fence_proxy_async();
                issue_tile_loads<C>(smem, bar, jobs(tile_of(k + 1)));
            }
        });
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

// NATRIX_JACOBI_VARIANT forces one tile shape on every single grid (for
// comparison runs): 0 the shared-memory kernel, 1 / 2 / 3 the register tiles
// RtA / RtB / RtC (TB on grids at most 96 cells wide, which the register
// tiles do not serve); otherwise the tile shape is chosen by jacobi_config.
int forced_variant() {
    static int v = -2;
    if (v == -2) {
        const char* e = getenv("NATRIX_JACOBI_VARIANT");
        v = (e && e[0] >= '0' && e[0] <= '3' && e[1] == 0) ? e[0] - '0' : -1;
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

template <class K>
cudaError_t set_smem(K kernel, int bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <class C, class Jobs>
cudaError_t launch_rt_jobs(const Jobs& jobs, int* status, cudaStream_t st, bool pdl) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = set_smem(k_jacobi_rt<C, Jobs>, C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (jobs.n == 0) return cudaSuccess;
    const int grid = jobs.n < num_sms() ? jobs.n : num_sms();
    return launch_kernel(pdl, k_jacobi_rt<C, Jobs>, dim3(grid), dim3(C::THREADS), C::SMEM, st, jobs,
                         status);
}

template <class C, class Jobs>
cudaError_t launch_tb_jobs(const Jobs& jobs, int* status, cudaStream_t st, bool pdl) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = set_smem(k_jacobi_tb<C, Jobs>, C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (jobs.n == 0) return cudaSuccess;
    return launch_kernel(pdl, k_jacobi_tb<C, Jobs>, dim3(jobs.n), dim3(C::THREADS_X, C::THREADS_Y),
                         C::SMEM, st, jobs, status);
}

template <class C>
void box_of(int* bx, int* by, int* bfx) {
    *bx = C::RX;
    *by = C::RY;
    *bfx = C::RXF;
}

}  // namespace

int jacobi_max_sweeps_per_launch() { return Tb::HALO < RtA::HALO ? Tb::HALO : RtA::HALO; }

// Time of one sweep launch in units of a row sweep on one SM: rounds of
// tiles over the SMs times the region rows each tile sweeps.
template <class C>
long rt_latency(Grid g) {
    const long tx = (g.W + C::TX - 1) / C::TX, ty = (g.H + C::TY - 1) / C::TY;
    const long sms = num_sms();
    return (tx * ty + sms - 1) / sms * C::RY;
}

int jacobi_config(Grid g) {
    const int forced = forced_variant();
    if (forced == JACOBI_TB) return JACOBI_TB;
    // grids narrower than one register tile waste most of its 128 columns
    if (g.W <= 96) return JACOBI_TB;
    if (forced > 0) return forced;
    const int tall = rt_cost<RtB>(g) < rt_cost<RtA>(g) ? JACOBI_RT_B : JACOBI_RT_A;
    const long t_tall = tall == JACOBI_RT_B ? rt_latency<RtB>(g) : rt_latency<RtA>(g);
    // short tiles where they shorten the launch (grids whose tall tiles
    // leave most SMs idle).  Measured per step (eps 0.35, 12 discs; 256^2
    // eps 0, no discs): 256^2 K40 68.0 -> 40.2 us, 512^2 K80 158.8 -> 113.5,
    // 768^2 K80 171.4 -> 159.6; 1024^2 K40 113 with tall tiles, 138 short.
    return rt_latency<RtC>(g) < t_tall ? JACOBI_RT_C : tall;
}

template <class C>
void rt_marks(Grid g, TileMarks* m) {
    m->tx = C::TX;
    m->ty = C::TY;
    m->rx = C::RX;
    m->ry = C::RY;
    m->hxp = C::HXP;
    m->halo = C::HALO;
    m->tiles_x = (g.W + C::TX - 1) / C::TX;
    m->tiles_y = (g.H + C::TY - 1) / C::TY;
}

bool jacobi_tile_marks(int config, Grid g, TileMarks* out) {
    TileMarks m{};
    if (config == JACOBI_RT_A)
        rt_marks<RtA>(g, &m);
    else if (config == JACOBI_RT_B)
        rt_marks<RtB>(g, &m);
    else if (config == JACOBI_RT_C)
        rt_marks<RtC>(g, &m);
    else
        return false;
    const long tiles = (long)m.tiles_x * m.tiles_y;
    if (tiles > kMaxBalancedTiles) return false;
    m.words = (int)((tiles + 31) / 32);
    *out = m;
    return true;
}

void jacobi_tile(int config, int* tx, int* ty) {
    switch (config) {
        case JACOBI_RT_A: *tx = RtA::TX; *ty = RtA::TY; break;
        case JACOBI_RT_B: *tx = RtB::TX; *ty = RtB::TY; break;
        case JACOBI_RT_C: *tx = RtC::TX; *ty = RtC::TY; break;
        default: *tx = Tb::TX; *ty = Tb::TY; break;
    }
}

bool jacobi_encode_maps_for(JacobiMaps* maps, int config, float* p0, float* p1, float* div,
                            uint8_t* flags, Grid g, const char** err) {
    int bx, by, bfx;
    if (config == JACOBI_RT_A)
        box_of<RtA>(&bx, &by, &bfx);
    else if (config == JACOBI_RT_B)
        box_of<RtB>(&bx, &by, &bfx);
    else if (config == JACOBI_RT_C)
        box_of<RtC>(&bx, &by, &bfx);
    else
        box_of<Tb>(&bx, &by, &bfx);
    maps->config = config;
    return encode_2d(&maps->p[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p0, g, bx, by, err) &&
           encode_2d(&maps->p[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p1, g, bx, by, err) &&
           encode_2d(&maps->div, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, div, g, bx, by, err) &&
           encode_2d(&maps->flags, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, flags, g, bfx, by, err);
}

cudaError_t launch_jacobi(const JacobiMaps* d_maps, int config, float* const pbuf[2], int src,
                          Grid g, int sweeps, const uint32_t* slow, int static_ready,
                          const float2* vin, float2* vout, int* status, cudaStream_t st) {
    if (sweeps < 1 || sweeps > jacobi_max_sweeps_per_launch()) return cudaErrorInvalidValue;
    // the fused gradient needs the register-tiled kernel and one valid halo cell
    if (vin && (config == JACOBI_TB || sweeps >= jacobi_max_sweeps_per_launch()))
        return cudaErrorInvalidValue;
    int tx, ty;
    jacobi_tile(config, &tx, &ty);
    const int tiles_x = (g.W + tx - 1) / tx, tiles_y = (g.H + ty - 1) / ty;
    const GridJobs jobs{&d_maps->p[src], &d_maps->div, &d_maps->flags, pbuf[1 - src], g,
                        sweeps, tiles_x, tiles_x * tiles_y, tx, ty, slow, vin, vout,
                        static_ready ? 1 : 0};
    const bool pdl = pdl_enabled();
    if (config == JACOBI_RT_A) return launch_rt_jobs<RtA>(jobs, status, st, pdl);
    if (config == JACOBI_RT_B) return launch_rt_jobs<RtB>(jobs, status, st, pdl);
    if (config == JACOBI_RT_C) return launch_rt_jobs<RtC>(jobs, status, st, pdl);
    return launch_tb_jobs<Tb>(jobs, status, st, pdl);
}

cudaError_t launch_jacobi_batch(int config, const JacobiBatchItem* items, int n_items,
                                const JacobiBatchSim* sims, int* status, cudaStream_t st) {
    const BatchJobs jobs{items, sims, n_items};
    // replayed from a CUDA graph: plain stream order
    if (config == JACOBI_RT_A) return launch_rt_jobs<RtA>(jobs, status, st, false);
    if (config == JACOBI_RT_B) return launch_rt_jobs<RtB>(jobs, status, st, false);
    return launch_tb_jobs<Tb>(jobs, status, st, false);
}

}  // namespace natrix
