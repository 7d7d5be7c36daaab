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
// A third, k_jacobi_chain, runs every chunk of HALO sweeps of a step in one
// persistent launch on grids with a register tile for every SM: tiles wait
// for their neighbours' previous chunk instead of a launch boundary (see the
// comment above it).
// Every mbarrier wait is bounded; on time-out the kernel records status bit 1,
// waits once more (bounded) for its copies, and returns without writing (the
// chain instead skips that tile and still counts it, so no CTA waits on it).
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

// Sweeps per chunk of the sweep chain (its tiles' halo) and the offset of the
// per-tile counters in its sync block (the claim counter in a line of its own).
constexpr int kChainSweeps = 8;
constexpr int kChainDone = 32;

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
__global__ void __launch_bounds__(C::THREADS, C::CTAS)
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

// ---------------------------------------------------------------------------
// A step's whole sweep phase in one persistent launch: `chunks` chunks of up
// to HALO sweeps (the last one may also subtract the gradient), each chunk
// over every tile, ping-ponging between the two pressure buffers (chunk m
// reads pbuf[(src0 + m) & 1]).  Items (chunk m, tile) are claimed from a
// counter in chunk order, the tiles of a chunk with the marked (obstacle)
// tiles first.  Instead of a launch boundary between chunks, an item of chunk
// m >= 1 waits until the 3x3 tiles around its own have finished chunk m - 1
// (one counter of finished chunks per tile): those are the only tiles whose
// output its region reads (HALO <= the tile size), and the only earlier
// readers of the output tile it overwrites (the buffer chunk m - 1 read).
// Dependencies point to items claimed earlier, so the earliest unfinished
// item can always run, whatever the number of resident CTAs; a CTA counts
// its finished tile before it waits on anything.
//
// Thread 0 claims the next item while the current one's copies land; once
// the current tile sits in registers it issues the next item's copies into
// the freed staging buffers, the pressure copy only if the neighbourhood is
// done (else after the tile, once it is).  After its output stores a tile is
// released (one fence) and counted.  Every launch starts from zeroed
// counters: the last CTA to leave (an exit count) zeroes them, when no other
// CTA touches them any more, so the launch's parameters do not change from
// step to step and a captured graph replays it correctly.  A wait that runs
// out (about a second) sets status bit 2 and the item runs anyway.
struct ChainJobs {
    const JacobiMaps* maps;  // device copy of the grid's maps
    float* pbuf[2];
    Grid g;
    int sweeps, chunks, src0;
    int tiles_x, tiles_y, n, tx, ty;
    const uint32_t* slow;  // tile marks of the step (null: tile order)
    const float2* vin;     // gradient subtraction fused into the last chunk, or null
    float2* vout;
    unsigned* sync;  // [0]: claims; [1]: CTAs done; [kChainDone + t]: chunks tile t finished
    __device__ __forceinline__ TileJob job(int chunk, int t) const {
        const int src = (src0 + chunk) & 1;
        const int left = sweeps - chunk * kChainSweeps;
        const bool last = chunk == chunks - 1;
        return TileJob{&maps->p[src], &maps->div, &maps->flags, pbuf[1 - src], g,
                       left < kChainSweeps ? left : kChainSweeps, (t % tiles_x) * tx,
                       (t / tiles_x) * ty, last ? vin : nullptr, last ? vout : nullptr};
    }
    // Have the tiles around t finished chunk m - 1?  The nine counters are
    // read together (relaxed); when they all have, one fence gives the copies
    // that follow acquire order.
    __device__ __forceinline__ bool deps_ready(int m, int t) const {
        if (m == 0) return true;
        const unsigned target = (unsigned)m;
        const int cx = t % tiles_x, cy = t / tiles_x;
        const int x0 = cx > 0 ? cx - 1 : cx, x1 = cx < tiles_x - 1 ? cx + 1 : cx;
        const int y0 = cy > 0 ? cy - 1 : cy, y1 = cy < tiles_y - 1 ? cy + 1 : cy;
        unsigned v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const int x = min(x0 + k % 3, x1), y = min(y0 + k / 3, y1);
            v[k] = ld_relaxed_u32(sync + kChainDone + y * tiles_x + x);
        }
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 9; ++k) ok = ok && (int)(v[k] - target) >= 0;
        if (ok) asm volatile("fence.acq_rel.gpu;" ::: "memory");
        return ok;
    }
    // bounded wait for deps_ready
    __device__ __forceinline__ bool wait_deps(int m, int t) const {
        for (int it = 0; it < (1 << 24); ++it) {
            if (deps_ready(m, t)) return true;
            __nanosleep(64);
        }
        return false;
    }
};

// Tiles of a chunk in claim order: the marked tiles, then the others, each
// in index order (one warp; n <= kMaxBalancedTiles).
__device__ void chain_order(const uint32_t* slow, int n, int* order) {
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
    int ps = is - __popc(ws), pz = n_slow + iz - __popc(wz);
    for (uint32_t w = ws; w; w &= w - 1u) order[ps++] = base + __ffs(w) - 1;
    for (uint32_t w = wz; w; w &= w - 1u) order[pz++] = base + __ffs(w) - 1;
}

template <class C>
__global__ void __launch_bounds__(C::THREADS, C::CTAS)
    k_jacobi_chain(const __grid_constant__ ChainJobs J, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
    __shared__ int s_order[kMaxBalancedTiles];
    // s_next is set by thread 0 during a tile (after the barrier that starts
    // it) and read by every thread after the tile
    __shared__ int s_cur, s_next, s_pending, s_ok, s_last;
    const int tid = threadIdx.x;
    const int total = J.chunks * J.n;
    const bool ordered = J.slow != nullptr && J.n <= kMaxBalancedTiles;

    pdl_wait();  // the divergence launch's pressure, divergence, flags and marks
    if (ordered && tid < 32) chain_order(J.slow, J.n, s_order);
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_barrier_init();
        s_cur = (int)atomicAdd(J.sync, 1u);
    }
    __syncthreads();
    pdl_trigger();
    int cur = s_cur;
    auto tile_of = [&](int i) {
        const int q = i % J.n;
        return ordered ? s_order[q] : q;
    };
    if (tid == 0 && cur < total) {
        const int t = tile_of(cur), m = cur / J.n;
        const TileJob j = J.job(m, t);
        issue_static_loads<C>(smem, bar, j);
        if (!J.wait_deps(m, t)) atomicOr(status, 2);
        fence_before_tma();
        issue_pressure_load<C>(smem, bar, j);
    }
    for (uint32_t parity = 0; cur < total; parity ^= 1u) {
        const int t = tile_of(cur);
        const TileJob job = J.job(cur / J.n, t);
        unsigned claimed = 0;  // thread 0: the next item, in flight during the copy wait
        if (tid == 0) {
            claimed = atomicAdd(J.sync, 1u);
            bool ok = wait_phase(bar, parity);
            if (!ok) {
                atomicOr(status, 1);
                wait_phase(bar, parity);  // let the copies land before the CTA goes on
            }
            s_ok = ok ? 1 : 0;
        }
        __syncthreads();
        // a copy that did not land (status bit 1): the tile is skipped but
        // still counted, so that no other CTA waits for it
        if (s_ok)
            rt_tile_body<C>(job, smem, [&] {
                // staging consumed: prefetch what of the next item is ready
                // into the freed staging buffers
                if (tid != 0) return;
                const int nx = (int)claimed;
                s_next = nx;
                s_pending = 0;
                if (nx >= total) return;
                const int nt = tile_of(nx), nm = nx / J.n;
                const TileJob nj = J.job(nm, nt);
                fence_proxy_async();
                issue_static_loads<C>(smem, bar, nj);
                if (J.deps_ready(nm, nt)) {
                    fence_before_tma();
                    issue_pressure_load<C>(smem, bar, nj);
                } else {
                    s_pending = 1;
                }
            });
        else if (tid == 0) {
            s_next = (int)claimed;
            s_pending = 2;  // nothing issued for it yet
        }
        __syncthreads();  // every output store of the tile issued; s_next set
        if (tid == 0) {
            // release the tile's stores (ordered before this thread by the
            // barrier), then count the tile
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" ::"l"(J.sync + kChainDone + t)
                         : "memory");
        }
        const int next = s_next;
        if (next < total && tid == 0 && s_pending) {
            const int t2 = tile_of(next), m2 = next / J.n;
            const TileJob nj = J.job(m2, t2);
            if (s_pending == 2) {
                fence_proxy_async();
                issue_static_loads<C>(smem, bar, nj);
            }
            if (!J.wait_deps(m2, t2)) atomicOr(status, 2);
            fence_before_tma();
            issue_pressure_load<C>(smem, bar, nj);
        }
        cur = next;
    }
    // Leave: this CTA's claims and counts are done (its last count and its
    // claim past the list come before the fence); the last CTA out zeroes
    // the counters for the next launch.
    if (tid == 0) {
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        s_last = atomicAdd(J.sync + 1, 1u) == gridDim.x - 1 ? 1 : 0;
        if (s_last) asm volatile("fence.acq_rel.gpu;" ::: "memory");
    }
    __syncthreads();
    if (s_last)
        for (int i = tid; i < kChainDone + J.n; i += C::THREADS) J.sync[i] = 0u;
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
// comparison runs): 0 the shared-memory kernel, 1 / 2 / 3 / 4 the register
// tiles RtA / RtB / RtC / RtD (TB on grids at most 96 cells wide, which the
// register tiles do not serve); otherwise the tile shape is chosen by
// jacobi_config.
int forced_variant() {
    static int v = -2;
    if (v == -2) {
        const char* e = getenv("NATRIX_JACOBI_VARIANT");
        v = (e && e[0] >= '0' && e[0] <= '4' && e[1] == 0) ? e[0] - '0' : -1;
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
    const int slots = num_sms() * C::CTAS;
    const int grid = jobs.n < slots ? jobs.n : slots;
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
    else if (config == JACOBI_RT_D)
        rt_marks<RtD>(g, &m);
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
        case JACOBI_RT_D: *tx = RtD::TX; *ty = RtD::TY; break;
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
    else if (config == JACOBI_RT_D)
        box_of<RtD>(&bx, &by, &bfx);
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
    if (config == JACOBI_RT_D) return launch_rt_jobs<RtD>(jobs, status, st, pdl);
    return launch_tb_jobs<Tb>(jobs, status, st, pdl);
}

// The chain pays where a chunk has a tile for every SM: measured per step,
// 2048^2 K80 (304 tiles) 341.9 -> 327.6 us; 256^2 K40 (48 tiles) 40.2 -> 45.2.
int jacobi_chain_sync_words(int config, Grid g) {
    if (config == JACOBI_TB) return 0;
    int tx, ty;
    jacobi_tile(config, &tx, &ty);
    const int tiles = ((g.W + tx - 1) / tx) * ((g.H + ty - 1) / ty);
    return tiles < num_sms() ? 0 : kChainDone + tiles;
}

template <class C>
cudaError_t launch_chain(const ChainJobs& jobs, int grid, int* status, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = set_smem(k_jacobi_chain<C>, C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return launch_kernel(pdl_enabled(), k_jacobi_chain<C>, dim3(grid), dim3(C::THREADS), C::SMEM,
                         st, jobs, status);
}

cudaError_t launch_jacobi_chain(const JacobiMaps* d_maps, int config, float* const pbuf[2],
                                int src, Grid g, int sweeps, const uint32_t* slow,
                                const float2* vin, float2* vout, unsigned* sync, bool* fused,
                                int* status, cudaStream_t st) {
    static_assert(kChainSweeps == RtA::HALO && kChainSweeps == RtB::HALO &&
                      kChainSweeps == RtC::HALO && kChainSweeps == RtD::HALO,
                  "a chunk is one tile halo of sweeps");
    if (config == JACOBI_TB || sweeps < 1) return cudaErrorInvalidValue;
    int tx, ty;
    jacobi_tile(config, &tx, &ty);
    const int tiles_x = (g.W + tx - 1) / tx, tiles_y = (g.H + ty - 1) / ty;
    const int chunks = (sweeps + kChainSweeps - 1) / kChainSweeps;
    const int last = sweeps - (chunks - 1) * kChainSweeps;
    // the fused gradient needs one valid halo cell after the last chunk
    const bool fuse = vin && last < kChainSweeps;
    const int n = tiles_x * tiles_y;
    const int slots = num_sms() * (config == JACOBI_RT_D ? RtD::CTAS : 1);
    const int grid = n * chunks < slots ? n * chunks : slots;
    const ChainJobs jobs{d_maps, {pbuf[0], pbuf[1]}, g, sweeps, chunks, src, tiles_x, tiles_y, n,
                         tx, ty, slow, fuse ? vin : nullptr, fuse ? vout : nullptr, sync};
    cudaError_t e;
    if (config == JACOBI_RT_A)
        e = launch_chain<RtA>(jobs, grid, status, st);
    else if (config == JACOBI_RT_B)
        e = launch_chain<RtB>(jobs, grid, status, st);
    else if (config == JACOBI_RT_C)
        e = launch_chain<RtC>(jobs, grid, status, st);
    else
        e = launch_chain<RtD>(jobs, grid, status, st);
    if (e == cudaSuccess) *fused = fuse;
    return e;
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
