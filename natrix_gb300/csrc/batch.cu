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
#include <vector>

#include "../../include/natrix.h"
#include "cells.cuh"

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
    int pad[2];
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
};

namespace {

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
    StepHeader hdr{dt, n, {0, 0}};
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
