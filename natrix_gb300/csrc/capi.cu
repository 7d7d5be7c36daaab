// C ABI (include/natrix.h): simulator and density handles, host-side op
// queues, per-step scheduling of the solver kernels.
//
// Step schedule (one FluidSimulator.update, natrix/core/fluid_simulator.py:174-280):
//   [obstacles]  queued shapes rasterised in one pass (fresh mask if the
//                previous step's reset is pending)
//   [forcing]    queued add_velocity / Gaussian splats in one pass, in place
//   advect       vel0 -> vel1          (InitBoundaries folded in)
//   [vorticity]  vel1 -> w, vel1 -> vel2     (skipped when vorticity == 0:
//                the reference then adds exactly zero force)
//   [viscosity]  cur -> other          (only when viscosity > 0, as :219-228)
//   divergence   cur -> div, flags, p = first sweep from zero
//   jacobi       iterations-1 sweeps, `sweeps_per_launch` fused per launch
//   subtract     cur, p -> vel0 (inside the last Jacobi launch when that one
//                has fewer sweeps than the tile halo, else its own launch)
//   obstacle reset: recorded on the host, applied lazily (the next raster
//                writes a fresh mask; until then kernels treat it as empty)
#include <cstdlib>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/natrix.h"
#include "kernels.cuh"

using namespace natrix;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace

// Restores the caller's current device on scope exit.
natrix::DeviceGuard::DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
}
natrix::DeviceGuard::~DeviceGuard() {
    int cur;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
}

int natrix::set_last_error(int code, const char* msg) {
    g_err = msg;
    return code;
}

namespace {

int cuda_fail(cudaError_t e, const char* what) {
    return fail(NATRIX_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define NX_CUDA(call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);        \
    } while (0)

// A kernel launch of handle `sim`, counted in its statistics.
#define NX_LAUNCH(sim, call)           \
    do {                               \
        NX_CUDA(call);                 \
        (sim)->stats.kernel_launches++; \
    } while (0)

int round_up(int v, int m) { return (v + m - 1) / m * m; }

}  // namespace

struct natrix_sim {
    int device = 0;
    Grid g{};
    natrix_params prm{};
    float2* vel[3] = {};
    float* p[2] = {};
    float* div = nullptr;
    float* vort = nullptr;
    uint8_t* mask = nullptr;
    uint8_t* flags = nullptr;
    int p_cur = 0;
    int* d_status = nullptr;
    double* d_res = nullptr;  // partials, then the 5 sums at the end
    double* h_res = nullptr;  // pinned
    int res_blocks = 0;
    JacobiMaps maps{};             // host copy (encoded at creation)
    JacobiMaps* d_maps = nullptr;  // device copy the sweep kernels read
    TileMarks marks{};             // sweep tiles next to obstacles (geometry; words = 0: off)
    uint32_t* d_marks[2] = {};     // this step's marks / the previous step's
    int marks_cur = 0;
    // counters of the one-launch sweep phase (launch_jacobi_chain)
    unsigned* d_chain = nullptr;
    int chain_words = 0;
    std::vector<ForceOp> fq;
    std::vector<ShapeOp> sq;
    bool mask_reset_pending = true;  // the mask memory does not hold the current obstacles
    // Blocks (kRasterBlock^2 cells) of the mask memory that may be non-zero;
    // mask_dirty_all when that is unknown (triangles, uploads, views handed out).
    std::vector<uint8_t> mask_dirty;
    bool mask_dirty_all = true;
    bool last_step_mask_zero = true;
    bool stepped = false;
    cudaStream_t last_stream = nullptr;
    natrix_stats stats{};
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timed;  // recorded phases
    std::vector<std::pair<int, int>> timed_counts;            // launches, sweeps
    std::vector<int> timed_fused;  // the phase's last launch also subtracted the gradient
};

struct natrix_density {
    natrix_sim* fluid = nullptr;
    Grid g{};
    float* rho[2] = {};
    int cur = 0;
    float speed = 500.0f;
    float dissipation = 1.0f;
    int simulate = 1;
    std::vector<ForceOp> fq;
};

namespace {

constexpr int kMaxSide = 32768;

void drop_timing_events(natrix_sim* s) {
    for (auto& pr : s->timed) {
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    s->timed.clear();
    s->timed_counts.clear();
    s->timed_fused.clear();
}

void free_sim(natrix_sim* s) {
    drop_timing_events(s);
    for (auto& v : s->vel) cudaFree(v);
    for (auto& q : s->p) cudaFree(q);
    cudaFree(s->div);
    cudaFree(s->vort);
    cudaFree(s->mask);
    cudaFree(s->flags);
    cudaFree(s->d_status);
    cudaFree(s->d_res);
    cudaFree(s->d_maps);
    cudaFree(s->d_marks[0]);
    cudaFree(s->d_marks[1]);
    cudaFree(s->d_chain);
    if (s->h_res) cudaFreeHost(s->h_res);
    delete s;
}

int default_sweeps() { return jacobi_max_sweeps_per_launch(); }

StepParams fluid_params(const natrix_sim* s, float dt, bool mask_zero) {
    StepParams sp{};
    sp.dt = dt;
    sp.speed = s->prm.speed;
    sp.dissipation = s->prm.dissipation;
    sp.vorticity = s->prm.vorticity;
    if (s->prm.viscosity > 0.0f) {
        // natrix/core/fluid_simulator.py:327-336: computed in double, passed as float
        const double alpha = 1.0 / (double)s->prm.viscosity;
        sp.alpha = (float)alpha;
        sp.rbeta = (float)(1.0 / (4.0 + alpha));
    }
    sp.has_borders = s->prm.has_borders ? 1 : 0;
    sp.mask_zero = mask_zero ? 1 : 0;
    return sp;
}

cudaStream_t stream_of(natrix_sim* s, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    s->last_stream = st;
    return st;
}

// Rasterise queued obstacle shapes.  Circles rasterise over the blocks they
// reach plus, when the mask is reset, the blocks the previous shapes left
// non-zero; the rest of the mask is already zero (or, without a reset,
// already right).  Triangles and unknown mask contents take the full grid.
int flush_shapes(natrix_sim* s, cudaStream_t st) {
    const Grid g = s->g;
    const int bx = (g.W + kRasterBlock - 1) / kRasterBlock, by = (g.H + kRasterBlock - 1) / kRasterBlock;
    const size_t nb = (size_t)bx * by;
    if (s->mask_dirty.size() != nb) {
        s->mask_dirty.assign(nb, 0);
        s->mask_dirty_all = true;
    }
    size_t done = 0;
    std::vector<uint8_t> cur;
    std::vector<uint16_t> ids;
    while (done < s->sq.size()) {
        const int n = (int)std::min<size_t>(kMaxOpsPerLaunch, s->sq.size() - done);
        const ShapeOp* ops = s->sq.data() + done;
        const bool fresh = s->mask_reset_pending;
        cur.assign(nb, 0);
        const bool bounded = nb <= 65536 && shape_blocks(ops, n, g, cur.data());
        bool full = !bounded || (fresh && s->mask_dirty_all);
        if (!full) {
            ids.clear();
            for (size_t b = 0; b < nb && !full; ++b)
                if (cur[b] || (fresh && s->mask_dirty[b])) {
                    if ((int)ids.size() == kMaxRasterBlocks) full = true;
                    else ids.push_back((uint16_t)b);
                }
        }
        if (full)
            NX_LAUNCH(s, launch_obstacles(s->mask, g, ops, n, fresh ? 1 : 0, st));
        else if (!ids.empty())
            NX_LAUNCH(s, launch_obstacles_blocks(s->mask, g, ops, n, fresh ? 1 : 0, ids.data(),
                                                 (int)ids.size(), st));
        if (fresh) {
            s->mask_dirty = cur;
            s->mask_dirty_all = !bounded;
        } else {
            for (size_t b = 0; b < nb; ++b) s->mask_dirty[b] |= cur[b];
            s->mask_dirty_all = s->mask_dirty_all || !bounded;
        }
        s->mask_reset_pending = false;
        done += n;
    }
    s->sq.clear();
    return NATRIX_OK;
}

// zeroed (may be null): ask the last launch to write the velocity border as
// zero (the start of a step, shader.InitBoundaries.comp); set to whether it
// did, which needs a velocity op in that launch.
int flush_force_list(natrix_sim* s, std::vector<ForceOp>& q, float2* vel, Grid gv, float* rho,
                     Grid gd, cudaStream_t st, bool* zeroed = nullptr) {
    if (zeroed) *zeroed = false;
    size_t done = 0;
    while (done < q.size()) {
        const int n = (int)std::min<size_t>(kMaxOpsPerLaunch, q.size() - done);
        bool zero = false;
        if (zeroed && vel && done + n == q.size())
            for (int k = 0; k < n && !zero; ++k)
                zero = q[done + k].kind == FORCE_CONE_VELOCITY || q[done + k].kind == FORCE_GAUSS;
        NX_LAUNCH(s, launch_forcing(vel, gv, rho, gd, q.data() + done, n, zero ? 1 : 0, st));
        if (zero) *zeroed = true;
        done += n;
    }
    q.clear();
    return NATRIX_OK;
}

int flush_fluid(natrix_sim* s, cudaStream_t st, bool* border_zeroed = nullptr) {
    int rc = flush_shapes(s, st);
    if (rc) return rc;
    return flush_force_list(s, s->fq, s->vel[0], s->g, nullptr, Grid{}, st, border_zeroed);
}

// Sparse velocity forcing for a step (on unless NATRIX_SPARSE_FORCING=0).
bool sparse_forcing_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("NATRIX_SPARSE_FORCING");
        return !(e && e[0] == '0');
    }();
    return on;
}

// The start of a step: the queued obstacles, then the velocity ops over the
// blocks they reach (launch_forcing_sparse) when that is possible, else over
// the whole grid.  *clamp_deferred: the advection must clamp its reads;
// *border_zeroed: the border holds zero.
int flush_fluid_for_step(natrix_sim* s, cudaStream_t st, bool* border_zeroed,
                         bool* clamp_deferred) {
    *clamp_deferred = false;
    int rc = flush_shapes(s, st);
    if (rc) return rc;
    if (sparse_forcing_enabled() && !s->fq.empty() && s->fq.size() <= (size_t)kMaxOpsPerLaunch) {
        cudaError_t e = cudaSuccess;
        if (launch_forcing_sparse(s->vel[0], s->g, s->fq.data(), (int)s->fq.size(),
                                  s->prm.has_borders ? 1 : 0, st, &e)) {
            NX_LAUNCH(s, e);
            s->fq.clear();
            *border_zeroed = s->prm.has_borders != 0;
            *clamp_deferred = true;
            return NATRIX_OK;
        }
    }
    return flush_force_list(s, s->fq, s->vel[0], s->g, nullptr, Grid{}, st,
                            s->prm.has_borders ? border_zeroed : nullptr);
}

int flush_density(natrix_density* d, cudaStream_t st) {
    return flush_force_list(d->fluid, d->fq, nullptr, Grid{}, d->rho[d->cur], d->g, st);
}

// NATRIX_JACOBI_CHAIN=0 runs a step's sweeps as one launch per chunk of the
// tile halo instead of one persistent launch.
bool jacobi_chain_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("NATRIX_JACOBI_CHAIN");
        return !(e && e[0] == '0');
    }();
    return on;
}

// `sweeps` Jacobi sweeps in launches of sweeps_per_launch.  With vin / vout
// the gradient subtraction rides on the last launch when that launch can
// take it (register-tiled tiles, fewer sweeps than the halo); *fused says
// whether it did.
int run_jacobi(natrix_sim* s, int sweeps, cudaStream_t st, const float2* vin = nullptr,
               float2* vout = nullptr, bool* fused = nullptr) {
    const int per = s->prm.sweeps_per_launch > 0 ? s->prm.sweeps_per_launch : default_sweeps();
    if (fused) *fused = false;
    if (sweeps <= 0) return NATRIX_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (s->timing) {
        NX_CUDA(cudaEventCreate(&e0));
        NX_CUDA(cudaEventCreate(&e1));
        NX_CUDA(cudaEventRecord(e0, st));
    }
    int launches = 0, total = sweeps;
    bool fuse_last = false;
    if (vin && s->prm.sweeps_per_launch == 0 && s->d_chain && jacobi_chain_enabled()) {
        // a step's sweeps: one persistent launch for every chunk
        const int chunks = (sweeps + default_sweeps() - 1) / default_sweeps();
        NX_LAUNCH(s, launch_jacobi_chain(s->d_maps, s->maps.config, s->p, s->p_cur, s->g, sweeps,
                                         s->d_marks[s->marks_cur], vin, vout, s->d_chain,
                                         &fuse_last, s->d_status, st));
        s->p_cur = (s->p_cur + chunks) & 1;
        sweeps = 0;
        launches = 1;
    }
    while (sweeps > 0) {
        const int k = sweeps < per ? sweeps : per;
        const bool last = k == sweeps;
        fuse_last = last && vin && s->maps.config != JACOBI_TB && k < default_sweeps();
        NX_LAUNCH(s, launch_jacobi(s->d_maps, s->maps.config, s->p, s->p_cur, s->g, k,
                                   s->d_marks[s->marks_cur], launches > 0 ? 1 : 0,
                                   fuse_last ? vin : nullptr, fuse_last ? vout : nullptr,
                                   s->d_status, st));
        s->p_cur ^= 1;
        sweeps -= k;
        ++launches;
    }
    s->stats.jacobi_launches += launches;
    s->stats.jacobi_sweeps += total;
    if (fused) *fused = fuse_last;
    if (s->timing) {
        NX_CUDA(cudaEventRecord(e1, st));
        s->timed.emplace_back(e0, e1);
        s->timed_counts.emplace_back(launches, total);
        s->timed_fused.push_back(fuse_last ? 1 : 0);
    }
    return NATRIX_OK;
}

bool valid_params(const natrix_params* p) {
    // natrix/core/fluid_simulator.py:58-111 (`value > 0` / `value >= 0`, so NaN fails)
    return p->speed > 0.0f && p->iterations > 0 && p->dissipation > 0.0f &&
           p->vorticity >= 0.0f && p->viscosity >= 0.0f && p->sweeps_per_launch >= 0 &&
           p->sweeps_per_launch <= jacobi_max_sweeps_per_launch();
}

int field_copy(natrix_sim* s, int32_t field, void* host, const void* chost, bool up,
               cudaStream_t st) {
    void* dev = nullptr;
    size_t esz = 4;
    switch (field) {
        case NATRIX_FIELD_VELOCITY: dev = s->vel[0]; esz = 8; break;
        case NATRIX_FIELD_PRESSURE: dev = s->p[s->p_cur]; break;
        case NATRIX_FIELD_DIVERGENCE: dev = s->div; break;
        case NATRIX_FIELD_VORTICITY: dev = s->vort; break;
        case NATRIX_FIELD_OBSTACLES: dev = s->mask; esz = 1; break;
        default: return fail(NATRIX_EINVAL, "unknown field id %d", field);
    }
    const size_t dpitch = (size_t)s->g.P * esz, hpitch = (size_t)s->g.W * esz;
    if (up)
        NX_CUDA(cudaMemcpy2DAsync(dev, dpitch, chost, hpitch, hpitch, s->g.H,
                                  cudaMemcpyHostToDevice, st));
    else
        NX_CUDA(cudaMemcpy2DAsync(host, hpitch, dev, dpitch, hpitch, s->g.H,
                                  cudaMemcpyDeviceToHost, st));
    return NATRIX_OK;
}

// Materialise a pending obstacle reset so the mask memory reads as empty.
int materialise_mask(natrix_sim* s, cudaStream_t st) {
    if (s->mask_reset_pending) {
        NX_CUDA(cudaMemsetAsync(s->mask, 0, (size_t)s->g.P * s->g.H, st));
        s->mask_reset_pending = false;
        std::fill(s->mask_dirty.begin(), s->mask_dirty.end(), (uint8_t)0);
        s->mask_dirty_all = false;
    }
    return NATRIX_OK;
}

}  // namespace

int natrix::sim_prepare_read(natrix_sim* s, cudaStream_t st, SimView* out) {
    s->last_stream = st;
    int rc = flush_fluid(s, st);
    if (rc) return rc;
    *out = SimView{s->vel[0], s->g, s->prm.speed, s->device};
    return NATRIX_OK;
}

void natrix::sim_describe(const natrix_sim* s, SimView* out) {
    *out = SimView{s->vel[0], s->g, s->prm.speed, s->device};
}

void natrix::sim_count_launches(natrix_sim* s, int n) { s->stats.kernel_launches += n; }

extern "C" {

const char* natrix_last_error(void) { return g_err.c_str(); }

const char* natrix_version(void) { return "natrix_gb300 0.1.0 (sm_103a)"; }

int natrix_create(int32_t width, int32_t height, natrix_sim** out) {
    if (!out) return fail(NATRIX_EINVAL, "out is NULL");
    *out = nullptr;
    if (width < 1 || height < 1)
        return fail(NATRIX_EINVAL, "grid size must be positive, got %dx%d", width, height);
    if (width > kMaxSide || height > kMaxSide)
        return fail(NATRIX_ERANGE, "grid side above the maximum %d: %dx%d", kMaxSide, width,
                    height);
    natrix_sim* s = new natrix_sim();
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        delete s;
        return fail(NATRIX_ECUDA, "no CUDA device");
    }
    s->g = Grid{width, height, round_up(width, 32)};
    s->prm = natrix_params{500.0f, 50, 1.0f, 0.0f, 0.1f, 1, 1, 0};
    const size_t cells = (size_t)s->g.P * s->g.H;
    auto alloc = [&](void** p, size_t bytes) {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
        return e;
    };
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 3 && e == cudaSuccess; ++i)
        e = alloc((void**)&s->vel[i], cells * sizeof(float2));
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = alloc((void**)&s->p[i], cells * 4);
    if (e == cudaSuccess) e = alloc((void**)&s->div, cells * 4);
    if (e == cudaSuccess) e = alloc((void**)&s->vort, cells * 4);
    if (e == cudaSuccess) e = alloc((void**)&s->mask, cells);
    if (e == cudaSuccess) e = alloc((void**)&s->flags, cells);
    if (e == cudaSuccess) e = alloc((void**)&s->d_status, sizeof(int));
    s->res_blocks = residual_partials(s->g);
    if (e == cudaSuccess) e = alloc((void**)&s->d_res, ((size_t)s->res_blocks + 1) * 5 * 8);
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_res, 5 * sizeof(double));
    if (e != cudaSuccess) {
        free_sim(s);
        return fail(e == cudaErrorMemoryAllocation ? NATRIX_ENOMEM : NATRIX_ECUDA,
                    "allocating a %dx%d simulator: %s", width, height, cudaGetErrorString(e));
    }
    s->mask_reset_pending = false;  // the memset left a valid empty mask
    s->mask_dirty.assign((size_t)((width + kRasterBlock - 1) / kRasterBlock) *
                             ((height + kRasterBlock - 1) / kRasterBlock),
                         0);
    s->mask_dirty_all = false;
    const char* err = nullptr;
    if (!jacobi_encode_maps_for(&s->maps, jacobi_config(s->g), s->p[0], s->p[1], s->div,
                                s->flags, s->g, &err)) {
        free_sim(s);
        return fail(NATRIX_ECUDA, "%s", err);
    }
    e = cudaMalloc(&s->d_maps, sizeof(JacobiMaps));
    if (e == cudaSuccess)
        e = cudaMemcpy(s->d_maps, &s->maps, sizeof(JacobiMaps), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && jacobi_tile_marks(s->maps.config, s->g, &s->marks)) {
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
            e = cudaMalloc(&s->d_marks[i], (size_t)s->marks.words * 4);
            if (e == cudaSuccess) e = cudaMemset(s->d_marks[i], 0, (size_t)s->marks.words * 4);
        }
    }
    s->chain_words = jacobi_chain_sync_words(s->maps.config, s->g);
    if (e == cudaSuccess && s->chain_words > 0) {
        e = cudaMalloc(&s->d_chain, (size_t)s->chain_words * 4);
        if (e == cudaSuccess) e = cudaMemset(s->d_chain, 0, (size_t)s->chain_words * 4);
    }
    if (e != cudaSuccess) {
        free_sim(s);
        return fail(NATRIX_ECUDA, "setting up the sweep tiles: %s", cudaGetErrorString(e));
    }
    *out = s;
    return NATRIX_OK;
}

int natrix_destroy(natrix_sim* s) {
    if (!s) return NATRIX_OK;
    DeviceGuard dg(s->device);
    cudaDeviceSynchronize();
    free_sim(s);
    return NATRIX_OK;
}

int natrix_set_params(natrix_sim* s, const natrix_params* p) {
    if (!s || !p) return fail(NATRIX_EINVAL, "NULL argument");
    if (!valid_params(p))
        return fail(NATRIX_EINVAL,
                    "invalid parameters: speed, iterations and dissipation must be > 0, "
                    "vorticity and viscosity >= 0, sweeps_per_launch in [0, %d]",
                    jacobi_max_sweeps_per_launch());
    s->prm = *p;
    return NATRIX_OK;
}

int natrix_get_params(const natrix_sim* s, natrix_params* p) {
    if (!s || !p) return fail(NATRIX_EINVAL, "NULL argument");
    *p = s->prm;
    return NATRIX_OK;
}

int natrix_add_velocity(natrix_sim* s, float px, float py, float vx, float vy, float radius) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    if (!s->prm.simulate) return NATRIX_OK;
    ForceOp op{FORCE_CONE_VELOCITY, px, py, radius, vx, vy, 0.0f, 0};
    s->fq.push_back(op);
    return NATRIX_OK;
}

int natrix_add_circle_obstacle(natrix_sim* s, float px, float py, float radius,
                               int32_t is_static) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    if (!s->prm.simulate) return NATRIX_OK;
    ShapeOp op{SHAPE_CIRCLE, is_static ? 1 : 0, {px, py, radius, 0, 0, 0}};
    s->sq.push_back(op);
    return NATRIX_OK;
}

int natrix_add_triangle_obstacle(natrix_sim* s, float x1, float y1, float x2, float y2,
                                 float x3, float y3, int32_t is_static) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    if (!s->prm.simulate) return NATRIX_OK;
    ShapeOp op{SHAPE_TRIANGLE, is_static ? 1 : 0, {x1, y1, x2, y2, x3, y3}};
    s->sq.push_back(op);
    return NATRIX_OK;
}

int natrix_add_splats(natrix_sim* s, natrix_density* d, const float* splats, int32_t n) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    if (n < 0 || (n > 0 && !splats)) return fail(NATRIX_EINVAL, "bad splat list");
    if (d && d->fluid != s) return fail(NATRIX_EINVAL, "density grid belongs to another simulator");
    for (int i = 0; i < n; ++i)
        if (!(splats[(size_t)i * NATRIX_SPLAT_FLOATS + 2] > 0.0f))
            return fail(NATRIX_EINVAL, "splat %d: radius must be > 0", i);
    if (!s->prm.simulate) return NATRIX_OK;
    for (int i = 0; i < n; ++i) {
        const float* r = splats + (size_t)i * NATRIX_SPLAT_FLOATS;
        s->fq.push_back(ForceOp{FORCE_GAUSS, r[0], r[1], r[2], r[3], r[4], r[5], 0});
        if (d && d->simulate)
            d->fq.push_back(ForceOp{FORCE_GAUSS, r[0], r[1], r[2], r[3], r[4], r[5], 0});
    }
    return NATRIX_OK;
}

int natrix_step(natrix_sim* s, float dt, void* stream) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    if (!s->prm.simulate) return NATRIX_OK;
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    bool border_zeroed = false, clamp_deferred = false;
    int rc = flush_fluid_for_step(s, st, &border_zeroed, &clamp_deferred);
    if (rc) return rc;
    const bool mask_zero = s->mask_reset_pending;
    const StepParams sp = fluid_params(s, dt, mask_zero);

    const Grid g = s->g;
    NX_LAUNCH(s, launch_advect(s->vel[0], s->vel[1], s->mask, g, sp, border_zeroed, st,
                               clamp_deferred));
    int cur = 1;
    if (s->prm.vorticity > 0.0f) {
        NX_LAUNCH(s, launch_vorticity(s->vel[cur], s->vel[3 - cur], s->vort, g, sp, st));
        cur = 3 - cur;
    }
    if (s->prm.viscosity > 0.0f) {
        NX_LAUNCH(s, launch_viscosity(s->vel[cur], s->vel[3 - cur], g, sp, st));
        cur = 3 - cur;
    }
    TileMarks tm{};
    if (s->marks.words > 0) {
        s->marks_cur ^= 1;
        tm = s->marks;
        tm.mark = s->d_marks[s->marks_cur];
        tm.clear = s->d_marks[1 - s->marks_cur];
    }
    NX_LAUNCH(s, launch_divergence(s->vel[cur], s->mask, s->div, s->flags, s->p[0], g, sp, tm, st));
    s->p_cur = 0;
    bool fused = false;
    rc = run_jacobi(s, s->prm.iterations - 1, st, s->vel[cur], s->vel[0], &fused);
    if (rc) return rc;
    if (!fused)
        NX_LAUNCH(s, launch_subtract_gradient(s->vel[cur], s->vel[0], s->p[s->p_cur], s->flags, g,
                                              st));
    // clear obstacles (fluid_simulator.py:267-280), applied lazily
    s->mask_reset_pending = true;
    s->last_step_mask_zero = mask_zero;
    s->stepped = true;
    return NATRIX_OK;
}

int natrix_jacobi(natrix_sim* s, int32_t sweeps, void* stream) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    if (sweeps < 0) return fail(NATRIX_EINVAL, "sweeps must be >= 0");
    DeviceGuard dg(s->device);
    return run_jacobi(s, sweeps, stream_of(s, stream));
}

int natrix_residual(natrix_sim* s, double out[5], void* stream) {
    if (!s || !out) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    // the obstacles the last step's sweeps used
    const StepParams sp = fluid_params(s, 0.0f, s->last_step_mask_zero);
    double* sums = s->d_res + (size_t)s->res_blocks * 5;
    NX_CUDA(launch_residual(s->p[s->p_cur], s->div, s->mask, s->flags, s->g, sp, s->d_res,
                            sums, st));
    s->stats.kernel_launches += 2;
    NX_CUDA(cudaMemcpyAsync(s->h_res, sums, 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
    NX_CUDA(cudaStreamSynchronize(st));
    std::memcpy(out, s->h_res, 5 * sizeof(double));
    return NATRIX_OK;
}

int natrix_residual_regions(natrix_sim* s, const int32_t* labels, int32_t n_labels,
                            double* sums, void* stream) {
    if (!s || !labels || !sums || n_labels < 1) return fail(NATRIX_EINVAL, "bad arguments");
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    NX_CUDA(launch_residual_labels(s->p[s->p_cur], s->div, s->flags, labels, n_labels, s->g, sums,
                                   st));
    s->stats.kernel_launches += 1;
    return NATRIX_OK;
}

int natrix_field(natrix_sim* s, int32_t field, void** dev_ptr, int64_t* pitch) {
    if (!s || !dev_ptr || !pitch) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(s->device);
    cudaStream_t st = s->last_stream;
    int rc = flush_fluid(s, st);
    if (rc) return rc;
    *pitch = s->g.P;
    switch (field) {
        case NATRIX_FIELD_VELOCITY: *dev_ptr = s->vel[0]; break;
        case NATRIX_FIELD_PRESSURE: *dev_ptr = s->p[s->p_cur]; break;
        case NATRIX_FIELD_DIVERGENCE: *dev_ptr = s->div; break;
        case NATRIX_FIELD_VORTICITY: *dev_ptr = s->vort; break;
        case NATRIX_FIELD_OBSTACLES:
            rc = materialise_mask(s, st);
            if (rc) return rc;
            s->mask_dirty_all = true;  // the caller may write through the view
            *dev_ptr = s->mask;
            break;
        default: return fail(NATRIX_EINVAL, "unknown field id %d", field);
    }
    return NATRIX_OK;
}

int natrix_upload(natrix_sim* s, int32_t field, const void* host, void* stream) {
    if (!s || !host) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    int rc = flush_fluid(s, st);
    if (rc) return rc;
    if (field == NATRIX_FIELD_OBSTACLES) {
        s->mask_reset_pending = false;
        s->mask_dirty_all = true;
    }
    return field_copy(s, field, nullptr, host, true, st);
}

int natrix_download(natrix_sim* s, int32_t field, void* host, void* stream) {
    if (!s || !host) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    int rc = flush_fluid(s, st);
    if (rc) return rc;
    if (field == NATRIX_FIELD_OBSTACLES) {
        rc = materialise_mask(s, st);
        if (rc) return rc;
    }
    return field_copy(s, field, host, nullptr, false, st);
}

int natrix_sync(natrix_sim* s, void* stream) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    NX_CUDA(cudaStreamSynchronize(st));
    int status = 0;
    NX_CUDA(cudaMemcpy(&status, s->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (status) {
        NX_CUDA(cudaMemset(s->d_status, 0, sizeof(int)));
        if (s->d_chain)  // a sweep launch leaves its counters zeroed; make sure of it
            NX_CUDA(cudaMemset(s->d_chain, 0, (size_t)s->chain_words * 4));
        return fail(NATRIX_EDEVICE, "a kernel reported status 0x%x (bounded wait ran out)",
                    status);
    }
    return NATRIX_OK;
}

int natrix_inject_status(natrix_sim* s, int32_t status, void* stream) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    // from pageable memory: the call returns once the value is staged
    const int v = status;
    NX_CUDA(cudaMemcpyAsync(s->d_status, &v, sizeof(int), cudaMemcpyHostToDevice, st));
    return NATRIX_OK;
}

int natrix_set_timing(natrix_sim* s, int32_t enable) {
    if (!s) return fail(NATRIX_EINVAL, "NULL handle");
    s->timing = enable != 0;
    return NATRIX_OK;
}

int natrix_get_stats(natrix_sim* s, natrix_stats* out, int32_t reset) {
    if (!s || !out) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(s->device);
    for (size_t i = 0; i < s->timed.size(); ++i) {
        NX_CUDA(cudaEventSynchronize(s->timed[i].second));
        float ms = 0.0f;
        NX_CUDA(cudaEventElapsedTime(&ms, s->timed[i].first, s->timed[i].second));
        s->stats.jacobi_ms += ms;
        s->stats.timed_phases += 1;
        s->stats.timed_launches += s->timed_counts[i].first;
        s->stats.timed_sweeps += s->timed_counts[i].second;
        s->stats.timed_fused += s->timed_fused[i];
    }
    drop_timing_events(s);
    *out = s->stats;
    if (reset) s->stats = natrix_stats{};
    return NATRIX_OK;
}

// ----------------------------------------------------------------- density
int natrix_density_create(natrix_sim* fluid, int32_t width, int32_t height,
                          natrix_density** out) {
    if (!fluid || !out) return fail(NATRIX_EINVAL, "NULL argument");
    *out = nullptr;
    if (width < 1 || height < 1 || width > kMaxSide || height > kMaxSide)
        return fail(width < 1 || height < 1 ? NATRIX_EINVAL : NATRIX_ERANGE,
                    "bad density grid size %dx%d", width, height);
    DeviceGuard dg(fluid->device);
    natrix_density* d = new natrix_density();
    d->fluid = fluid;
    d->g = Grid{width, height, round_up(width, 32)};
    const size_t bytes = (size_t)d->g.P * d->g.H * 4;
    cudaError_t e = cudaMalloc(&d->rho[0], bytes);
    if (e == cudaSuccess) e = cudaMemset(d->rho[0], 0, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&d->rho[1], bytes);
    if (e == cudaSuccess) e = cudaMemset(d->rho[1], 0, bytes);
    if (e != cudaSuccess) {
        natrix_density_destroy(d);
        return fail(NATRIX_ENOMEM, "allocating a %dx%d density grid: %s", width, height,
                    cudaGetErrorString(e));
    }
    *out = d;
    return NATRIX_OK;
}

int natrix_density_destroy(natrix_density* d) {
    if (!d) return NATRIX_OK;
    cudaDeviceSynchronize();
    cudaFree(d->rho[0]);
    cudaFree(d->rho[1]);
    delete d;
    return NATRIX_OK;
}

int natrix_density_set_params(natrix_density* d, float speed, float dissipation,
                              int32_t simulate) {
    if (!d) return fail(NATRIX_EINVAL, "NULL handle");
    // demo/smooth_particles_area.py:48-68
    if (!(speed > 0.0f) || !(dissipation > 0.0f))
        return fail(NATRIX_EINVAL, "speed and dissipation must be > 0");
    d->speed = speed;
    d->dissipation = dissipation;
    d->simulate = simulate ? 1 : 0;
    return NATRIX_OK;
}

int natrix_density_add(natrix_density* d, float px, float py, float radius, float strength) {
    if (!d) return fail(NATRIX_EINVAL, "NULL handle");
    if (!d->simulate) return NATRIX_OK;
    // demo/smooth_particles_area.py:80-81 dispatches ceil(W/16) groups in y too
    const int rows = std::min(d->g.H, 16 * ((d->g.W + 15) / 16));
    d->fq.push_back(ForceOp{FORCE_CONE_DENSITY, px, py, radius, 0.0f, 0.0f, strength, rows});
    return NATRIX_OK;
}

int natrix_density_step(natrix_density* d, float dt, void* stream) {
    if (!d) return fail(NATRIX_EINVAL, "NULL handle");
    if (!d->simulate) return NATRIX_OK;
    natrix_sim* s = d->fluid;
    DeviceGuard dg(s->device);
    cudaStream_t st = stream_of(s, stream);
    int rc = flush_fluid(s, st);
    if (rc) return rc;
    rc = flush_density(d, st);
    if (rc) return rc;
    StepParams sp = fluid_params(s, dt, s->mask_reset_pending);
    sp.d_speed = d->speed;
    sp.d_dissipation = d->dissipation;
    NX_LAUNCH(s, launch_density_advect(d->rho[d->cur], d->rho[1 - d->cur], d->g, s->vel[0], s->mask,
                                  s->g, sp, st));
    d->cur ^= 1;
    return NATRIX_OK;
}

int natrix_density_field(natrix_density* d, void** dev_ptr, int64_t* pitch) {
    if (!d || !dev_ptr || !pitch) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(d->fluid->device);
    int rc = flush_density(d, d->fluid->last_stream);
    if (rc) return rc;
    *dev_ptr = d->rho[d->cur];
    *pitch = d->g.P;
    return NATRIX_OK;
}

int natrix_density_upload(natrix_density* d, const float* host, void* stream) {
    if (!d || !host) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(d->fluid->device);
    cudaStream_t st = stream_of(d->fluid, stream);
    int rc = flush_density(d, st);
    if (rc) return rc;
    NX_CUDA(cudaMemcpy2DAsync(d->rho[d->cur], (size_t)d->g.P * 4, host, (size_t)d->g.W * 4,
                              (size_t)d->g.W * 4, d->g.H, cudaMemcpyHostToDevice, st));
    return NATRIX_OK;
}

int natrix_density_download(natrix_density* d, float* host, void* stream) {
    if (!d || !host) return fail(NATRIX_EINVAL, "NULL argument");
    DeviceGuard dg(d->fluid->device);
    cudaStream_t st = stream_of(d->fluid, stream);
    int rc = flush_density(d, st);
    if (rc) return rc;
    NX_CUDA(cudaMemcpy2DAsync(host, (size_t)d->g.W * 4, d->rho[d->cur], (size_t)d->g.P * 4,
                              (size_t)d->g.W * 4, d->g.H, cudaMemcpyDeviceToHost, st));
    return NATRIX_OK;
}

}  // extern "C"
