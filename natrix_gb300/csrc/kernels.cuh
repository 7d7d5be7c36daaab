// Kernel launchers shared between the solver translation units and the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace natrix {

// Per-step scalars.  The single-grid path passes them by value in each
// launch's parameter block; the batch path keeps one block per simulation in
// device memory, so its captured CUDA graph replays with new values.
struct StepParams {
    float dt;
    float speed;
    float dissipation;
    float vorticity;
    float alpha;  // 1/nu           (natrix/core/fluid_simulator.py:327-336)
    float rbeta;  // 1/(4 + alpha)
    int has_borders;
    int mask_zero;  // the obstacle mask holds no obstacle (cleared, not written)
    int n_force;    // forcing ops in this block
    int n_shapes;   // obstacle shapes in this block
    float d_speed;  // density grid (SmoothParticlesArea) speed / dissipation
    float d_dissipation;
};

// Forcing operation kinds, applied in queue order per cell.
enum ForceKind : int {
    FORCE_CONE_VELOCITY = 0,  // shader.AddVelocity.comp (+ clamp of every cell)
    FORCE_GAUSS = 1,          // Gaussian splat on velocity and density
    FORCE_CONE_DENSITY = 2    // demo/shaders/shader.AddParticle.comp
};

struct ForceOp {
    int kind;
    float px, py, r, vx, vy, s;
    int rows;  // FORCE_CONE_DENSITY: rows the reference's dispatch reaches
};

enum ShapeKind : int { SHAPE_CIRCLE = 0, SHAPE_TRIANGLE = 1 };

struct ShapeOp {
    int kind;
    int is_static;
    float a[6];  // circle: px, py, r; triangle: x1, y1, x2, y2, x3, y3
};

// Maximum ops one forcing / obstacle launch stages in shared memory; the
// host splits longer queues into several launches (same result: each cell
// applies the ops in order).
constexpr int kMaxOpsPerLaunch = 256;

// An op list passed by value as a kernel parameter (at most CAP ops).
template <typename Op, int CAP>
struct OpBlock {
    int n;
    Op op[CAP];
};

// Tiles of the persistent register-tiled sweep whose region holds a cell next
// to an obstacle (one bit per tile, row-major).  Such tiles take the per-cell
// select path and cost up to ~1.7x a plain tile; the divergence kernel marks
// them and the sweep launch deals them to CTAs paired with plain tiles.  The
// marks only steer scheduling: every order computes the same values.
constexpr int kMaxBalancedTiles = 1024;  // one 32-bit word per lane of one warp
struct TileMarks {
    uint32_t* mark;   // bits of this step, zero on entry (null: no marking)
    uint32_t* clear;  // bits of the previous step, zeroed for the next one
    int words;
    int tx, ty, rx, ry, hxp, halo, tiles_x, tiles_y;
};

// Record `msg` as the calling thread's natrix_last_error() and return `code`.
int set_last_error(int code, const char* msg);

// What other translation units need of a simulator handle: its velocity
// state buffer and geometry after every queued op has been applied.
struct SimView {
    const float2* vel;
    Grid g;
    float speed;
    int device;
};

}  // namespace natrix

struct natrix_sim;

namespace natrix {

// Apply the handle's queued ops on `st` and describe its velocity field.
int sim_prepare_read(natrix_sim* sim, cudaStream_t st, SimView* out);
// Describe the handle without launching anything.
void sim_describe(const natrix_sim* sim, SimView* out);
// Make `sim`'s device current for the lifetime of the guard.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev);
    ~DeviceGuard();
};
// Count `n` kernel launches in the handle's statistics.
void sim_count_launches(natrix_sim* sim, int n);

// ---- per-cell kernels (solver_kernels.cu) --------------------------------
// `ops` is host memory (n <= kMaxOpsPerLaunch), copied into the launch.
cudaError_t launch_obstacles(uint8_t* mask, Grid g, const ShapeOp* ops, int n, int fresh,
                             cudaStream_t st);
// Obstacle rasters and density forcing work on blocks of kRasterBlock^2 cells
// (row-major block ids); a launch over listed blocks takes at most
// kMaxRasterBlocks of them.
constexpr int kRasterBlock = 32;
constexpr int kMaxRasterBlocks = 2048;
// Mark in hit[] (zeroed by the caller, one byte per block) every block a
// circle of ops[0..n) can mark (bounding box, two cells of margin); false if
// a shape cannot be bounded (a triangle: never culled).
bool shape_blocks(const ShapeOp* ops, int n, Grid g, uint8_t* hit);
// The raster of launch_obstacles restricted to blocks ids[0..n_ids); the
// caller guarantees the mask is already right (zero when `fresh`) elsewhere.
cudaError_t launch_obstacles_blocks(uint8_t* mask, Grid g, const ShapeOp* ops, int n, int fresh,
                                    const uint16_t* ids, int n_ids, cudaStream_t st);
// zero_border: also write the velocity grid's border cells as zero after the
// ops (takes effect when the list holds a velocity op).
cudaError_t launch_forcing(float2* vel, Grid gv, float* rho, Grid gd, const ForceOp* ops,
                           int n, int zero_border, cudaStream_t st);
// Velocity ops over the blocks their footprints reach plus (zero_border)
// the blocks on the grid's edge, which get their border cells zeroed.  The
// reference's first velocity op clamps every cell of the grid; outside the
// listed blocks that clamp is left to the advection's reads (clamp_on_read),
// which is exact because no op changes a cell there and clamping is
// idempotent.  Returns false, launching nothing, when the list is unbounded
// (too many blocks) or holds no velocity op; the caller then runs
// launch_forcing.  Only for a step's own flush, whose next launch is the
// advection: nothing else may read the velocity in between.
bool launch_forcing_sparse(float2* vel, Grid gv, const ForceOp* ops, int n, int zero_border,
                           cudaStream_t st, cudaError_t* err);
// border_zeroed: vin's border cells already hold zero (no test on read).
// clamp_on_read: clamp every velocity read to [-1, 1] (after
// launch_forcing_sparse; needs border_zeroed or no borders).
cudaError_t launch_advect(const float2* vin, float2* vout, const uint8_t* mask, Grid g,
                          const StepParams& sp, bool border_zeroed, cudaStream_t st,
                          bool clamp_on_read = false);
// calc + apply in one pass (same results); writes the curl to w
cudaError_t launch_vorticity(const float2* vin, float2* vout, float* w, Grid g,
                             const StepParams& sp, cudaStream_t st);
cudaError_t launch_viscosity(const float2* vin, float2* vout, Grid g, const StepParams& sp,
                             cudaStream_t st);
// `marks` (may have a null `mark`) receives the tiles with obstacle rows.
cudaError_t launch_divergence(const float2* v, const uint8_t* mask, float* div,
                              uint8_t* flags, float* p1, Grid g, const StepParams& sp,
                              const TileMarks& marks, cudaStream_t st);
cudaError_t launch_subtract_gradient(const float2* vin, float2* vout, const float* p,
                                     const uint8_t* flags, Grid g, cudaStream_t st);
cudaError_t launch_density_advect(const float* rin, float* rout, Grid gd, const float2* v,
                                  const uint8_t* mask, Grid gv, const StepParams& sp,
                                  cudaStream_t st);
// Residual sums {n, sum r, sum r^2, sum b, sum b^2} into out[5] (device),
// using `partials` (device, >= residual_partials(g) * 5 doubles).
int residual_partials(Grid g);
cudaError_t launch_residual(const float* p, const float* div, const uint8_t* mask,
                            const uint8_t* flags, Grid g, const StepParams& sp,
                            double* partials, double* out, cudaStream_t st);

// Per-region residual sums: labels dense W*H (fluid region id, < 0 for
// obstacles), sums n_labels x 5 doubles (zeroed first).
cudaError_t launch_residual_labels(const float* p, const float* div, const uint8_t* flags,
                                   const int* labels, int n_labels, Grid g, double* sums,
                                   cudaStream_t st);

// ---- U-Net weight gradient on the tensor cores (unet_wgrad.cu) ----
// cin = c0 + c1 <= 128, cout a multiple of 16 up to 128, channels multiples of 8.
int wgrad_tc(const uint16_t* dz, int cout, const uint16_t* x0, int c0, const uint16_t* x1, int c1,
             int B, int H, int W, float* dw, float* db, cudaStream_t st);

// ---- Jacobi (jacobi_tma.cu) ------------------------------------------------
// Jacobi tile kernels: shared-memory sweeps on 64x32 tiles, or register tiled
// with 112x112 / 112x128 output tiles.
enum JacobiConfig : int {
    JACOBI_TB = 0,
    JACOBI_RT_A = 1,
    JACOBI_RT_B = 2,
    JACOBI_RT_C = 3,
    JACOBI_RT_D = 4
};

// Tensor maps of one grid for the sweep kernels, encoded for one
// configuration's boxes.  Kernels read them from device memory (64-byte
// aligned: cudaMalloc'd).
struct JacobiMaps {
    CUtensorMap p[2];  // pressure ping-pong buffers as sources
    CUtensorMap div;
    CUtensorMap flags;
    int config;
};

// One simulation of a batch, as the batched sweep kernels see it.
struct JacobiBatchSim {
    JacobiMaps maps;
    float* p[2];
    Grid g;
};

// One tile of one batched launch.
struct JacobiBatchItem {
    int sim, src, sweeps, tile_x, tile_y;
};

// Largest sweep count one launch fuses (the tile halo).
int jacobi_max_sweeps_per_launch();
// Configuration chosen for a single grid (tile shape against SM count).
int jacobi_config(Grid g);
// Output tile of a configuration.
void jacobi_tile(int config, int* tx, int* ty);

// Tile geometry of a register-tiled configuration for grid g (false for the
// shared-memory configuration or more than kMaxBalancedTiles tiles).
bool jacobi_tile_marks(int config, Grid g, TileMarks* out);
// Encode the tensor maps of the buffers for a configuration (false + message on error).
bool jacobi_encode_maps_for(JacobiMaps* maps, int config, float* p0, float* p1, float* div,
                            uint8_t* flags, Grid g, const char** err);
// `sweeps` (1..max) Jacobi sweeps of one grid from pbuf[src] into pbuf[1 - src];
// `d_maps` is the device copy of the grid's maps.
// `slow` (device, may be null) holds the tile marks of the current step.
// static_ready: the previous launch on `st` is a sweep launch of the same
// grid (divergence, flags and marks are final before it starts).
// vin / vout (may be null): also subtract the pressure gradient, vout = vin -
// grad p with the result's pressure (register-tiled configurations, sweeps
// below the per-launch maximum).
cudaError_t launch_jacobi(const JacobiMaps* d_maps, int config, float* const pbuf[2], int src,
                          Grid g, int sweeps, const uint32_t* slow, int static_ready,
                          const float2* vin, float2* vout, int* status, cudaStream_t st);
// A step's whole sweep phase in one persistent launch (register-tiled
// configurations): `sweeps` sweeps from pbuf[src] in chunks of the tile halo,
// the last chunk's result in pbuf[(src + chunks) & 1]; vin / vout as for
// launch_jacobi, fused into the last chunk when it has fewer sweeps than the
// halo (*fused says whether it was).  `sync` (device, jacobi_chain_sync_words
// words, zeroed once) holds the counters the launch's CTAs wait on; the
// launch leaves them zeroed, so its parameters are the same every step (a
// captured graph replays it).
// jacobi_chain_sync_words is 0 where the chain does not pay (fewer tiles than
// SMs) or cannot run (the shared-memory configuration).
int jacobi_chain_sync_words(int config, Grid g);
cudaError_t launch_jacobi_chain(const JacobiMaps* d_maps, int config, float* const pbuf[2],
                                int src, Grid g, int sweeps, const uint32_t* slow,
                                const float2* vin, float2* vout, unsigned* sync, bool* fused,
                                int* status, cudaStream_t st);
// One batched launch: every item is one tile of one simulation (device arrays).
cudaError_t launch_jacobi_batch(int config, const JacobiBatchItem* items, int n_items,
                                const JacobiBatchSim* sims, int* status, cudaStream_t st);

}  // namespace natrix
