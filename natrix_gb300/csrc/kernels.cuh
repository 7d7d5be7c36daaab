// Kernel launchers shared between the solver translation units and the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace natrix {

// Per-step scalars, resident in device memory so a captured CUDA graph can
// replay a step with new values (the host copies a fresh block each step).
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
cudaError_t launch_obstacles(uint8_t* mask, Grid g, const ShapeOp* ops, int n, int fresh,
                             cudaStream_t st);
cudaError_t launch_forcing(float2* vel, Grid gv, float* rho, Grid gd, const ForceOp* ops,
                           int n, cudaStream_t st);
cudaError_t launch_advect(const float2* vin, float2* vout, const uint8_t* mask, Grid g,
                          const StepParams* sp, cudaStream_t st);
cudaError_t launch_calc_vorticity(const float2* v, float* w, Grid g, cudaStream_t st);
cudaError_t launch_apply_vorticity(const float2* vin, float2* vout, const float* w, Grid g,
                                   const StepParams* sp, cudaStream_t st);
cudaError_t launch_viscosity(const float2* vin, float2* vout, Grid g, const StepParams* sp,
                             cudaStream_t st);
cudaError_t launch_divergence(const float2* v, const uint8_t* mask, float* div,
                              uint8_t* flags, float* p1, Grid g, const StepParams* sp,
                              cudaStream_t st);
cudaError_t launch_subtract_gradient(const float2* vin, float2* vout, const float* p,
                                     const uint8_t* flags, Grid g, cudaStream_t st);
cudaError_t launch_density_advect(const float* rin, float* rout, Grid gd, const float2* v,
                                  const uint8_t* mask, Grid gv, const StepParams* sp,
                                  cudaStream_t st);
// Residual sums {n, sum r, sum r^2, sum b, sum b^2} into out[5] (device),
// using `partials` (device, >= residual_partials(g) * 5 doubles).
int residual_partials(Grid g);
cudaError_t launch_residual(const float* p, const float* div, const uint8_t* mask,
                            const uint8_t* flags, Grid g, const StepParams* sp,
                            double* partials, double* out, cudaStream_t st);

// ---- Jacobi (jacobi_tma.cu) ------------------------------------------------
// Tensor maps of one solver grid for the temporally blocked sweep kernel.
struct JacobiMaps {
    CUtensorMap p[2];  // pressure ping-pong buffers as sources
    CUtensorMap div;
    CUtensorMap flags;
    int config;  // kernel configuration the boxes were encoded for
};

// Kernel configuration picked for a grid (0 = shared-memory sweeps,
// 1 / 2 = register-tiled persistent with 112x112 / 112x128 output tiles).
int jacobi_config(Grid g);

// Largest sweep count one launch fuses (the tile halo).
int jacobi_max_sweeps_per_launch();
// Encode the tensor maps for the buffers (returns false + message on error).
bool jacobi_encode_maps(JacobiMaps* maps, float* p0, float* p1, float* div, uint8_t* flags,
                        Grid g, const char** err);
// `sweeps` (1..max) Jacobi sweeps from p[src] into p[1 - src].
cudaError_t launch_jacobi(const JacobiMaps& maps, float* const pbuf[2], int src, Grid g,
                          int sweeps, int* status, cudaStream_t st);

}  // namespace natrix
