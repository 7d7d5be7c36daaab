/* natrix_gb300 — C ABI of the GB300 (sm_103a) fluid solver.
 *
 * Drop-in for the per-step solver behind natrix.core's FluidSimulator
 * (natrix/core/fluid_simulator.py) and the demo's SmoothParticlesArea
 * (demo/smooth_particles_area.py).  Each entry point names the reference
 * member it replaces.
 *
 * Conventions
 *  - Every entry point returns 0 on success or a negative NATRIX_E* code;
 *    natrix_last_error() gives the message of the calling thread's last error.
 *  - The library owns the device memory of each handle (cudaMalloc at
 *    creation, cudaFree at destroy), on the device current at creation.
 *  - `stream` arguments are cudaStream_t values passed as void*; NULL is the
 *    legacy default stream.  Work on one handle must be issued on one stream
 *    (or externally ordered); separate handles are independent.
 *  - Not thread-safe per handle.
 *  - Mutating calls (add_*, step) are no-ops while the `simulate` parameter
 *    is 0, as in the reference.  add_* calls are queued on the host and
 *    applied by one fused kernel before the next step or field access.
 *  - Device fields are row-major with a row pitch in elements
 *    (natrix_field); pitch >= width and rows are 128-byte aligned.
 */
#ifndef NATRIX_GB300_NATRIX_H
#define NATRIX_GB300_NATRIX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NATRIX_OK 0
#define NATRIX_EINVAL -1  /* bad argument (the reference raises ValueError) */
#define NATRIX_ECUDA -2   /* a CUDA runtime call failed */
#define NATRIX_ENOMEM -3  /* device or host allocation failed */
#define NATRIX_EDEVICE -4 /* a kernel reported an error status (bounded wait) */
#define NATRIX_ERANGE -5  /* size beyond a documented maximum */

typedef struct natrix_sim natrix_sim;
typedef struct natrix_density natrix_density;

/* Simulator parameters; defaults as natrix/core/fluid_simulator.py:28-35. */
typedef struct natrix_params {
    float speed;       /* > 0, default 500   (FluidSimulator.speed, :58-66)       */
    int32_t iterations; /* > 0, default 50   (FluidSimulator.iterations, :68-76)  */
    float dissipation; /* > 0, default 1.0   (FluidSimulator.dissipation, :78-86) */
    float vorticity;   /* >= 0, default 0    (FluidSimulator.vorticity, :88-96)   */
    float viscosity;   /* >= 0, default 0.1  (FluidSimulator.viscosity, :98-111)  */
    int32_t has_borders; /* default 1        (FluidSimulator.has_borders, :34)    */
    int32_t simulate;  /* default 1          (FluidSimulator.simulate, :35)       */
    int32_t sweeps_per_launch; /* Jacobi sweeps fused per launch (temporal
                                  blocking); 0 = library default */
} natrix_params;

/* Fields of a simulator (natrix_field / natrix_upload / natrix_download). */
enum natrix_field_id {
    NATRIX_FIELD_VELOCITY = 0,   /* float2 [H][pitch]; FluidSimulator.get_velocity_buffer, :113-114 */
    NATRIX_FIELD_PRESSURE = 1,   /* float  [H][pitch]; pressure after the last step's sweeps */
    NATRIX_FIELD_DIVERGENCE = 2, /* float  [H][pitch] */
    NATRIX_FIELD_VORTICITY = 3,  /* float  [H][pitch] */
    NATRIX_FIELD_OBSTACLES = 4,  /* uint8  [H][pitch]; bit0 = obstacle (x), bit1 = static triangle (y) */
    NATRIX_FIELD_DENSITY = 5     /* float  [H][pitch]; batches only (density grid of each simulation) */
};

/* Number of floats per splat record passed to natrix_add_splats. */
#define NATRIX_SPLAT_FLOATS 6

/* Create a width x height simulator (FluidSimulator.__init__,
 * natrix/core/fluid_simulator.py:37-48; the bgfx vertex layout has no
 * counterpart).  Fields start at zero, parameters at their defaults. */
int natrix_create(int32_t width, int32_t height, natrix_sim** out);

/* Free every device buffer of the handle (FluidSimulator.destroy, :476-515). */
int natrix_destroy(natrix_sim* sim);

/* Set / get all parameters.  Validation follows the property setters of
 * natrix/core/fluid_simulator.py:58-111: speed, iterations and dissipation
 * must be > 0, vorticity and viscosity >= 0, else NATRIX_EINVAL. */
int natrix_set_params(natrix_sim* sim, const natrix_params* params);
int natrix_get_params(const natrix_sim* sim, natrix_params* params);

/* Cone velocity splat at a normalised position with radius in cells, then
 * the clamp of every cell to [-1, 1] (FluidSimulator.add_velocity, :116-131;
 * shader.AddVelocity.comp). */
int natrix_add_velocity(natrix_sim* sim, float px, float py, float vx, float vy, float radius);

/* Obstacle disc (FluidSimulator.add_circle_obstacle, :135-153;
 * shader.AddCircleObstacle.comp). */
int natrix_add_circle_obstacle(natrix_sim* sim, float px, float py, float radius,
                               int32_t is_static);

/* Obstacle triangle in normalised coordinates (FluidSimulator.add_triangle_obstacle,
 * :156-172; shader.AddTriangleObstacle.comp). */
int natrix_add_triangle_obstacle(natrix_sim* sim, float x1, float y1, float x2, float y2,
                                 float x3, float y3, int32_t is_static);

/* Gaussian splat forcing of velocity and, when `density` is not NULL, of
 * that density grid: `n` host records of NATRIX_SPLAT_FLOATS floats
 * {px, py, radius_cells, vx, vy, density}.  No reference counterpart: it is
 * the forcing of the benchmark workloads (weight exp(-d^2/r^2) inside 3r,
 * velocity clamped to [-1, 1] after each splat, density to [0, 255]). */
int natrix_add_splats(natrix_sim* sim, natrix_density* density, const float* splats,
                      int32_t n);

/* Advance one step (FluidSimulator.update, :174-280): boundaries, advection,
 * vorticity confinement, viscosity, divergence, `iterations` Jacobi sweeps
 * from zero, gradient subtraction, obstacle reset. */
int natrix_step(natrix_sim* sim, float dt, void* stream);

/* Device pointer and row pitch (elements) of a field's current buffer.  The
 * pointer can change after natrix_step; query it again after each step. */
int natrix_field(natrix_sim* sim, int32_t field, void** dev_ptr, int64_t* pitch_elems);

/* Copy a field between a dense host array (H*W elements, rows of W) and the
 * device (stream-ordered; the host buffer should be pinned for async copies,
 * the call returns after enqueueing). */
int natrix_upload(natrix_sim* sim, int32_t field, const void* host, void* stream);
int natrix_download(natrix_sim* sim, int32_t field, void* host, void* stream);

/* Residual of the pressure system the sweeps iterate, over fluid cells:
 * out = {n, sum r, sum r^2, sum b, sum b^2} with r = b - (sum p_nbr - 4 p)
 * (same neighbour rule as shader.Poisson.comp).  Synchronises `stream`.
 * No reference counterpart. */
int natrix_residual(natrix_sim* sim, double out[5], void* stream);

/* The residual sums of natrix_residual per connected fluid region: `labels`
 * (device, W*H int32, row-major without padding) gives each fluid cell its
 * region in [0, n_labels) and obstacle cells a negative value; `sums`
 * (device, n_labels x 5 doubles) receives {n, sum r, sum r^2, sum b, sum b^2}
 * per region.  The pressure system is pure Neumann on every region, so the
 * residual is defined up to each region's mean.  Stream-ordered, no sync.
 * No reference counterpart. */
int natrix_residual_regions(natrix_sim* sim, const int32_t* labels, int32_t n_labels,
                            double* sums, void* stream);

/* Run `sweeps` more Jacobi sweeps on the current pressure (no reset), with
 * the divergence and obstacles of the last step.  No reference counterpart
 * (used for residual-driven solves and warm starts). */
int natrix_jacobi(natrix_sim* sim, int32_t sweeps, void* stream);

/* Wait for the handle's work and return NATRIX_EDEVICE if a kernel recorded
 * an error status (bounded waits that ran out).  Clears the status. */
int natrix_sync(natrix_sim* sim, void* stream);

/* Fault injection on the host side, for tests of the error path: write
 * `status` into the handle's device status word on `stream`, as a kernel
 * whose bounded wait ran out does (status bit 1: a sweep's tile wait).  The
 * next natrix_sync returns NATRIX_EDEVICE and clears the word.  Nothing stalls
 * or faults on the GPU.  No reference counterpart. */
int natrix_inject_status(natrix_sim* sim, int32_t status, void* stream);

/* --- density grid: SmoothParticlesArea (demo/smooth_particles_area.py) --- */

/* Density grid of its own size, advected by `fluid`'s velocity
 * (SmoothParticlesArea.__init__, :28-46). */
int natrix_density_create(natrix_sim* fluid, int32_t width, int32_t height,
                          natrix_density** out);
int natrix_density_destroy(natrix_density* d);

/* speed > 0 and dissipation > 0 (SmoothParticlesArea.speed / .dissipation,
 * :48-68); simulate as the reference's flag (:26). */
int natrix_density_set_params(natrix_density* d, float speed, float dissipation,
                              int32_t simulate);

/* Cone density splat, clamped to [0, 255] inside the radius
 * (SmoothParticlesArea.add_particles, :70-83; shader.AddParticle.comp).
 * Rows the reference's dispatch does not reach (y >= 16*ceil(W/16)) are
 * left unchanged. */
int natrix_density_add(natrix_density* d, float px, float py, float radius, float strength);

/* Advect the density by the fluid's current velocity
 * (SmoothParticlesArea.update, :85-104; shader.AdvectParticle.comp). */
int natrix_density_step(natrix_density* d, float dt, void* stream);

int natrix_density_field(natrix_density* d, void** dev_ptr, int64_t* pitch_elems);
int natrix_density_upload(natrix_density* d, const float* host, void* stream);
int natrix_density_download(natrix_density* d, float* host, void* stream);

/* --- Lagrangian particles (no reference counterpart) ---------------------
 * Point particles moved through a simulator's velocity field by RK2
 * (midpoint) with the bilinear sampler of shader.AdvectVelocity.comp:38-48
 * and displacement v * dt * speed (the simulator's speed), clamped to the
 * grid, then splatted with unit mass into a density grid of the simulator's
 * size by a 3x3 normalised linear hat around the nearest cell centre. */
typedef struct natrix_particles natrix_particles;

/* `n` particles bound to `fluid` (positions in cells, x then y). */
int natrix_particles_create(natrix_sim* fluid, int64_t n, natrix_particles** out);
int natrix_particles_destroy(natrix_particles* p);
/* Copy n float2 positions from / to host memory (stream-ordered). */
int natrix_particles_upload(natrix_particles* p, const float* host_xy, void* stream);
int natrix_particles_download(natrix_particles* p, float* host_xy, void* stream);
/* One step: advect every particle; if `splat`, clear the density grid and
 * deposit every particle into it. */
int natrix_particles_step(natrix_particles* p, float dt, int32_t splat, void* stream);
/* Integer cell (floor(p + 0.5) per axis) of every particle, n int2 to host. */
int natrix_particles_cells(natrix_particles* p, int32_t* host_cells, void* stream);
/* Device pointers of the positions (float2[n]) and the density grid (float,
 * rows of `pitch` elements). */
int natrix_particles_field(natrix_particles* p, void** pos, void** density, int64_t* pitch);

/* --- batches of independent simulations (no reference counterpart) -------
 * n simulations of their own sizes, each a FluidSimulator with a density grid
 * of the same size (SmoothParticlesArea), advanced together: one launch per
 * phase covers every simulation and the whole step is captured once as a
 * CUDA graph and replayed.  Each simulation gives the same result, bit for
 * bit, as a single simulator stepped through the same calls (obstacles are
 * discs; forcing is add_velocity cones and Gaussian splats on velocity and
 * density). */
typedef struct natrix_batch natrix_batch;

int natrix_batch_create(int32_t n, const int32_t* widths, const int32_t* heights,
                        natrix_batch** out);
int natrix_batch_destroy(natrix_batch* b);
/* Parameters of simulation `sim` (-1 = all); validation as natrix_set_params. */
int natrix_batch_set_params(natrix_batch* b, int32_t sim, const natrix_params* p);
int natrix_batch_set_density_params(natrix_batch* b, int32_t sim, float speed,
                                    float dissipation);
/* Jacobi tile configuration (0 = 64x32 shared-memory tiles, 1 = 112x112 and
 * 2 = 112x128 register tiles) and sweeps per launch (1..8) for a size class
 * (0: side <= 128, 1: <= 256, 2: larger). */
int natrix_batch_set_tuning(natrix_batch* b, int32_t size_class, int32_t config,
                            int32_t sweeps_per_launch);
/* Replay a captured CUDA graph per step (default 1) or launch directly (0). */
int natrix_batch_set_graph(natrix_batch* b, int32_t enable);
/* Step the whole batch in one persistent launch (1, the default: resident
 * CTAs claim the step's work items in dependency order, each waiting for its
 * simulation's previous phase) or in one launch per phase (0).  Both give the
 * same values, bit for bit.  The persistent step stages rows of at most 3008
 * cells (wider simulations: NATRIX_ERANGE at the next step; use 0).  No
 * reference counterpart. */
int natrix_batch_set_persistent(natrix_batch* b, int32_t enable);
/* Queued per simulation for the next step (at most 256 ops and 256 shapes
 * per simulation per step, else NATRIX_ERANGE). */
int natrix_batch_add_velocity(natrix_batch* b, int32_t sim, float px, float py, float vx,
                              float vy, float radius);
int natrix_batch_add_splats(natrix_batch* b, int32_t sim, const float* splats, int32_t n);
int natrix_batch_add_circle_obstacle(natrix_batch* b, int32_t sim, float px, float py,
                                     float radius, int32_t is_static);
/* The same for every simulation at once: counts[n] records per simulation,
 * records concatenated in simulation order (splats: NATRIX_SPLAT_FLOATS
 * floats each; circles: px, py, radius). */
int natrix_batch_add_splats_bulk(natrix_batch* b, const int32_t* counts, const float* splats);
int natrix_batch_add_circles_bulk(natrix_batch* b, const int32_t* counts, const float* circles);
/* One step of every simulation (fluid update, then density update). */
int natrix_batch_step(natrix_batch* b, float dt, void* stream);
int natrix_batch_field(natrix_batch* b, int32_t sim, int32_t field, void** dev_ptr,
                       int64_t* pitch_elems);
int natrix_batch_download(natrix_batch* b, int32_t sim, int32_t field, void* host,
                          void* stream);
/* Kernels launched so far and per step. */
int natrix_batch_launches(natrix_batch* b, int64_t* total, int32_t* per_step);
int natrix_batch_sync(natrix_batch* b, void* stream);

/* Counters of one handle (and the density grids attached to it). */
typedef struct natrix_stats {
    int64_t kernel_launches; /* kernels this library launched for the handle */
    int64_t jacobi_launches; /* of which temporally blocked Jacobi launches */
    int64_t jacobi_sweeps;   /* Jacobi sweeps those launches ran */
    int64_t timed_phases;    /* Jacobi phases bracketed by CUDA events */
    int64_t timed_launches;  /* Jacobi launches inside the timed phases */
    int64_t timed_sweeps;    /* sweeps inside the timed phases */
    double jacobi_ms;        /* device time of the timed phases (CUDA events) */
    int64_t timed_fused;     /* timed phases whose last launch also subtracted the gradient */
} natrix_stats;

/* Bracket the Jacobi phase of every following step with CUDA events on the
 * step's stream (enable = 1) or stop (0).  No reference counterpart. */
int natrix_set_timing(natrix_sim* sim, int32_t enable);

/* Read the counters (waits for the timed events); reset = 1 zeroes them. */
int natrix_get_stats(natrix_sim* sim, natrix_stats* out, int32_t reset);

/* ---- headless visualisation (demo/shaders/demo.*) ----
 * No graphics pipeline: each shader becomes a kernel writing a device
 * buffer of RGBA8 pixels (4 bytes, R first).  Device pointers, stream
 * ordered, no sync (the first call on a device also builds a 256-entry colour
 * table and waits for it).
 *
 * natrix_render_density replaces demo.ComputeShader.comp:9-20 (density ->
 * rgba8 texture, `texture`) and demo.FieldFragmentShader.frag:95-99 (the
 * plasma(fbm(c)) colour with alpha c, `colour`) at one pixel per density
 * cell.  `density` has `pitch` floats per row; both outputs have `out_pitch`
 * pixels per row; either output may be NULL.  UNORM8 conversion: 0 for NaN
 * and v <= 0, 255 for v >= 1, else round-half-even(v * 255). */
int natrix_render_density(const float* density, int32_t width, int32_t height, int64_t pitch,
                          uint8_t* texture, uint8_t* colour, int64_t out_pitch, void* stream);

/* Arrow tiles of a win_w x win_h quiver overlay with tiles of `tile` pixels
 * (1 <= tile <= 65536): nx = floor((win_w - 0.5) / tile) + 1, ny alike. */
int natrix_quiver_tiles(int32_t win_w, int32_t win_h, float tile, int32_t* nx, int32_t* ny);

/* demo.QuiverFragmentShader.frag: `arrows` (nx * ny float2, row-major)
 * receives each tile's arrow in window pixels, field(tile centre) * tile *
 * 0.4, with the shader's sampling of the velocity (width x height float2,
 * `pitch` float2 per row); if `overlay` is not NULL it receives the
 * win_w x win_h overlay (white, alpha 1 - clamp(distance to the arrow, 0, 1)),
 * `overlay_pitch` pixels per row, pixel (x, y) sampled at (x + 0.5, y + 0.5). */
int natrix_quiver(const float* velocity, int32_t width, int32_t height, int64_t pitch,
                  int32_t win_w, int32_t win_h, float tile, float* arrows, uint8_t* overlay,
                  int64_t overlay_pitch, void* stream);

/* Largest grid, in cells, that natrix_residual_noalloc accepts (4096 x 4096). */
#define NATRIX_NOALLOC_MAX_CELLS (4096 * 4096)

/* Residual sums of a pressure system, computed without allocating anything.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc (code running inside another framework's memory pool, plugins
 * that must not touch the allocator, hosts with a fixed device budget) and so
 * cannot create a simulator handle, whose natrix_residual uses scratch that
 * natrix_create allocated.  Here the caller passes its own device buffers:
 * pressure `p` and divergence `div` (float, rows of `pitch` elements), an
 * optional obstacle mask (uint8, same pitch in bytes; NULL = no obstacles)
 * and `out_dev`, 5 doubles in device memory that receive
 * {n, sum r, sum r^2, sum b, sum b^2} exactly as natrix_residual defines them.
 * The scratch is a fixed array inside the library, sized for grids of up to
 * NATRIX_NOALLOC_MAX_CELLS cells (larger grids return NATRIX_ERANGE); it
 * stays resident on every GPU that loads the library until the process exits.
 * All calls share that array, so calls whose kernels overlap on the GPU race
 * and may return wrong sums: order them on one stream.  The first call on a
 * device looks up the array's device address (with that device current);
 * make that first call before any stream capture.  That address is kept for
 * the process: do not call this entry point on a device after
 * cudaDeviceReset there.  A pitch above INT_MAX returns NATRIX_ERANGE.
 * Stream-ordered on `stream`; runs on the calling thread's current device. */
int natrix_residual_noalloc(const float* p, const float* div, const uint8_t* mask,
                            int32_t width, int32_t height, int64_t pitch, double* out_dev,
                            void* stream);

/* Message of the calling thread's last error ("" if none). */
const char* natrix_last_error(void);

/* Library version string. */
const char* natrix_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NATRIX_GB300_NATRIX_H */
