/* CPU oracle for the per-step fluid solver — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's compute shaders
 * (the twelve natrix/core/shaders/originals/shader.*.comp kernels,
 * demo/shaders/shader.AddParticle.comp, demo/shaders/shader.AdvectParticle.comp), plus the workload's additions
 * that have no reference counterpart (Gaussian splat forcing, the pressure
 * residual, Lagrangian particles).  Each kernel is instantiated in float
 * (*_f32: the same IEEE operation sequence as the shader text) and double
 * (*_f64: the ground truth the tolerances are measured against).
 *
 * Parity pin: the float instantiation is compared bit-for-bit with the
 * reference's own shader sources compiled as C++ (oracle/ref_kernels.cpp,
 * built by oracle/build_ref.sh) and with the golden vectors in tests/golden/.
 * What that pin cannot cover is the GPU driver's arithmetic for the GLSL
 * built-ins (mix, inversesqrt), which the reference leaves to bgfx's shader
 * compiler and the vendor driver; the choices made here are stated in
 * oracle_impl.h.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library.  Compiled with -O2 -fopenmp -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* exp for the float instantiation of the Gaussian splat weight.  Cody-Waite
 * range reduction x = k*ln2 + r (ln2 split as 0.693359375 - 2.12194440e-4 so
 * k*C1 is exact), then exp(r) by its degree-7 Taylor polynomial in Horner
 * form, then an exact scaling by 2^k.  Every step rounds separately; the CUDA
 * kernels evaluate the same sequence, so both sides produce the same bits.
 * Accuracy against libm expf is checked by the CPU tests (a few ulp on the
 * splat's argument range [-9, 0]). */
float nx_expf(float x) {
    if (x < -87.0f) x = -87.0f;
    if (x > 88.0f) x = 88.0f;
    float kf = floorf(x * 1.44269502f + 0.5f);
    int k = (int)kf;
    float r = x - kf * 0.693359375f;
    r = r - kf * -2.12194440e-4f;
    float p = 0.000198412701f;
    p = 0.00138888892f + r * p;
    p = 0.00833333377f + r * p;
    p = 0.0416666679f + r * p;
    p = 0.166666672f + r * p;
    p = 0.5f + r * p;
    p = 1.0f + r * p;
    p = 1.0f + r * p;
    return ldexpf(p, k);
}

#define REAL float
#define SUFFIX _f32
#define SQRT sqrtf
#define CEIL ceilf
#define FLOOR floorf
#define FABS fabsf
#define EXP nx_expf
#include "oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef SQRT
#undef CEIL
#undef FLOOR
#undef FABS
#undef EXP

#define REAL double
#define SUFFIX _f64
#define SQRT sqrt
#define CEIL ceil
#define FLOOR floor
#define FABS fabs
#define EXP exp
#include "oracle_impl.h"

/* Particle -> cell index and 3x3 tent weights (no reference counterpart).
 * cell c = floor(p + 0.5) per axis (nearest cell centre), f = p - c in
 * [-0.5, 0.5]; the hat of half-width 1.5 gives a_{-1} = 0.5 - f,
 * a_0 = 1.5 - |f|, a_{+1} = 0.5 + f, normalised by their sum 2.5 - |f|.
 * Targets outside the grid are clamped onto the edge cell (mass is kept). */
void orc_particle_cells(const float* pos, long n, int32_t* cells) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n; ++k) {
        cells[2 * k] = (int32_t)floorf(pos[2 * k] + 0.5f);
        cells[2 * k + 1] = (int32_t)floorf(pos[2 * k + 1] + 0.5f);
    }
}

static void tent3(float p, int c, float w[3]) {
    float f = p - (float)c;
    float af = fabsf(f);
    float s = 2.5f - af;
    w[0] = (0.5f - f) / s;
    w[1] = (1.5f - af) / s;
    w[2] = (0.5f + f) / s;
}

/* Splat every particle with unit mass into rho (W*H, accumulated in double,
 * serial so the sum is deterministic). */
void orc_particles_splat(const float* pos, long n, double* rho, int W, int H) {
    for (long k = 0; k < n; ++k) {
        float px = pos[2 * k], py = pos[2 * k + 1];
        int cx = (int)floorf(px + 0.5f), cy = (int)floorf(py + 0.5f);
        float wx[3], wy[3];
        tent3(px, cx, wx);
        tent3(py, cy, wy);
        for (int j = 0; j < 3; ++j) {
            int yy = cy + j - 1;
            yy = yy < 0 ? 0 : (yy > H - 1 ? H - 1 : yy);
            for (int i = 0; i < 3; ++i) {
                int xx = cx + i - 1;
                xx = xx < 0 ? 0 : (xx > W - 1 ? W - 1 : xx);
                rho[(long)yy * W + xx] += (double)(wx[i] * wy[j]);
            }
        }
    }
}

int orc_num_threads(void) {
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    extern void omp_set_num_threads(int);
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
