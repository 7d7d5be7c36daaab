/* Oracle kernels, instantiated twice by oracle.c: once with REAL=float
 * (suffix _f32) and once with REAL=double (suffix _f64).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a CPU restatement of the reference's
 * per-step fluid solver, written from the shader math.  Only the tests, the
 * smoke check and bench.py's CPU-baseline leg may load it, as the checker;
 * the product never calls it.
 *
 * Layouts (row-major, idx = y*W + x, contiguous rows):
 *   velocity   REAL[H][W][2]          (the reference's vec2 velocity buffer)
 *   scalars    REAL[H][W]             (pressure, divergence, vorticity, density)
 *   obstacles  uint8[H][W]            bit0 = reference obstacle .x > 0 (dynamic)
 *                                     bit1 = reference obstacle .y > 0 (static triangle)
 * obs(c) <=> mask[c] != 0, which is the reference's `o.x > 0 || o.y > 0`.
 *
 * Every binary operation is written in the order the shader writes it, and
 * the file is compiled with -ffp-contract=off, so the float instantiation
 * rounds exactly as the shader text prescribes (mix = a + t*(b - a),
 * inversesqrt = 1/sqrt).  Geometric decisions that switch a cell in or out
 * (obstacle rasterisation, splat cut-offs, particle cells) are taken in float
 * in both instantiations so the float and double trajectories see the same
 * masks; values are computed in REAL.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

/* clamped 4-neighbour indices: natrix/core/shaders/originals/common.sh:9-19 */
static inline void FN(nbrs)(int x, int y, int W, int H, long* L, long* R, long* B, long* T) {
    int xl = x - 1 < 0 ? 0 : x - 1;
    int xr = x + 1 > W - 1 ? W - 1 : x + 1;
    int yb = y - 1 < 0 ? 0 : y - 1;
    int yt = y + 1 > H - 1 ? H - 1 : y + 1;
    *L = (long)y * W + xl;
    *R = (long)y * W + xr;
    *B = (long)yb * W + x;
    *T = (long)yt * W + x;
}

static inline REAL FN(clampr)(REAL v, REAL lo, REAL hi) {
    /* GLSL clamp = min(max(x, lo), hi) */
    REAL m = v > lo ? v : lo;
    return m < hi ? m : hi;
}

static inline REAL FN(mixr)(REAL a, REAL b, REAL t) { return a + t * (b - a); }

/* Bilinear sample of a 2-component field, shader.AdvectVelocity.comp:38-48
 * (also GetVelocity, demo/shaders/shader.AdvectParticle.comp:21-35): corner
 * indices from ceil/floor clamped to the grid, delta NOT clamped. */
static inline void FN(sample2)(const REAL* v, int W, int H, REAL fx, REAL fy, REAL* ox, REAL* oy) {
    REAL bx = (REAL)(W - 1), by = (REAL)(H - 1);
    int trx = (int)FN(clampr)(CEIL(fx), (REAL)0, bx);
    int try_ = (int)FN(clampr)(CEIL(fy), (REAL)0, by);
    int blx = (int)FN(clampr)(FLOOR(fx), (REAL)0, bx);
    int bly = (int)FN(clampr)(FLOOR(fy), (REAL)0, by);
    REAL dx = fx - (REAL)blx;
    REAL dy = fy - (REAL)bly;
    const REAL* lt = v + 2 * ((long)try_ * W + blx);
    const REAL* rt = v + 2 * ((long)try_ * W + trx);
    const REAL* lb = v + 2 * ((long)bly * W + blx);
    const REAL* rb = v + 2 * ((long)bly * W + trx);
    REAL h1x = FN(mixr)(lt[0], rt[0], dx), h1y = FN(mixr)(lt[1], rt[1], dx);
    REAL h2x = FN(mixr)(lb[0], rb[0], dx), h2y = FN(mixr)(lb[1], rb[1], dx);
    *ox = FN(mixr)(h2x, h1x, dy);
    *oy = FN(mixr)(h2y, h1y, dy);
}

/* Same sampler for a scalar field (shader.AdvectParticle.comp:58-69). */
static inline REAL FN(sample1)(const REAL* s, int W, int H, REAL fx, REAL fy) {
    REAL bx = (REAL)(W - 1), by = (REAL)(H - 1);
    int trx = (int)FN(clampr)(CEIL(fx), (REAL)0, bx);
    int try_ = (int)FN(clampr)(CEIL(fy), (REAL)0, by);
    int blx = (int)FN(clampr)(FLOOR(fx), (REAL)0, bx);
    int bly = (int)FN(clampr)(FLOOR(fy), (REAL)0, by);
    REAL dx = fx - (REAL)blx;
    REAL dy = fy - (REAL)bly;
    REAL lt = s[(long)try_ * W + blx], rt = s[(long)try_ * W + trx];
    REAL lb = s[(long)bly * W + blx], rb = s[(long)bly * W + trx];
    REAL h1 = FN(mixr)(lt, rt, dx);
    REAL h2 = FN(mixr)(lb, rb, dx);
    return FN(mixr)(h2, h1, dy);
}

/* shader.InitBoundaries.comp:11-35: zero velocity on the border, in place. */
void FN(orc_init_boundaries)(REAL* v, int W, int H) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            if (x == 0 || x == W - 1 || y == 0 || y == H - 1) {
                long i = (long)y * W + x;
                v[2 * i] = 0;
                v[2 * i + 1] = 0;
            }
}

/* shader.AddVelocity.comp:19-36: cone splat then clamp every cell to [-1,1]. */
void FN(orc_add_velocity)(const REAL* vin, REAL* vout, int W, int H, float px, float py,
                          float vx, float vy, float radius) {
    REAL spx = (REAL)(px * (float)W), spy = (REAL)(py * (float)H);
    REAL r = radius, Vx = vx, Vy = vy;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long i = (long)y * W + x;
            REAL ax = vin[2 * i], ay = vin[2 * i + 1];
            REAL dx = spx - (REAL)x, dy = spy - (REAL)y;
            REAL len = SQRT(dx * dx + dy * dy);
            if (len <= r) {
                ax = ax + Vx * (r - len) / r;
                ay = ay + Vy * (r - len) / r;
            }
            vout[2 * i] = FN(clampr)(ax, (REAL)-1, (REAL)1);
            vout[2 * i + 1] = FN(clampr)(ay, (REAL)-1, (REAL)1);
        }
}

/* shader.AdvectVelocity.comp:19-51 (obstacle -> 0, else backtrace by
 * v*dt*speed, bilinear, *dissipation, clamp to [-1,1]). */
void FN(orc_advect_velocity)(const REAL* vin, REAL* vout, const unsigned char* obs, int W,
                             int H, REAL dt, REAL speed, REAL diss) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long i = (long)y * W + x;
            if (obs[i]) {
                vout[2 * i] = 0;
                vout[2 * i + 1] = 0;
                continue;
            }
            REAL fx = (REAL)x - vin[2 * i] * dt * speed;
            REAL fy = (REAL)y - vin[2 * i + 1] * dt * speed;
            REAL sx, sy;
            FN(sample2)(vin, W, H, fx, fy, &sx, &sy);
            vout[2 * i] = FN(clampr)(sx * diss, (REAL)-1, (REAL)1);
            vout[2 * i + 1] = FN(clampr)(sy * diss, (REAL)-1, (REAL)1);
        }
}

/* shader.CalcVorticity.comp:13-27. */
void FN(orc_calc_vorticity)(const REAL* v, REAL* w, int W, int H) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            w[i] = (REAL)0.5 * ((v[2 * R + 1] - v[2 * L + 1]) - (v[2 * T] - v[2 * B]));
        }
}

/* shader.ApplyVorticity.comp:19-40. */
void FN(orc_apply_vorticity)(const REAL* vin, REAL* vout, const REAL* w, int W, int H,
                             REAL dt, REAL scale) {
    const REAL eps = (REAL)2.4414e-4f;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            REAL wL = w[L], wR = w[R], wB = w[B], wT = w[T], wC = w[i];
            REAL fx = (REAL)0.5 * (FABS(wT) - FABS(wB));
            REAL fy = (REAL)0.5 * (FABS(wR) - FABS(wL));
            REAL d = fx * fx + fy * fy;
            REAL m = eps > d ? eps : d; /* max(EPSILON, dot) */
            REAL rs = (REAL)1 / SQRT(m);
            fx = fx * rs;
            fy = fy * rs;
            REAL s = scale * wC;
            fx = fx * (s * (REAL)1);
            fy = fy * (s * (REAL)-1);
            vout[2 * i] = vin[2 * i] + fx * dt;
            vout[2 * i + 1] = vin[2 * i + 1] + fy * dt;
        }
}

/* shader.Viscosity.comp:17-32 (alpha = 1/nu, rbeta = 1/(4+alpha)). */
void FN(orc_viscosity)(const REAL* vin, REAL* vout, int W, int H, REAL alpha, REAL rbeta) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            for (int c = 0; c < 2; ++c)
                vout[2 * i + c] = (vin[2 * L + c] + vin[2 * R + c] + vin[2 * B + c] +
                                   vin[2 * T + c] + vin[2 * i + c] * alpha) * rbeta;
        }
}

/* shader.Divergence.comp:15-41 (obstacle neighbours contribute 0 velocity). */
void FN(orc_divergence)(const REAL* v, const unsigned char* obs, REAL* div, int W, int H) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            REAL x1 = obs[L] ? (REAL)0 : v[2 * L];
            REAL x2 = obs[R] ? (REAL)0 : v[2 * R];
            REAL y1 = obs[B] ? (REAL)0 : v[2 * B + 1];
            REAL y2 = obs[T] ? (REAL)0 : v[2 * T + 1];
            div[i] = (REAL)0.5 * ((x2 - x1) + (y2 - y1));
        }
}

/* shader.Poisson.comp:17-38: one Jacobi sweep, obstacle neighbour -> centre. */
void FN(orc_jacobi)(const REAL* pin, REAL* pout, const REAL* div, const unsigned char* obs,
                    int W, int H) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            REAL p = pin[i];
            REAL x1 = obs[L] ? p : pin[L];
            REAL x2 = obs[R] ? p : pin[R];
            REAL y1 = obs[B] ? p : pin[B];
            REAL y2 = obs[T] ? p : pin[T];
            pout[i] = (x1 + x2 + y1 + y2 - div[i]) * (REAL)0.25;
        }
}

/* `sweeps` Jacobi sweeps starting from pin; the result ends in pout.
 * `scratch` is a second W*H buffer.  pin is left unchanged. */
void FN(orc_jacobi_n)(const REAL* pin, REAL* pout, REAL* scratch, const REAL* div,
                      const unsigned char* obs, int W, int H, int sweeps) {
    const REAL* src = pin;
    for (int s = 0; s < sweeps; ++s) {
        /* the last sweep writes pout */
        REAL* dst = ((sweeps - 1 - s) % 2 == 0) ? pout : scratch;
        FN(orc_jacobi)(src, dst, div, obs, W, H);
        src = dst;
    }
    if (sweeps == 0)
        for (long i = 0; i < (long)W * H; ++i) pout[i] = pin[i];
}

/* shader.SubtractGradient.comp:17-47. */
void FN(orc_subtract_gradient)(const REAL* vin, REAL* vout, const REAL* p,
                               const unsigned char* obs, int W, int H) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            REAL pc = p[i];
            REAL x1 = obs[L] ? pc : p[L];
            REAL x2 = obs[R] ? pc : p[R];
            REAL y1 = obs[B] ? pc : p[B];
            REAL y2 = obs[T] ? pc : p[T];
            vout[2 * i] = vin[2 * i] - (REAL)0.5 * (x2 - x1);
            vout[2 * i + 1] = vin[2 * i + 1] - (REAL)0.5 * (y2 - y1);
        }
}

/* demo/shaders/shader.AddParticle.comp:18-36: density cone splat, clamp to
 * [0,255] inside the radius only.  `rows` limits the rows the reference's
 * dispatch reaches (demo/smooth_particles_area.py:80-81 launches the x group
 * count in both dimensions); cells outside keep their value. */
void FN(orc_add_particle)(const REAL* rin, REAL* rout, int Wp, int Hp, float px, float py,
                          float radius, float value, int rows) {
    REAL spx = (REAL)(px * (float)Wp), spy = (REAL)(py * (float)Hp);
    REAL r = radius, S = value;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < Hp; ++y)
        for (int x = 0; x < Wp; ++x) {
            long i = (long)y * Wp + x;
            REAL val = rin[i];
            if (y < rows) {
                REAL dx = spx - (REAL)x, dy = spy - (REAL)y;
                REAL len = SQRT(dx * dx + dy * dy);
                if (len <= r) val = FN(clampr)(val + S * (r - len) / r, (REAL)0, (REAL)255);
            }
            rout[i] = val;
        }
}

/* demo/shaders/shader.AdvectParticle.comp:21-71: density advection on its own
 * grid by the velocity field sampled at the matching normalised position. */
void FN(orc_advect_particle)(const REAL* rin, REAL* rout, const REAL* v,
                             const unsigned char* obs, int Wp, int Hp, int Wv, int Hv,
                             REAL dt, REAL speed, REAL diss) {
    REAL sx = (REAL)((float)Wp / (float)Wv), sy = (REAL)((float)Hp / (float)Hv);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < Hp; ++y)
        for (int x = 0; x < Wp; ++x) {
            long i = (long)y * Wp + x;
            /* normalised position scaled to the velocity grid; the obstacle
             * cell is chosen from the float value in both precisions */
            float nxf = (float)x / (float)Wp * (float)Wv;
            float nyf = (float)y / (float)Hp * (float)Hv;
            long oi = (long)(unsigned)nyf * Wv + (long)(unsigned)nxf;
            if (obs && obs[oi]) {
                rout[i] = 0;
                continue;
            }
            REAL nx = (REAL)x / (REAL)Wp * (REAL)Wv;
            REAL ny = (REAL)y / (REAL)Hp * (REAL)Hv;
            REAL ux, uy;
            FN(sample2)(v, Wv, Hv, nx, ny, &ux, &uy);
            ux = ux * sx;
            uy = uy * sy;
            REAL fx = (REAL)x - ux * dt * speed;
            REAL fy = (REAL)y - uy * dt * speed;
            rout[i] = FN(sample1)(rin, Wp, Hp, fx, fy) * diss;
        }
}

/* shader.AddCircleObstacle.comp:17-37 (both branches write the vec2 (1,0):
 * bit0 alone). */
void FN(orc_add_circle_obstacle)(unsigned char* obs, int W, int H, float px, float py,
                                 float radius) {
    float spx = px * (float)W, spy = py * (float)H;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float dx = spx - (float)x, dy = spy - (float)y;
            if (sqrtf(dx * dx + dy * dy) <= radius) obs[(long)y * W + x] = 1;
        }
}

/* shader.AddTriangleObstacle.comp:19-52 (static -> (0,1) = bit1, else bit0). */
static inline float FN(tsign)(float p1x, float p1y, float p2x, float p2y, float p3x, float p3y) {
    return ((p1x - p3x) * (p2y - p3y)) - ((p2x - p3x) * (p1y - p3y));
}
void FN(orc_add_triangle_obstacle)(unsigned char* obs, int W, int H, float x1, float y1,
                                   float x2, float y2, float x3, float y3, int is_static) {
    unsigned char bit = is_static ? 2 : 1;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float ptx = (float)x / (float)W, pty = (float)y / (float)H;
            int b1 = FN(tsign)(ptx, pty, x1, y1, x2, y2) < 0.0f;
            int b2 = FN(tsign)(ptx, pty, x2, y2, x3, y3) < 0.0f;
            int b3 = FN(tsign)(ptx, pty, x3, y3, x1, y1) < 0.0f;
            if (b1 == b2 && b2 == b3) {
                long i = (long)y * W + x;
                /* the shader overwrites the vec2: the last triangle wins */
                obs[i] = (unsigned char)((obs[i] & ~3) | bit);
            }
        }
}

/* Gaussian splat forcing (no reference counterpart; the workload's forcing).
 * For each splat s in order, every cell gets
 *   w = exp(-d^2 / r^2)  when d^2 <= (3r)^2 (decided in float), else 0
 *   v = clamp(v + w*(svx, svy), -1, 1)        (every cell, like AddVelocity)
 *   rho = clamp(rho + w*sd, 0, 255)           (cells inside the cut-off)
 * on the grid the field lives on; the centre is (px*W, py*H).
 * splats: n records of 6 floats {px, py, radius, svx, svy, sdensity}. */
void FN(orc_gauss_splats)(REAL* v, int W, int H, REAL* rho, int Wp, int Hp,
                          const float* splats, int n) {
    if (v) {
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                long i = (long)y * W + x;
                REAL ax = v[2 * i], ay = v[2 * i + 1];
                for (int s = 0; s < n; ++s) {
                    const float* sp = splats + 6 * s;
                    float cxf = sp[0] * (float)W, cyf = sp[1] * (float)H, rf = sp[2];
                    float dxf = (float)x - cxf, dyf = (float)y - cyf;
                    float cut = 3.0f * rf;
                    if (dxf * dxf + dyf * dyf <= cut * cut) {
                        REAL dx = (REAL)x - (REAL)cxf, dy = (REAL)y - (REAL)cyf;
                        REAL r = rf;
                        REAL w = EXP(-(dx * dx + dy * dy) / (r * r));
                        ax = ax + w * (REAL)sp[3];
                        ay = ay + w * (REAL)sp[4];
                    }
                    ax = FN(clampr)(ax, (REAL)-1, (REAL)1);
                    ay = FN(clampr)(ay, (REAL)-1, (REAL)1);
                }
                v[2 * i] = ax;
                v[2 * i + 1] = ay;
            }
    }
    if (rho) {
#pragma omp parallel for schedule(static)
        for (int y = 0; y < Hp; ++y)
            for (int x = 0; x < Wp; ++x) {
                long i = (long)y * Wp + x;
                REAL a = rho[i];
                for (int s = 0; s < n; ++s) {
                    const float* sp = splats + 6 * s;
                    float cxf = sp[0] * (float)Wp, cyf = sp[1] * (float)Hp, rf = sp[2];
                    float dxf = (float)x - cxf, dyf = (float)y - cyf;
                    float cut = 3.0f * rf;
                    if (dxf * dxf + dyf * dyf <= cut * cut) {
                        REAL dx = (REAL)x - (REAL)cxf, dy = (REAL)y - (REAL)cyf;
                        REAL r = rf;
                        REAL w = EXP(-(dx * dx + dy * dy) / (r * r));
                        a = FN(clampr)(a + w * (REAL)sp[5], (REAL)0, (REAL)255);
                    }
                }
                rho[i] = a;
            }
    }
}

/* Residual of the pressure system the Jacobi sweep iterates
 * (shader.Poisson.comp:17-38 fixed point: sum(pN) - 4 p = div, with the same
 * neighbour substitution), r = div - (sum(pN) - 4 p), accumulated over fluid
 * cells (mask == 0) in double: out = {n, sum r, sum r^2, sum b, sum b^2}. */
void FN(orc_residual)(const REAL* p, const REAL* div, const unsigned char* obs, int W, int H,
                      double* out) {
    double n = 0, sr = 0, srr = 0, sb = 0, sbb = 0;
#pragma omp parallel for schedule(static) reduction(+ : n, sr, srr, sb, sbb)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            if (obs[i]) continue;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            double pc = p[i];
            double x1 = obs[L] ? pc : (double)p[L];
            double x2 = obs[R] ? pc : (double)p[R];
            double y1 = obs[B] ? pc : (double)p[B];
            double y2 = obs[T] ? pc : (double)p[T];
            double b = div[i];
            double r = b - ((x1 + x2 + y1 + y2) - 4.0 * pc);
            n += 1;
            sr += r;
            srr += r * r;
            sb += b;
            sbb += b * b;
        }
    out[0] = n;
    out[1] = sr;
    out[2] = srr;
    out[3] = sb;
    out[4] = sbb;
}

/* The same residual sums per connected fluid region: labels[i] in
 * [0, n_labels) on fluid cells, < 0 on obstacles; out holds n_labels x 5
 * doubles (zeroed here).  The system is pure Neumann on each region, so its
 * residual is defined up to one constant per region. */
void FN(orc_residual_regions)(const REAL* p, const REAL* div, const unsigned char* obs,
                              const int* labels, int n_labels, int W, int H, double* out) {
    for (long k = 0; k < (long)n_labels * 5; ++k) out[k] = 0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long L, R, B, T, i = (long)y * W + x;
            if (obs[i] || labels[i] < 0) continue;
            FN(nbrs)(x, y, W, H, &L, &R, &B, &T);
            double pc = p[i];
            double x1 = obs[L] ? pc : (double)p[L];
            double x2 = obs[R] ? pc : (double)p[R];
            double y1 = obs[B] ? pc : (double)p[B];
            double y2 = obs[T] ? pc : (double)p[T];
            double b = div[i];
            double r = b - ((x1 + x2 + y1 + y2) - 4.0 * pc);
            double* o = out + (long)labels[i] * 5;
            o[0] += 1;
            o[1] += r;
            o[2] += r * r;
            o[3] += b;
            o[4] += b * b;
        }
}

/* Lagrangian particles (no reference counterpart): RK2 midpoint advection in
 * the velocity field with the AdvectVelocity sampler, positions in cells,
 * displacement = v * dt * speed as in the reference, clamped to the grid:
 *   u1 = S(p);  m = p + (h*0.5) * u1;  u2 = S(m);  p' = clamp(p + h*u2, 0, dim-1)
 * with h = dt*speed computed once in float. */
void FN(orc_particles_advect)(float* pos, long n, const REAL* v, int W, int H, float dt,
                              float speed) {
    float h = dt * speed;
    float hh = h * 0.5f;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n; ++k) {
        float px = pos[2 * k], py = pos[2 * k + 1];
        REAL ux, uy;
        FN(sample2)(v, W, H, (REAL)px, (REAL)py, &ux, &uy);
        float mx = px + hh * (float)ux, my = py + hh * (float)uy;
        FN(sample2)(v, W, H, (REAL)mx, (REAL)my, &ux, &uy);
        float qx = px + h * (float)ux, qy = py + h * (float)uy;
        float bx = (float)(W - 1), by = (float)(H - 1);
        qx = qx > 0.0f ? qx : 0.0f;
        qx = qx < bx ? qx : bx;
        qy = qy > 0.0f ? qy : 0.0f;
        qy = qy < by ? qy : by;
        pos[2 * k] = qx;
        pos[2 * k + 1] = qy;
    }
}
