/* CPU oracle for the headless visualisation kernels — TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference demo's display shaders:
 *   demo/shaders/demo.ComputeShader.comp:9-20     density -> rgba8 texture
 *   demo/shaders/demo.FieldFragmentShader.frag    plasma(fbm(texel)) colour
 *   demo/shaders/demo.QuiverFragmentShader.frag   velocity arrows overlay
 * evaluated per output pixel with no graphics pipeline: one output pixel per
 * texel for the field, pixel centres (x + 0.5, y + 0.5) for the quiver.
 *
 * Choices the shader text leaves to the GPU driver, made identically in the
 * CUDA kernels (natrix_gb300/csrc/render.cu):
 *   - float -> UNORM8: 0 for NaN and v <= 0, 255 for v >= 1, else
 *     round-to-nearest-even(v * 255);
 *   - texel fetch of byte k returns k / 255.0f (correctly rounded);
 *   - sin(n) in the hash is sin of the float argument evaluated in double and
 *     rounded to float (GLSL leaves its precision open);
 *   - mix(a, b, t) = a + t * (b - a), length(v) = sqrt(x*x + y*y), every
 *     operation rounding separately (compiled with -ffp-contract=off).
 * Only tests/ load this library.
 */
#include <math.h>
#include <stdint.h>

static unsigned char unorm8(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 1.0f) return 255;
    return (unsigned char)rintf(v * 255.0f);
}

/* rand(n) = fract(sin(n) * 43758.5453123), demo.FieldFragmentShader.frag:75 */
static float hash1(float n) {
    float s = (float)sin((double)n);
    float y = s * 43758.5453123f;
    return y - floorf(y);
}

/* noise and fbm (5 octaves, shift 100), demo.FieldFragmentShader.frag:77-93 */
static float noise1(float p) {
    float fl = floorf(p);
    float fc = p - floorf(p);
    float a = hash1(fl), b = hash1(fl + 1.0f);
    return a + fc * (b - a);
}

static float fbm(float x) {
    float v = 0.0f, a = 0.5f;
    const float shift = 100.0f;
    for (int i = 0; i < 5; ++i) {
        v = v + a * noise1(x);
        x = x * 2.0f + shift;
        a = a * 0.5f;
    }
    return v;
}

/* plasma colour map polynomial, demo.FieldFragmentShader.frag:21-33 */
static const float kPlasma[7][3] = {
    {0.05873234392399702f, 0.02333670892565664f, 0.5433401826748754f},
    {2.176514634195958f, 0.2383834171260182f, 0.7539604599784036f},
    {-2.689460476458034f, -7.455851135738909f, 3.110799939717086f},
    {6.130348345893603f, 42.3461881477227f, -28.51885465332158f},
    {-11.10743619062271f, -82.66631109428045f, 60.13984767418263f},
    {10.02306557647065f, 71.41361770095349f, -54.07218655560067f},
    {-3.658713842777788f, -22.93153465461149f, 18.19190778539828f},
};

static float plasma(float t, int ch) {
    float r = kPlasma[6][ch];
    for (int i = 5; i >= 0; --i) r = kPlasma[i][ch] + t * r;
    return r;
}

/* Colour of texel byte k: gl_FragColor = vec4(plasma(fbm(c)), c), c = k/255
 * (demo.FieldFragmentShader.frag:95-99), stored as RGBA8. */
void orc_plasma_palette(uint8_t* pal /* 256 x 4 */) {
    for (int k = 0; k < 256; ++k) {
        float c = (float)k / 255.0f;
        float t = fbm(c);
        for (int ch = 0; ch < 3; ++ch) pal[4 * k + ch] = unorm8(plasma(t, ch));
        pal[4 * k + 3] = unorm8(c);
    }
}

/* density (W*H float, row-major) -> texture (rgba8, the compute shader's
 * imageStore of vec4(v)) and colour (the field shader's output). */
void orc_render_density(const float* rho, int W, int H, uint8_t* tex, uint8_t* col) {
    uint8_t pal[256 * 4];
    orc_plasma_palette(pal);
    for (long i = 0; i < (long)W * H; ++i) {
        unsigned char k = unorm8(rho[i]);
        for (int ch = 0; ch < 4; ++ch) {
            if (tex) tex[4 * i + ch] = k;
            if (col) col[4 * i + ch] = pal[4 * k + ch];
        }
    }
}

/* ---- quiver (demo.QuiverFragmentShader.frag) ---- */

/* _arrow_tile_center_coord, :14-16 */
static float tile_centre(float p, float T) { return (floorf(p / T) + 0.5f) * T; }

/* _field, :49-64: bilinear sample at the flipped position.  The shader's
 * mix weights are vec2(delta, 0), so only the x component is interpolated;
 * the y component is the lower-left corner's. */
static void field_at(const float* v, int VW, int VH, float winW, float winH, float px, float py,
                     float out[2]) {
    float fx = (1.0f - px / winW) * (float)VW;
    float fy = (1.0f - py / winH) * (float)VH;
    float bx = (float)(VW - 1), by = (float)(VH - 1);
    float tx = fminf(fmaxf(ceilf(fx), 0.0f), bx), ty = fminf(fmaxf(ceilf(fy), 0.0f), by);
    float lx = fminf(fmaxf(floorf(fx), 0.0f), bx), ly = fminf(fmaxf(floorf(fy), 0.0f), by);
    float dx = fx - lx, dy = fy - ly;
    long itx = (long)tx, ity = (long)ty, ilx = (long)lx, ily = (long)ly;
    const float* lt = v + 2 * (ity * VW + ilx);
    const float* rt = v + 2 * (ity * VW + itx);
    const float* lb = v + 2 * (ily * VW + ilx);
    const float* rb = v + 2 * (ily * VW + itx);
    float h1x = lt[0] + dx * (rt[0] - lt[0]);
    float h2x = lb[0] + dx * (rb[0] - lb[0]);
    float h1y = lt[1] + 0.0f * (rt[1] - lt[1]);
    float h2y = lb[1] + 0.0f * (rb[1] - lb[1]);
    float mx = h2x + dy * (h1x - h2x);
    float my = h2y + 0.0f * (h1y - h2y);
    out[0] = (-1.0f * mx) * (winW / (float)VW);
    out[1] = (-1.0f * my) * (winH / (float)VH);
}

/* Arrow of every tile: field(tile centre) * T * 0.4 (:68), nx = ceil(winW/T)
 * tiles per row, row-major. */
void orc_quiver_arrows(const float* v, int VW, int VH, int winW, int winH, float T, float* arrows,
                       int nx, int ny) {
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            float cx = ((float)i + 0.5f) * T, cy = ((float)j + 0.5f) * T;
            float f[2];
            field_at(v, VW, VH, (float)winW, (float)winH, cx, cy, f);
            arrows[2 * ((long)j * nx + i)] = (f[0] * T) * 0.4f;
            arrows[2 * ((long)j * nx + i) + 1] = (f[1] * T) * 0.4f;
        }
}

static float len2(float x, float y) { return sqrtf(x * x + y * y); }

/* _line, :18-26 */
static float seg(float px, float py, float ax, float ay, float bx, float by) {
    float cx = (ax + bx) * 0.5f, cy = (ay + by) * 0.5f;
    float ex = bx - ax, ey = by - ay;
    float len = len2(ex, ey);
    float dx = ex / len, dy = ey / len;
    float rx = px - cx, ry = py - cy;
    float d1 = fabsf(rx * dy + ry * -dx);
    float d2 = fabsf(rx * dx + ry * dy) - 0.5f * len;
    return fmaxf(d1, d2);
}

/* _vector, :28-47, with p already relative to the tile centre */
static float arrow_dist(float px, float py, float vx, float vy, float T) {
    float mag = len2(vx, vy);
    if (!(mag > 0.001f)) return 1.0f;
    float dx = vx / mag, dy = vy / mag;
    mag = fminf(fmaxf(mag, 0.0f), T * 0.5f);
    vx = dx * mag;
    vy = dy * mag;
    float shaft = seg(px, py, vx, vy, -vx, -vy);
    float h1 = seg(px, py, vx, vy, 0.4f * vx + 0.2f * -vy, 0.4f * vy + 0.2f * vx);
    float h2 = seg(px, py, vx, vy, 0.4f * vx + 0.2f * vy, 0.4f * vy + 0.2f * -vx);
    return fminf(shaft, fminf(h1, h2));
}

/* Overlay pixel (x, y): gl_FragCoord = (x + 0.5, y + 0.5), colour
 * vec4(1, 1, 1, 1 - clamp(dist, 0, 1)) (:66-70), as RGBA8. */
void orc_quiver_overlay(const float* arrows, int nx, int winW, int winH, float T, uint8_t* out) {
    for (int y = 0; y < winH; ++y)
        for (int x = 0; x < winW; ++x) {
            float px = (float)x + 0.5f, py = (float)y + 0.5f;
            float cx = tile_centre(px, T), cy = tile_centre(py, T);
            long ti = (long)(floorf(py / T)) * nx + (long)floorf(px / T);
            float d = arrow_dist(px - cx, py - cy, arrows[2 * ti], arrows[2 * ti + 1], T);
            float a = 1.0f - fminf(fmaxf(d, 0.0f), 1.0f);
            uint8_t* o = out + 4 * ((long)y * winW + x);
            o[0] = o[1] = o[2] = 255;
            o[3] = unorm8(a);
        }
}
