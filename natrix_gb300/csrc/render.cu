// Headless visualisation: the reference demo's display shaders as CUDA
// kernels writing device buffers (no graphics pipeline).
//
//  * density -> RGBA8 texture, demo/shaders/demo.ComputeShader.comp:9-20
//    (imageStore of vec4(v) into an rgba8 image: four equal bytes);
//  * field colour, demo/shaders/demo.FieldFragmentShader.frag:95-99:
//    vec4(plasma(fbm(c)), c) with c the texel read back (k / 255).  The
//    colour depends on the texel byte alone, so a 256-entry palette is built
//    once per device and the per-pixel kernel is a table lookup: 4 bytes
//    read and 4 (texture) + 4 (colour) written per pixel, HBM-bound;
//  * quiver overlay, demo/shaders/demo.QuiverFragmentShader.frag: one
//    arrow per tile (the field sampled at the tile centre), then per window
//    pixel the distance to the arrow's shaft and head -> white with alpha.
//
// Driver-dependent choices (UNORM rounding, sin precision in the hash) are
// fixed as: UNORM8 = 0 for NaN and v <= 0, 255 for v >= 1, else
// round-half-even(v * 255); sin(n) = sin of the float argument in double,
// rounded to float.  Compiled with -fmad=false: each operation rounds
// separately, as the shader text reads.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/natrix.h"
#include "kernels.cuh"

using namespace natrix;

namespace {

constexpr int kMaxDevices = 64;
__device__ uchar4 g_palette[256];
std::mutex g_palette_mu;
bool g_palette_ready[kMaxDevices] = {};

__device__ __forceinline__ unsigned char unorm8(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 1.0f) return 255;
    return (unsigned char)rintf(v * 255.0f);
}

__device__ __forceinline__ float hash1(float n) {
    const float s = (float)sin((double)n);
    const float y = s * 43758.5453123f;
    return y - floorf(y);
}

__device__ __forceinline__ float noise1(float p) {
    const float fl = floorf(p);
    const float fc = p - floorf(p);
    const float a = hash1(fl), b = hash1(fl + 1.0f);
    return a + fc * (b - a);
}

__device__ float fbm(float x) {
    float v = 0.0f, a = 0.5f;
    const float shift = 100.0f;
#pragma unroll 1
    for (int i = 0; i < 5; ++i) {
        v = v + a * noise1(x);
        x = x * 2.0f + shift;
        a = a * 0.5f;
    }
    return v;
}

// plasma colour map polynomial coefficients (c0..c6 per channel), from the
// field shader's plasma(): c0 + t*(c1 + t*(c2 + ... + t*c6))
__constant__ float kPlasma[7][3] = {
    {0.05873234392399702f, 0.02333670892565664f, 0.5433401826748754f},
    {2.176514634195958f, 0.2383834171260182f, 0.7539604599784036f},
    {-2.689460476458034f, -7.455851135738909f, 3.110799939717086f},
    {6.130348345893603f, 42.3461881477227f, -28.51885465332158f},
    {-11.10743619062271f, -82.66631109428045f, 60.13984767418263f},
    {10.02306557647065f, 71.41361770095349f, -54.07218655560067f},
    {-3.658713842777788f, -22.93153465461149f, 18.19190778539828f},
};

__device__ __forceinline__ float plasma(float t, int ch) {
    float r = kPlasma[6][ch];
#pragma unroll
    for (int i = 5; i >= 0; --i) r = kPlasma[i][ch] + t * r;
    return r;
}

__global__ void k_palette() {
    const int k = threadIdx.x;
    const float c = (float)k / 255.0f;
    const float t = fbm(c);
    g_palette[k] = make_uchar4(unorm8(plasma(t, 0)), unorm8(plasma(t, 1)), unorm8(plasma(t, 2)),
                               unorm8(c));
}

constexpr int kRenderThreads = 256;

// Four pixels of one row per thread when the row start, pitches and buffers
// allow 16-byte accesses; a scalar path otherwise and for row tails.
__global__ void __launch_bounds__(kRenderThreads)
    k_render_density(const float* __restrict__ rho, int W, int H, long pitch,
                     uchar4* __restrict__ tex, uchar4* __restrict__ col, long opitch, bool vec) {
    __shared__ uchar4 pal[256];
    pal[threadIdx.x] = g_palette[threadIdx.x];
    __syncthreads();
    const int qw = (W + 3) / 4;
    const long total = (long)qw * H;
    for (long q = (long)blockIdx.x * kRenderThreads + threadIdx.x; q < total;
         q += (long)gridDim.x * kRenderThreads) {
        const int y = (int)(q / qw), x0 = (int)(q % qw) * 4;
        const float* src = rho + (long)y * pitch + x0;
        const long o = (long)y * opitch + x0;
        if (vec && x0 + 3 < W) {
            const float4 v = __ldcs(reinterpret_cast<const float4*>(src));
            const unsigned char k0 = unorm8(v.x), k1 = unorm8(v.y), k2 = unorm8(v.z),
                                k3 = unorm8(v.w);
            if (tex) {
                uint4 t;
                t.x = 0x01010101u * k0;
                t.y = 0x01010101u * k1;
                t.z = 0x01010101u * k2;
                t.w = 0x01010101u * k3;
                __stcs(reinterpret_cast<uint4*>(tex + o), t);
            }
            if (col) {
                uint4 c;
                const uchar4 p0 = pal[k0], p1 = pal[k1], p2 = pal[k2], p3 = pal[k3];
                c.x = *reinterpret_cast<const unsigned*>(&p0);
                c.y = *reinterpret_cast<const unsigned*>(&p1);
                c.z = *reinterpret_cast<const unsigned*>(&p2);
                c.w = *reinterpret_cast<const unsigned*>(&p3);
                __stcs(reinterpret_cast<uint4*>(col + o), c);
            }
        } else {
            for (int i = 0; i < 4 && x0 + i < W; ++i) {
                const unsigned char k = unorm8(src[i]);
                if (tex) tex[o + i] = make_uchar4(k, k, k, k);
                if (col) col[o + i] = pal[k];
            }
        }
    }
}

// ---- quiver ----

struct QuiverGeom {
    int VW, VH;       // velocity grid
    long vpitch;      // float2 elements per velocity row
    float winW, winH; // window (overlay) size in pixels
    float T;          // arrow tile size in pixels
    int nx, ny;       // tiles
};

// _field (QuiverFragmentShader.frag:49-64): the shader's mix weights are
// vec2(delta, 0), so only x is interpolated; y is the lower-left corner's.
__device__ float2 field_at(const float2* __restrict__ v, const QuiverGeom& g, float px, float py) {
    const float fx = (1.0f - px / g.winW) * (float)g.VW;
    const float fy = (1.0f - py / g.winH) * (float)g.VH;
    const float bx = (float)(g.VW - 1), by = (float)(g.VH - 1);
    const float tx = fminf(fmaxf(ceilf(fx), 0.0f), bx), ty = fminf(fmaxf(ceilf(fy), 0.0f), by);
    const float lx = fminf(fmaxf(floorf(fx), 0.0f), bx), ly = fminf(fmaxf(floorf(fy), 0.0f), by);
    const float dx = fx - lx, dy = fy - ly;
    const long itx = (long)tx, ity = (long)ty, ilx = (long)lx, ily = (long)ly;
    const float2 lt = v[ity * g.vpitch + ilx], rt = v[ity * g.vpitch + itx];
    const float2 lb = v[ily * g.vpitch + ilx], rb = v[ily * g.vpitch + itx];
    const float h1x = lt.x + dx * (rt.x - lt.x);
    const float h2x = lb.x + dx * (rb.x - lb.x);
    const float h1y = lt.y + 0.0f * (rt.y - lt.y);
    const float h2y = lb.y + 0.0f * (rb.y - lb.y);
    const float mx = h2x + dy * (h1x - h2x);
    const float my = h2y + 0.0f * (h1y - h2y);
    return make_float2((-1.0f * mx) * (g.winW / (float)g.VW), (-1.0f * my) * (g.winH / (float)g.VH));
}

__global__ void k_quiver_arrows(const float2* __restrict__ v, QuiverGeom g,
                                float2* __restrict__ arrows) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)g.nx * g.ny) return;
    const int i = (int)(t % g.nx), j = (int)(t / g.nx);
    const float2 f = field_at(v, g, ((float)i + 0.5f) * g.T, ((float)j + 0.5f) * g.T);
    arrows[t] = make_float2((f.x * g.T) * 0.4f, (f.y * g.T) * 0.4f);
}

__device__ __forceinline__ float len2(float x, float y) { return sqrtf(x * x + y * y); }

// _line (:18-26)
__device__ float seg(float px, float py, float ax, float ay, float bx, float by) {
    const float cx = (ax + bx) * 0.5f, cy = (ay + by) * 0.5f;
    const float ex = bx - ax, ey = by - ay;
    const float len = len2(ex, ey);
    const float dx = ex / len, dy = ey / len;
    const float rx = px - cx, ry = py - cy;
    const float d1 = fabsf(rx * dy + ry * -dx);
    const float d2 = fabsf(rx * dx + ry * dy) - 0.5f * len;
    return fmaxf(d1, d2);
}

// _vector (:28-47), p relative to the tile centre
__device__ float arrow_dist(float px, float py, float vx, float vy, float T) {
    float mag = len2(vx, vy);
    if (!(mag > 0.001f)) return 1.0f;
    const float dx = vx / mag, dy = vy / mag;
    mag = fminf(fmaxf(mag, 0.0f), T * 0.5f);
    vx = dx * mag;
    vy = dy * mag;
    const float shaft = seg(px, py, vx, vy, -vx, -vy);
    const float h1 = seg(px, py, vx, vy, 0.4f * vx + 0.2f * -vy, 0.4f * vy + 0.2f * vx);
    const float h2 = seg(px, py, vx, vy, 0.4f * vx + 0.2f * vy, 0.4f * vy + 0.2f * -vx);
    return fminf(shaft, fminf(h1, h2));
}

__global__ void __launch_bounds__(kRenderThreads)
    k_quiver_overlay(const float2* __restrict__ arrows, QuiverGeom g, int W, int H,
                     uchar4* __restrict__ out, long opitch) {
    const long total = (long)W * H;
    for (long p = (long)blockIdx.x * kRenderThreads + threadIdx.x; p < total;
         p += (long)gridDim.x * kRenderThreads) {
        const int y = (int)(p / W), x = (int)(p % W);
        const float px = (float)x + 0.5f, py = (float)y + 0.5f;
        int ti = (int)floorf(px / g.T), tj = (int)floorf(py / g.T);
        ti = min(max(ti, 0), g.nx - 1);
        tj = min(max(tj, 0), g.ny - 1);
        const float cx = (floorf(px / g.T) + 0.5f) * g.T, cy = (floorf(py / g.T) + 0.5f) * g.T;
        const float2 a = arrows[(long)tj * g.nx + ti];
        const float d = arrow_dist(px - cx, py - cy, a.x, a.y, g.T);
        const float alpha = 1.0f - fminf(fmaxf(d, 0.0f), 1.0f);
        out[(long)y * opitch + x] = make_uchar4(255, 255, 255, unorm8(alpha));
    }
}

// Integer tile sizes: one block per tile.  The arrow's three segments (shaft
// and two head strokes) depend only on the tile, so one thread evaluates
// _line's per-segment terms (centre, direction, half length) once and every
// pixel does the two dot products; the values are those arrow_dist computes,
// so the overlay is identical to the per-pixel kernel's.
struct Seg {
    float cx, cy, dx, dy, hl;
};

__device__ Seg make_seg(float ax, float ay, float bx, float by) {
    Seg s;
    s.cx = (ax + bx) * 0.5f;
    s.cy = (ay + by) * 0.5f;
    const float ex = bx - ax, ey = by - ay;
    const float len = len2(ex, ey);
    s.dx = ex / len;
    s.dy = ey / len;
    s.hl = 0.5f * len;
    return s;
}

__device__ __forceinline__ float seg_dist(const Seg& s, float px, float py) {
    const float rx = px - s.cx, ry = py - s.cy;
    const float d1 = fabsf(rx * s.dy + ry * -s.dx);
    const float d2 = fabsf(rx * s.dx + ry * s.dy) - s.hl;
    return fmaxf(d1, d2);
}

__global__ void __launch_bounds__(kRenderThreads)
    k_quiver_overlay_tiles(const float2* __restrict__ arrows, QuiverGeom g, int W, int H, int T,
                           uchar4* __restrict__ out, long opitch) {
    __shared__ Seg segs[3];
    __shared__ int s_live;
    for (long tile = blockIdx.x; tile < (long)g.nx * g.ny; tile += gridDim.x) {
        const int ti = (int)(tile % g.nx), tj = (int)(tile / g.nx);
        if (threadIdx.x == 0) {
            float vx = arrows[tile].x, vy = arrows[tile].y;
            float mag = len2(vx, vy);
            s_live = mag > 0.001f;
            if (s_live) {
                const float ux = vx / mag, uy = vy / mag;
                mag = fminf(fmaxf(mag, 0.0f), g.T * 0.5f);
                vx = ux * mag;
                vy = uy * mag;
                segs[0] = make_seg(vx, vy, -vx, -vy);
                segs[1] = make_seg(vx, vy, 0.4f * vx + 0.2f * -vy, 0.4f * vy + 0.2f * vx);
                segs[2] = make_seg(vx, vy, 0.4f * vx + 0.2f * vy, 0.4f * vy + 0.2f * -vx);
            }
        }
        __syncthreads();
        const float cx = ((float)ti + 0.5f) * g.T, cy = ((float)tj + 0.5f) * g.T;
        const int x0 = ti * T, y0 = tj * T;
        const bool live = s_live != 0;
        for (int k = threadIdx.x; k < T * T; k += kRenderThreads) {
            const int x = x0 + k % T, y = y0 + k / T;
            if (x >= W || y >= H) continue;
            float d = 1.0f;
            if (live) {
                const float px = ((float)x + 0.5f) - cx, py = ((float)y + 0.5f) - cy;
                d = fminf(seg_dist(segs[0], px, py),
                          fminf(seg_dist(segs[1], px, py), seg_dist(segs[2], px, py)));
            }
            const float alpha = 1.0f - fminf(fmaxf(d, 0.0f), 1.0f);
            out[(long)y * opitch + x] = make_uchar4(255, 255, 255, unorm8(alpha));
        }
        __syncthreads();
    }
}

int fail(int code, const char* msg) { return set_last_error(code, msg); }

int cuda_fail(cudaError_t e) { return set_last_error(NATRIX_ECUDA, cudaGetErrorString(e)); }

int grid_blocks(long work) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long need = (work + kRenderThreads - 1) / kRenderThreads;
    const long cap = (long)sms * 8;
    return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

int ensure_palette(cudaStream_t st) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e);
    if (dev < 0 || dev >= kMaxDevices) return fail(NATRIX_EDEVICE, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_palette_mu);
    if (g_palette_ready[dev]) return NATRIX_OK;
    k_palette<<<1, 256, 0, st>>>();
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
    // later launches on any stream read the table: finish it first
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e);
    g_palette_ready[dev] = true;
    return NATRIX_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" {

int natrix_render_density(const float* density, int32_t W, int32_t H, int64_t pitch,
                          uint8_t* texture, uint8_t* colour, int64_t out_pitch, void* stream) {
    if (!density || W < 1 || H < 1 || pitch < W || out_pitch < W)
        return fail(NATRIX_EINVAL, "render_density: bad pointer or size");
    if (!texture && !colour) return NATRIX_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = ensure_palette(st);
    if (rc != NATRIX_OK) return rc;
    const bool vec = aligned16(density) && pitch % 4 == 0 && out_pitch % 4 == 0 &&
                     (!texture || aligned16(texture)) && (!colour || aligned16(colour));
    const long quads = (long)((W + 3) / 4) * H;
    k_render_density<<<grid_blocks(quads), kRenderThreads, 0, st>>>(
        density, W, H, pitch, reinterpret_cast<uchar4*>(texture), reinterpret_cast<uchar4*>(colour),
        out_pitch, vec);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NATRIX_OK : cuda_fail(e);
}

int natrix_quiver_tiles(int32_t win_w, int32_t win_h, float tile, int32_t* nx, int32_t* ny) {
    if (win_w < 1 || win_h < 1 || !(tile >= 1.0f) || !(tile <= 65536.0f) || !nx || !ny)
        return fail(NATRIX_EINVAL, "quiver: window must be >= 1 pixel and tile in [1, 65536]");
    // the largest tile index a pixel centre reaches, + 1
    *nx = (int32_t)floorf(((float)win_w - 0.5f) / tile) + 1;
    *ny = (int32_t)floorf(((float)win_h - 0.5f) / tile) + 1;
    return NATRIX_OK;
}

int natrix_quiver(const float* velocity, int32_t W, int32_t H, int64_t pitch, int32_t win_w,
                  int32_t win_h, float tile, float* arrows, uint8_t* overlay, int64_t overlay_pitch,
                  void* stream) {
    if (!velocity || !arrows || W < 1 || H < 1 || pitch < W)
        return fail(NATRIX_EINVAL, "quiver: bad velocity or arrow buffer");
    int32_t nx = 0, ny = 0;
    int rc = natrix_quiver_tiles(win_w, win_h, tile, &nx, &ny);
    if (rc != NATRIX_OK) return rc;
    if (overlay && overlay_pitch < win_w) return fail(NATRIX_EINVAL, "quiver: overlay pitch < width");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    QuiverGeom g{W, H, pitch, (float)win_w, (float)win_h, tile, nx, ny};
    const long tiles = (long)nx * ny;
    k_quiver_arrows<<<(unsigned)((tiles + 127) / 128), 128, 0, st>>>(
        reinterpret_cast<const float2*>(velocity), g, reinterpret_cast<float2*>(arrows));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e);
    if (overlay) {
        const int ti = (int)tile;
        if ((float)ti == tile && ti <= 256) {
            const long nt = tiles < 65535L * 8 ? tiles : 65535L * 8;
            k_quiver_overlay_tiles<<<(unsigned)nt, kRenderThreads, 0, st>>>(
                reinterpret_cast<const float2*>(arrows), g, win_w, win_h, ti,
                reinterpret_cast<uchar4*>(overlay), overlay_pitch);
        } else {
            const long px = (long)win_w * win_h;
            k_quiver_overlay<<<grid_blocks(px), kRenderThreads, 0, st>>>(
                reinterpret_cast<const float2*>(arrows), g, win_w, win_h,
                reinterpret_cast<uchar4*>(overlay), overlay_pitch);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
    }
    return NATRIX_OK;
}

}  // extern "C"
