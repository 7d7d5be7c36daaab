// U-Net warm start: every kernel but the tensor-core convolutions
// (unet_conv.cu).  Activations are NHWC bf16; gradients of activations bf16;
// parameters, their gradients and the Adam state FP32.
//
//  * pack_weights: FP32 [cout][cin][3][3] master weights -> bf16 B operand in
//    the tcgen05 SWIZZLE_NONE K-major layout (forward: rows = cout, K =
//    (tap, cin); input gradient: rows = cin, K = (tap, cout), taps flipped).
//  * wgrad: dW[co][ci][t] = sum_p dZ[p][co] * X[p + off(t)][ci] and
//    db[co] = sum_p dZ[p][co] on CUDA cores: each CTA owns one tap and a
//    slice of the pixels, accumulates in registers, then one atomic per weight.
//  * prep / pool / upsample (and their gradients with the ReLU gate), head
//    gradient, loss + gradient, Adam.
//  * FP64 conjugate gradients on the pressure operator of the solver
//    (shader.Poisson.comp:17-38 fixed point restricted to fluid cells), one
//    independent system per image, for the training targets.
#include <cuda_runtime.h>

#include <cstdlib>

#include "../../include/natrix.h"
#include "../../include/natrix_nn.h"
#include "kernels.cuh"

namespace natrix {

namespace {

__device__ __forceinline__ float bf(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }
__device__ __forceinline__ uint16_t tobf(float f) {
    uint32_t u = __float_as_uint(f);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

inline unsigned blocks(long n, int t) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------------ weights
// element (row n, K index k) of an N x K operand -> byte offset in the layout
__device__ __forceinline__ size_t core_off(int n, int k, int N) {
    const size_t lbo = (size_t)(N / 8) * 128;
    return (size_t)(n / 8) * 128 + (size_t)(k / 8) * lbo + (n % 8) * 16 + (k % 8) * 2;
}

__global__ void k_pack(const float* __restrict__ w, int cout, int cin, int rows, int kc,
                       int dgrad, uint16_t* __restrict__ out) {
    // rows x (9 * kc) operand; forward: rows = cout (padded), kc = cin padded;
    // dgrad: rows = cin (padded), kc = cout padded
    const long total = (long)rows * 9 * kc;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
         i += (long)gridDim.x * blockDim.x) {
        const int n = (int)(i / (9 * kc));
        const int k = (int)(i % (9 * kc));
        const int t = k / kc, c = k % kc;
        float v = 0.0f;
        if (!dgrad) {
            if (n < cout && c < cin) v = w[((size_t)n * cin + c) * 9 + t];
        } else {
            if (n < cin && c < cout) v = w[((size_t)c * cin + n) * 9 + (8 - t)];
        }
        out[core_off(n, k, rows) / 2] = tobf(v);
    }
}

// -------------------------------------------------------------------- wgrad
// grid = (9 taps, pixel slices); block = 256 threads, each owning a 4 x 4
// register block of (co, ci) pairs; PIX pixels staged in shared memory.
constexpr int WG_PIX = 32;

__global__ void __launch_bounds__(256)
    k_wgrad(const uint16_t* __restrict__ dz, int cout, const uint16_t* __restrict__ x0, int c0,
            const uint16_t* __restrict__ x1, int c1, int B, int H, int W, float* __restrict__ dw,
            float* __restrict__ db) {
    const int cin = c0 + c1;
    const int t = blockIdx.x, dy = t / 3 - 1, dx = t % 3 - 1;
    extern __shared__ float sm[];
    float* sdz = sm;                        // WG_PIX x cout
    float* sx = sm + WG_PIX * cout;         // WG_PIX x cin
    const int co_blocks = (cout + 3) / 4, ci_blocks = (cin + 3) / 4;
    const int pairs = co_blocks * ci_blocks;
    float acc[4][4];
    float bacc[4] = {0, 0, 0, 0};
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
    const long npix = (long)B * H * W;
    const long per = (npix + gridDim.y - 1) / gridDim.y;
    const long p0 = (long)blockIdx.y * per, p1 = p0 + per < npix ? p0 + per : npix;
    // thread -> register block (several passes when pairs > 256)
    for (int pb = threadIdx.x; pb - threadIdx.x < pairs; pb += 256) {
        const bool mine = pb < pairs;
        const int cob = mine ? pb / ci_blocks : 0, cib = mine ? pb % ci_blocks : 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            bacc[a] = 0.0f;
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
        }
        for (long base = p0; base < p1; base += WG_PIX) {
            __syncthreads();
            // stage WG_PIX pixels: 8 channels (16 bytes) per load, 32-bit indices
            const int cz8 = cout / 8, ci8 = cin / 8, c08 = c0 / 8;
            for (int i = threadIdx.x; i < WG_PIX * cz8; i += 256) {
                const int k = i / cz8, q = i % cz8;
                const int p = (int)base + k;
                float* d = sdz + k * cout + 8 * q;
                if (p < (int)p1) {
                    const uint4 u = *reinterpret_cast<const uint4*>(dz + (size_t)p * cout + 8 * q);
                    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        d[2 * j] = bf((uint16_t)(w[j] & 0xffffu));
                        d[2 * j + 1] = bf((uint16_t)(w[j] >> 16));
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 8; ++j) d[j] = 0.0f;
                }
            }
            for (int i = threadIdx.x; i < WG_PIX * ci8; i += 256) {
                const int k = i / ci8, q = i % ci8;
                const int p = (int)base + k;
                float* d = sx + k * cin + 8 * q;
                uint4 u = make_uint4(0, 0, 0, 0);
                if (p < (int)p1) {
                    const int xx = p % W, yb = p / W;
                    const int yy = yb % H, bb = yb / H;
                    const int sx_ = xx + dx, sy_ = yy + dy;
                    if (sx_ >= 0 && sx_ < W && sy_ >= 0 && sy_ < H) {
                        const int src = (bb * H + sy_) * W + sx_;
                        u = q < c08 ? *reinterpret_cast<const uint4*>(x0 + (size_t)src * c0 + 8 * q)
                                    : *reinterpret_cast<const uint4*>(x1 + (size_t)src * c1 +
                                                                       8 * (q - c08));
                    }
                }
                const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    d[2 * j] = bf((uint16_t)(w[j] & 0xffffu));
                    d[2 * j + 1] = bf((uint16_t)(w[j] >> 16));
                }
            }
            __syncthreads();
            if (mine) {
                const int np = (int)(p1 - base < WG_PIX ? p1 - base : WG_PIX);
                for (int k = 0; k < np; ++k) {
                    float g[4], xv[4];
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const int co = cob * 4 + a;
                        g[a] = co < cout ? sdz[k * cout + co] : 0.0f;
                    }
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const int ci = cib * 4 + b;
                        xv[b] = ci < cin ? sx[k * cin + ci] : 0.0f;
                    }
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        bacc[a] += g[a];
#pragma unroll
                        for (int b = 0; b < 4; ++b) acc[a][b] += g[a] * xv[b];
                    }
                }
            }
        }
        if (mine) {
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const int co = cob * 4 + a;
                if (co >= cout) continue;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int ci = cib * 4 + b;
                    if (ci < cin) atomicAdd(dw + ((size_t)co * cin + ci) * 9 + t, acc[a][b]);
                }
                if (db && t == 4 && cib == 0) atomicAdd(db + co, bacc[a]);
            }
        }
    }
}

// ------------------------------------------------------------- elementwise
// x = [div / scale, obstacle, 0 x 6] (8-channel NHWC bf16)
__global__ void k_prep(const float* __restrict__ div, const uint8_t* __restrict__ mask,
                       const float* __restrict__ inv_scale, int B, int H, int W, int pitch,
                       uint16_t* __restrict__ x) {
    const long n = (long)B * H * W;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const long b = i / ((long)H * W);
        const long r = i % ((long)H * W);
        const long src = b * (long)H * pitch + (r / W) * pitch + r % W;
        const float d = div[src] * inv_scale[b];
        const float m = mask && mask[src] ? 1.0f : 0.0f;
        uint4 v = make_uint4((uint32_t)tobf(d) | ((uint32_t)tobf(m) << 16), 0, 0, 0);
        *reinterpret_cast<uint4*>(x + i * 8) = v;
    }
}

// Pooling / upsampling and their gradients on NHWC bf16 tensors, eight
// channels (16 bytes) per thread, 32-bit pixel indices (C is a multiple of 8).
struct Bf8 {
    float v[8];
};

__device__ __forceinline__ Bf8 ld8(const uint16_t* p) {
    const uint4 q = *reinterpret_cast<const uint4*>(p);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
    Bf8 r;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        r.v[2 * j] = bf((uint16_t)(w[j] & 0xffffu));
        r.v[2 * j + 1] = bf((uint16_t)(w[j] >> 16));
    }
    return r;
}

__device__ __forceinline__ void st8(uint16_t* p, const Bf8& r) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
        w[j] = (uint32_t)tobf(r.v[2 * j]) | ((uint32_t)tobf(r.v[2 * j + 1]) << 16);
    *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
}

// 2x2 average pooling: one thread per output pixel and 8-channel chunk
__global__ void k_pool(const uint16_t* __restrict__ in, int B, int H, int W, int C,
                       uint16_t* __restrict__ out) {
    const int Ho = H / 2, Wo = W / 2, CC = C / 8;
    const int n = B * Ho * Wo * CC;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int q = i % CC, p = i / CC;
        const int x = p % Wo, yb = p / Wo;  // yb = b * Ho + y
        const int y = yb % Ho, b = yb / Ho;
        const int src = (b * H + 2 * y) * W + 2 * x;
        const Bf8 a = ld8(in + (size_t)src * C + 8 * q), c = ld8(in + (size_t)(src + 1) * C + 8 * q),
                  d = ld8(in + (size_t)(src + W) * C + 8 * q),
                  e = ld8(in + (size_t)(src + W + 1) * C + 8 * q);
        Bf8 r;
#pragma unroll
        for (int j = 0; j < 8; ++j) r.v[j] = 0.25f * (((a.v[j] + c.v[j]) + d.v[j]) + e.v[j]);
        st8(out + (size_t)i * 8, r);
    }
}

// nearest upsampling x2: one thread per input pixel and chunk, four stores
__global__ void k_up(const uint16_t* __restrict__ in, int B, int H, int W, int C,
                     uint16_t* __restrict__ out) {
    const int CC = C / 8, Wo = 2 * W;
    const int n = B * H * W * CC;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int q = i % CC, p = i / CC;
        const int x = p % W, yb = p / W;  // yb = b * H + y
        const uint4 v = *reinterpret_cast<const uint4*>(in + (size_t)i * 8);
        const int dst = (2 * yb) * Wo + 2 * x;  // (b * 2H + 2y) * 2W + 2x
        *reinterpret_cast<uint4*>(out + (size_t)dst * C + 8 * q) = v;
        *reinterpret_cast<uint4*>(out + (size_t)(dst + 1) * C + 8 * q) = v;
        *reinterpret_cast<uint4*>(out + (size_t)(dst + Wo) * C + 8 * q) = v;
        *reinterpret_cast<uint4*>(out + (size_t)(dst + Wo + 1) * C + 8 * q) = v;
    }
}

// gradient of nearest upsampling (sum of the 4 children), times (gate > 0)
__global__ void k_up_back(const uint16_t* __restrict__ dup, int B, int H, int W, int C,
                          const uint16_t* __restrict__ gate, uint16_t* __restrict__ out) {
    const int CC = C / 8, Wf = 2 * W;
    const int n = B * H * W * CC;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int q = i % CC, p = i / CC;
        const int x = p % W, yb = p / W;
        const int src = (2 * yb) * Wf + 2 * x;
        const Bf8 a = ld8(dup + (size_t)src * C + 8 * q), c = ld8(dup + (size_t)(src + 1) * C + 8 * q),
                  d = ld8(dup + (size_t)(src + Wf) * C + 8 * q),
                  e = ld8(dup + (size_t)(src + Wf + 1) * C + 8 * q);
        const Bf8 g = ld8(gate + (size_t)i * 8);
        Bf8 r;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float s = ((a.v[j] + c.v[j]) + d.v[j]) + e.v[j];
            r.v[j] = g.v[j] > 0.0f ? s : 0.0f;
        }
        st8(out + (size_t)i * 8, r);
    }
}

// (skip + gradient of 2x2 average pooling) times (gate > 0): one thread per
// coarse pixel and chunk, writing its four fine pixels
__global__ void k_pool_back(const uint16_t* __restrict__ skip, const uint16_t* __restrict__ dq,
                            int B, int H, int W, int C, const uint16_t* __restrict__ gate,
                            uint16_t* __restrict__ out) {
    const int Hc = H / 2, Wc = W / 2, CC = C / 8;
    const int n = B * Hc * Wc * CC;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int q = i % CC, p = i / CC;
        const int x = p % Wc, yb = p / Wc;  // yb = b * Hc + y
        const Bf8 d = ld8(dq + (size_t)i * 8);
        const int base = (2 * yb) * W + 2 * x;  // (b * H + 2y) * W + 2x
        const int fine[4] = {base, base + 1, base + W, base + W + 1};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const size_t o = (size_t)fine[k] * C + 8 * q;
            const Bf8 sk = ld8(skip + o), g = ld8(gate + o);
            Bf8 r;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float s = sk.v[j] + 0.25f * d.v[j];
                r.v[j] = g.v[j] > 0.0f ? s : 0.0f;
            }
            st8(out + o, r);
        }
    }
}

// head (1x1, 16 -> 1) gradient: dWh += dp * d1, dbh += dp, dZ = dp * Wh * (d1 > 0)
__global__ void __launch_bounds__(256)
    k_head_back(const float* __restrict__ dp, const uint16_t* __restrict__ d1, int C, long n,
                const float* __restrict__ hw, float* __restrict__ dhw, float* __restrict__ dhb,
                uint16_t* __restrict__ dz) {
    __shared__ float s[16 + 1];
    if (threadIdx.x < 17) s[threadIdx.x] = 0.0f;
    __syncthreads();
    float acc[16];
    float accb = 0.0f;
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = 0.0f;
    float w[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) w[c] = hw[c];
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const float g = dp[i];
        accb += g;
        // the pixel's 16 channels: two 16-byte loads and two 16-byte stores
        const uint4* src = reinterpret_cast<const uint4*>(d1 + i * 16);
        const uint4 u0 = src[0], u1 = src[1];
        const uint32_t in[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
        uint32_t out[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float a0 = bf((uint16_t)(in[k] & 0xffffu)), a1 = bf((uint16_t)(in[k] >> 16));
            acc[2 * k] += g * a0;
            acc[2 * k + 1] += g * a1;
            const uint16_t z0 = a0 > 0.0f ? tobf(g * w[2 * k]) : (uint16_t)0;
            const uint16_t z1 = a1 > 0.0f ? tobf(g * w[2 * k + 1]) : (uint16_t)0;
            out[k] = (uint32_t)z0 | ((uint32_t)z1 << 16);
        }
        uint4* dst = reinterpret_cast<uint4*>(dz + i * 16);
        dst[0] = make_uint4(out[0], out[1], out[2], out[3]);
        dst[1] = make_uint4(out[4], out[5], out[6], out[7]);
    }
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        const float v = warp_sum_f(acc[c]);
        if ((threadIdx.x & 31) == 0) atomicAdd(&s[c], v);
    }
    const float vb = warp_sum_f(accb);
    if ((threadIdx.x & 31) == 0) atomicAdd(&s[16], vb);
    __syncthreads();
    if (threadIdx.x < 16) atomicAdd(dhw + threadIdx.x, s[threadIdx.x]);
    if (threadIdx.x == 0) atomicAdd(dhb, s[16]);
}

// -------------------------------------------------------------------- loss
// Per image b (fluid cells f, mask == 0):
//   pressure term  Lp = mean_f (e - mean_f e)^2,  e = p - target (both in the
//                  divergence-normalised units of the network)
//   residual term  Lr = sum_f r^2 / sum_f b^2,    r = b - A p (the sweep's operator)
// loss = sum_b (Lp + lambda Lr) / B.  dp is the gradient of that loss.
// Pass 1 accumulates per-image sums; pass 2 writes dp.
__device__ __forceinline__ void nbr_sub(const uint8_t* mask, int x, int y, int W, int H, int P,
                                        size_t base, bool& sl, bool& sr, bool& sb, bool& st) {
    sl = x == 0 || (mask && mask[base + (size_t)y * P + x - 1]);
    sr = x == W - 1 || (mask && mask[base + (size_t)y * P + x + 1]);
    sb = y == 0 || (mask && mask[base + (size_t)(y - 1) * P + x]);
    st = y == H - 1 || (mask && mask[base + (size_t)(y + 1) * P + x]);
}

// (A p)_c with the neighbour rule of the sweep; p dense (image stride H*W)
__device__ __forceinline__ float apply_op(const float* p, size_t pb, const uint8_t* mask,
                                          size_t mb, int x, int y, int W, int H, int P) {
    bool sl, sr, sb, st;
    nbr_sub(mask, x, y, W, H, P, mb, sl, sr, sb, st);
    const size_t c = pb + (size_t)y * W + x;
    const float pc = p[c];
    const float l = sl ? pc : p[c - 1], r = sr ? pc : p[c + 1];
    const float b = sb ? pc : p[c - W], t = st ? pc : p[c + W];
    return (((l + r) + b) + t) - 4.0f * pc;
}

__global__ void __launch_bounds__(256)
    k_loss_sums(const float* __restrict__ p, const float* __restrict__ target,
                const float* __restrict__ div, const float* __restrict__ inv_scale,
                const uint8_t* __restrict__ mask, int H, int W, int P,
                double* __restrict__ sums /* B x 6: n, se, see, srr, sbb, pad */) {
    const int b = blockIdx.y;
    const size_t pb = (size_t)b * H * W, mb = (size_t)b * H * P;
    // per-thread partial sums in FP32 over the thread's pixels (loss_blocks
    // gives each thread several), float-float across the warp, FP64 after
    float fa[5] = {0, 0, 0, 0, 0};
    const int hw = H * W;
    const float scale = inv_scale[b];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < hw; i += gridDim.x * blockDim.x) {
        const int y = i / W, x = i - y * W;
        if (mask && mask[mb + (size_t)y * P + x]) continue;
        const float e = p[pb + i] - target[pb + i];
        const float bb = div[mb + (size_t)y * P + x] * scale;
        const float r = bb - apply_op(p, pb, mask, mb, x, y, W, H, P);
        fa[0] += 1.0f;
        fa[1] += e;
        fa[2] += e * e;
        fa[3] += r * r;
        fa[4] += bb * bb;
    }
    // warp sums in float-float on the FP32 pipe (FP64 shuffles would cost
    // every thread 25 FP64 additions), lane 0 converts; then the block's sum
    // and one FP64 atomic per block and value
    __shared__ double part[8][5];
    const int warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        FF v{fa[j], 0.0f};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v = ff_add(v, FF{__shfl_down_sync(0xffffffffu, v.h, o),
                             __shfl_down_sync(0xffffffffu, v.l, o)});
        if ((threadIdx.x & 31) == 0) part[warp][j] = (double)v.h + (double)v.l;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w][threadIdx.x];
        atomicAdd(sums + b * 6 + threadIdx.x, t);
    }
}

// residual r on fluid cells (0 elsewhere), for the gradient of the residual
// term; blockIdx.y is the image
__global__ void k_loss_resid(const float* __restrict__ p, const float* __restrict__ div,
                             const float* __restrict__ inv_scale, const uint8_t* __restrict__ mask,
                             int B, int H, int W, int P, float* __restrict__ r) {
    const int b = blockIdx.y, hw = H * W;
    const size_t pb = (size_t)b * hw, mb = (size_t)b * H * P;
    const float scale = inv_scale[b];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < hw; k += gridDim.x * blockDim.x) {
        const int y = k / W, x = k - y * W;
        if (mask && mask[mb + (size_t)y * P + x]) {
            r[pb + k] = 0.0f;
            continue;
        }
        const float bb = div[mb + (size_t)y * P + x] * scale;
        r[pb + k] = bb - apply_op(p, pb, mask, mb, x, y, W, H, P);
    }
}

// dp = (2/(B n)) (e - mean e) on fluid cells  -  lambda (2/(B sbb)) A r
// (A is symmetric on the fluid cells, where r is supported)
__global__ void k_loss_grad(const float* __restrict__ p, const float* __restrict__ target,
                            const float* __restrict__ r, const uint8_t* __restrict__ mask,
                            const double* __restrict__ sums, float lambda, int B, int H, int W,
                            int P, float* __restrict__ dp) {
    // blockIdx.y is the image; its constants (FP64 divisions) once per block
    const int b = blockIdx.y, hw = H * W;
    const size_t pb = (size_t)b * hw, mb = (size_t)b * H * P;
    __shared__ float s_c[3];
    if (threadIdx.x == 0) {
        const double* s = sums + b * 6;
        const double nf = s[0] > 0 ? s[0] : 1.0;
        s_c[0] = (float)(s[1] / nf);
        s_c[1] = (float)(2.0 / (B * nf));
        s_c[2] = -lambda * (float)(2.0 / (B * (s[4] > 0 ? s[4] : 1.0)));
    }
    __syncthreads();
    const float mean_e = s_c[0], c1 = s_c[1], c2 = s_c[2];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < hw; k += gridDim.x * blockDim.x) {
        const int y = k / W, x = k - y * W;
        const size_t i = pb + k;
        if (mask && mask[mb + (size_t)y * P + x]) {
            dp[i] = 0.0f;
            continue;
        }
        const float e = p[i] - target[i] - mean_e;
        const float g1 = c1 * e;
        const float ar = apply_op(r, pb, mask, mb, x, y, W, H, P);
        const float g2 = c2 * ar;
        dp[i] = g1 + g2;
    }
}

// --------------------------------------------------------------------- adam
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, long n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / c1, vh = vi / c2;
        w[i] -= lr * mh / (sqrtf(vh) + eps);
    }
}

// ---------------------------------------------------------- FP64 CG solver
// Dense per-image vectors (stride H*W); mask pitch P (bytes per row).  The
// kernels run on a per-image grid (blockIdx.y = image) with 32-bit indices
// inside an image (H*W < 2^31), and read per-image scalars once per block.
__global__ void __launch_bounds__(256)
    k_cg_apply(const double* __restrict__ x, const uint8_t* __restrict__ mask, int H, int W,
               int P, double* __restrict__ y) {
    const int b = blockIdx.y;
    const size_t base = (size_t)b * H * W, mb = (size_t)b * H * P;
    for (int yy = blockIdx.x; yy < H; yy += gridDim.x) {
        const double* xr = x + base + (size_t)yy * W;
        double* yr = y + base + (size_t)yy * W;
        const uint8_t* mr = mask ? mask + mb + (size_t)yy * P : nullptr;
        for (int xx = threadIdx.x; xx < W; xx += blockDim.x) {
            if (mr && mr[xx]) {
                yr[xx] = 0.0;
                continue;
            }
            bool sl, sr, sb, st;
            nbr_sub(mask, xx, yy, W, H, P, mb, sl, sr, sb, st);
            // substituted neighbours read the centre itself (indices stay in the image)
            const double c = xr[xx];
            const double l = xr[sl ? xx : xx - 1], r = xr[sr ? xx : xx + 1];
            const double bo = xr[sb ? xx : xx - W], t = xr[st ? xx : xx + W];
            // negated so the operator is positive semi-definite for CG
            yr[xx] = -((((l + r) + bo) + t) - 4.0 * c);
        }
    }
}

// out[b] += sum over image b of a*c (fluid cells only when mask given)
__global__ void __launch_bounds__(256)
    k_cg_dot(const double* __restrict__ a, const double* __restrict__ c,
             const uint8_t* __restrict__ mask, int H, int W, int P, double* __restrict__ out) {
    const int b = blockIdx.y;
    const size_t base = (size_t)b * H * W, mb = (size_t)b * H * P;
    double acc = 0;
    for (int yy = blockIdx.x; yy < H; yy += gridDim.x) {
        const double* ar = a + base + (size_t)yy * W;
        const double* cr = c + base + (size_t)yy * W;
        const uint8_t* mr = mask ? mask + mb + (size_t)yy * P : nullptr;
        for (int xx = threadIdx.x; xx < W; xx += blockDim.x)
            if (!mr || !mr[xx]) acc += ar[xx] * cr[xx];
    }
    acc = warp_sum_d(acc);
    __shared__ double s[8];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < 8; ++k) t += s[k];
        atomicAdd(out + b, t);
    }
}

// y += sign * (num[b] / den[b]) * d, two elements per thread and iteration
// when `vec` (cg_vec: even image stride, 16-byte aligned vectors)
__global__ void __launch_bounds__(256)
    k_cg_axpy(double* __restrict__ y, const double* __restrict__ d,
              const double* __restrict__ num, const double* __restrict__ den, double sign,
              int per, bool vec) {
    const int b = blockIdx.y;
    __shared__ double s_a;
    if (threadIdx.x == 0) s_a = den[b] != 0.0 ? sign * (num[b] / den[b]) : 0.0;
    __syncthreads();
    const double a = s_a;
    const size_t base = (size_t)b * per;
    const int stride = gridDim.x * blockDim.x;
    if (vec) {
        double2* y2 = reinterpret_cast<double2*>(y + base);
        const double2* d2 = reinterpret_cast<const double2*>(d + base);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per / 2; i += stride) {
            double2 v = y2[i];
            const double2 w = d2[i];
            v.x += a * w.x;
            v.y += a * w.y;
            y2[i] = v;
        }
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per; i += stride)
            y[base + i] += a * d[base + i];
    }
}

// d = r + (rr_new[b] / rr_old[b]) d, two elements at a time when `vec`
__global__ void __launch_bounds__(256)
    k_cg_dir(double* __restrict__ d, const double* __restrict__ r,
             const double* __restrict__ rr_new, const double* __restrict__ rr_old, int per,
             bool vec) {
    const int b = blockIdx.y;
    __shared__ double s_beta;
    if (threadIdx.x == 0) s_beta = rr_old[b] != 0.0 ? rr_new[b] / rr_old[b] : 0.0;
    __syncthreads();
    const double beta = s_beta;
    const size_t base = (size_t)b * per;
    const int stride = gridDim.x * blockDim.x;
    if (vec) {
        double2* d2 = reinterpret_cast<double2*>(d + base);
        const double2* r2 = reinterpret_cast<const double2*>(r + base);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per / 2; i += stride) {
            double2 v = d2[i];
            const double2 w = r2[i];
            v.x = w.x + beta * v.x;
            v.y = w.y + beta * v.y;
            d2[i] = v;
        }
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per; i += stride)
            d[base + i] = r[base + i] + beta * d[base + i];
    }
}

// Block sum of one double per thread, added to out[b] by thread 0.
__device__ __forceinline__ void block_add_d(double v, double* out) {
    v = warp_sum_d(v);
    __shared__ double s[8];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < 8; ++k) t += s[k];
        atomicAdd(out, t);
    }
}

// q = -(A d) as k_cg_apply, and dq[b] += d . q over the image (q is 0 on
// obstacle cells, so the sum is over fluid cells): one pass instead of
// apply + dot.
__global__ void __launch_bounds__(256)
    k_cg_apply_dot(const double* __restrict__ d, const uint8_t* __restrict__ mask, int H, int W,
                   int P, double* __restrict__ q, double* __restrict__ dq) {
    const int b = blockIdx.y;
    const size_t base = (size_t)b * H * W, mb = (size_t)b * H * P;
    double acc = 0.0;
    for (int yy = blockIdx.x; yy < H; yy += gridDim.x) {
        const double* xr = d + base + (size_t)yy * W;
        double* yr = q + base + (size_t)yy * W;
        const uint8_t* mr = mask ? mask + mb + (size_t)yy * P : nullptr;
        for (int xx = threadIdx.x; xx < W; xx += blockDim.x) {
            if (mr && mr[xx]) {
                yr[xx] = 0.0;
                continue;
            }
            bool sl, sr, sb, st;
            nbr_sub(mask, xx, yy, W, H, P, mb, sl, sr, sb, st);
            const double c = xr[xx];
            const double l = xr[sl ? xx : xx - 1], r = xr[sr ? xx : xx + 1];
            const double bo = xr[sb ? xx : xx - W], t = xr[st ? xx : xx + W];
            const double v = -((((l + r) + bo) + t) - 4.0 * c);
            yr[xx] = v;
            acc += c * v;
        }
    }
    block_add_d(acc, dq + b);
}

// With alpha = rr[b] / dq[b]: x += alpha d, r -= alpha q, and rr_new[b] +=
// r . r (r is 0 on obstacle cells): the two axpys and the next dot in one
// pass.
__global__ void __launch_bounds__(256)
    k_cg_update(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ d,
                const double* __restrict__ q, const double* __restrict__ rr,
                const double* __restrict__ dq, double* __restrict__ rr_new, int per, bool vec) {
    const int b = blockIdx.y;
    __shared__ double s_a;
    if (threadIdx.x == 0) s_a = dq[b] != 0.0 ? rr[b] / dq[b] : 0.0;
    __syncthreads();
    const double a = s_a;
    const size_t base = (size_t)b * per;
    const int stride = gridDim.x * blockDim.x;
    double acc = 0.0;
    if (vec) {
        double2* x2 = reinterpret_cast<double2*>(x + base);
        double2* r2 = reinterpret_cast<double2*>(r + base);
        const double2* d2 = reinterpret_cast<const double2*>(d + base);
        const double2* q2 = reinterpret_cast<const double2*>(q + base);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per / 2; i += stride) {
            double2 xv = x2[i], rv = r2[i];
            const double2 dv = d2[i], qv = q2[i];
            xv.x += a * dv.x;
            xv.y += a * dv.y;
            rv.x -= a * qv.x;
            rv.y -= a * qv.y;
            x2[i] = xv;
            r2[i] = rv;
            acc += rv.x * rv.x + rv.y * rv.y;
        }
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per; i += stride) {
            x[base + i] += a * d[base + i];
            const double rv = r[base + i] - a * q[base + i];
            r[base + i] = rv;
            acc += rv * rv;
        }
    }
    block_add_d(acc, rr_new + b);
}

// Blocks per image for the CG kernels: about eight blocks of 256 threads per
// SM over the whole batch (full occupancy), at most one thread per element
// (or element pair).
int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            sms < 1)
            sms = 1;
    }
    return sms;
}

// Blocks of 256 threads per image for the loss kernels: about 32 per SM over
// the batch (a few waves of full occupancy), each thread looping over several
// pixels, at most one thread per pixel.  One pixel per thread had made the
// blocks so short that starting them (and the gradient's per-image FP64
// constants in every block) cost more than the pixels.
unsigned loss_blocks(long per, int B) {
    const long want = (32L * sm_count() + B - 1) / B;
    const long need = blocks(per, 256);
    return (unsigned)(need < want ? need : (want > 0 ? want : 1));
}

unsigned cg_blocks(long work_per_image, int B) {
    const int sms = sm_count();
    const long per_image = (8L * sms + B - 1) / B;
    const long need = blocks(work_per_image, 256);
    return (unsigned)(need < per_image ? need : per_image);
}

// Blocks per image for the row loops of apply and dot: at most one per row.
unsigned cg_rows(int H, int B) {
    const unsigned n = cg_blocks(1L << 30, B);
    return n < (unsigned)H ? n : (unsigned)H;
}

// Whether two-element (16-byte) accesses are valid: even image stride and
// 16-byte aligned vectors.
bool cg_vec(long per, const void* a, const void* b) {
    return (per & 1) == 0 && (((uintptr_t)a | (uintptr_t)b) & 15) == 0;
}

// The per-image grid holds up to 65535 images; indices inside an image are 32-bit.
int cg_range(long B, long per) {
    if (B > 65535 || per >= (1L << 31))
        return set_last_error(NATRIX_ERANGE, "CG: more than 65535 images or 2^31 cells per image");
    return NATRIX_OK;
}

}  // namespace

// ---------------------------------------------------------------- launchers
int launch_status() {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NATRIX_OK : set_last_error(NATRIX_ECUDA, cudaGetErrorString(e));
}

}  // namespace natrix

using namespace natrix;

extern "C" {

int natrix_nn_pack(const float* w, int32_t cout, int32_t cin, int32_t rows, int32_t kc,
                   int32_t dgrad, uint16_t* out, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const long total = (long)rows * 9 * kc;
    k_pack<<<blocks(total, 256) < 4096 ? blocks(total, 256) : 4096, 256, 0, st>>>(
        w, cout, cin, rows, kc, dgrad, out);
    return launch_status();
}

int natrix_nn_wgrad(const uint16_t* dz, int32_t cout, const uint16_t* x0, int32_t c0,
                    const uint16_t* x1, int32_t c1, int32_t B, int32_t H, int32_t W, float* dw,
                    float* db, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const long npix = (long)B * H * W;
    if (cout % 8 || c0 % 8 || c1 % 8 || (c1 && !x1) || npix >= (1L << 31))
        return set_last_error(NATRIX_EINVAL, "wgrad: channels must be multiples of 8, "
                                             "fewer than 2^31 pixels");
    if (c0 + c1 <= 128 && cout % 16 == 0 && cout <= 128 && getenv("NATRIX_WGRAD_CUDA_CORES") == nullptr)
        return wgrad_tc(dz, cout, x0, c0, x1, c1, B, H, W, dw, db, st);
    int slices = (int)((npix + 4095) / 4096);
    slices = slices < 1 ? 1 : (slices > 256 ? 256 : slices);
    const size_t smem = (size_t)WG_PIX * (cout + c0 + c1) * sizeof(float);
    k_wgrad<<<dim3(9, slices), 256, smem, st>>>(dz, cout, x0, c0, x1, c1, B, H, W, dw, db);
    return launch_status();
}

int natrix_nn_prep(const float* div, const uint8_t* mask, const float* inv_scale, int32_t B,
                   int32_t H, int32_t W, int32_t pitch, uint16_t* x, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const long n = (long)B * H * W;
    k_prep<<<blocks(n, 256) < 8192 ? blocks(n, 256) : 8192, 256, 0, st>>>(div, mask, inv_scale, B,
                                                                          H, W, pitch, x);
    return launch_status();
}

int natrix_nn_pool(const uint16_t* in, int32_t B, int32_t H, int32_t W, int32_t C, uint16_t* out,
                   void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (C % 8 || H % 2 || W % 2) return set_last_error(NATRIX_EINVAL, "pool: C % 8, H, W even");
    const long n = (long)B * (H / 2) * (W / 2) * (C / 8);
    k_pool<<<blocks(n, 256) < 8192 ? blocks(n, 256) : 8192, 256, 0, st>>>(in, B, H, W, C, out);
    return launch_status();
}

int natrix_nn_up(const uint16_t* in, int32_t B, int32_t H, int32_t W, int32_t C, uint16_t* out,
                 void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (C % 8) return set_last_error(NATRIX_EINVAL, "up: C must be a multiple of 8");
    const long n = (long)B * H * W * (C / 8);
    k_up<<<blocks(n, 256) < 8192 ? blocks(n, 256) : 8192, 256, 0, st>>>(in, B, H, W, C, out);
    return launch_status();
}

int natrix_nn_up_back(const uint16_t* dup, int32_t B, int32_t H, int32_t W, int32_t C,
                      const uint16_t* gate, uint16_t* out, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (C % 8) return set_last_error(NATRIX_EINVAL, "up_back: C must be a multiple of 8");
    const long n = (long)B * H * W * (C / 8);
    k_up_back<<<blocks(n, 256) < 8192 ? blocks(n, 256) : 8192, 256, 0, st>>>(dup, B, H, W, C,
                                                                            gate, out);
    return launch_status();
}

int natrix_nn_pool_back(const uint16_t* skip, const uint16_t* dq, int32_t B, int32_t H, int32_t W,
                        int32_t C, const uint16_t* gate, uint16_t* out, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (C % 8 || H % 2 || W % 2) return set_last_error(NATRIX_EINVAL, "pool_back: C % 8, H, W even");
    const long n = (long)B * (H / 2) * (W / 2) * (C / 8);
    k_pool_back<<<blocks(n, 256) < 8192 ? blocks(n, 256) : 8192, 256, 0, st>>>(skip, dq, B, H, W,
                                                                              C, gate, out);
    return launch_status();
}

int natrix_nn_head_back(const float* dp, const uint16_t* d1, int32_t C, int64_t n,
                        const float* hw, float* dhw, float* dhb, uint16_t* dz, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (C != 16) return set_last_error(NATRIX_EINVAL, "head: 16 channels expected");
    k_head_back<<<blocks(n, 256) < 2048 ? blocks(n, 256) : 2048, 256, 0, st>>>(dp, d1, C, n, hw,
                                                                              dhw, dhb, dz);
    return launch_status();
}

int natrix_nn_loss(const float* p, const float* target, const float* div, const float* inv_scale,
                   const uint8_t* mask, int32_t B, int32_t H, int32_t W, int32_t P, float lambda,
                   double* sums, float* r, float* dp, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(sums, 0, (size_t)B * 6 * sizeof(double), st) != cudaSuccess)
        return launch_status();
    const long per = (long)H * W;
    const unsigned gx = loss_blocks(per, B);
    k_loss_sums<<<dim3(gx, B), 256, 0, st>>>(p, target, div, inv_scale, mask, H, W, P, sums);
    if (dp) {
        k_loss_resid<<<dim3(gx, B), 256, 0, st>>>(p, div, inv_scale, mask, B, H, W, P, r);
        k_loss_grad<<<dim3(gx, B), 256, 0, st>>>(p, target, r, mask, sums, lambda, B, H, W, P, dp);
    }
    return launch_status();
}

int natrix_nn_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1,
                   float b2, float eps, int32_t step, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_adam<<<blocks(n, 256) < 4096 ? blocks(n, 256) : 4096, 256, 0, st>>>(w, g, m, v, n, lr, b1, b2,
                                                                          eps, c1, c2);
    return launch_status();
}

int natrix_nn_cg_apply(const double* x, const uint8_t* mask, int32_t B, int32_t H, int32_t W,
                       int32_t P, double* y, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (B < 1) return NATRIX_OK;
    if (int rc = cg_range(B, (long)H * W)) return rc;
    k_cg_apply<<<dim3(cg_rows(H, B), B), 256, 0, st>>>(x, mask, H, W, P, y);
    return launch_status();
}

int natrix_nn_cg_dot(const double* a, const double* c, const uint8_t* mask, int32_t B, int32_t H,
                     int32_t W, int32_t P, double* out, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (B < 1) return NATRIX_OK;
    if (int rc = cg_range(B, (long)H * W)) return rc;
    if (cudaMemsetAsync(out, 0, (size_t)B * sizeof(double), st) != cudaSuccess)
        return launch_status();
    k_cg_dot<<<dim3(cg_rows(H, B), B), 256, 0, st>>>(a, c, mask, H, W, P, out);
    return launch_status();
}

int natrix_nn_cg_axpy(double* y, const double* d, const double* num, const double* den,
                      double sign, int32_t B, int64_t per, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (B < 1 || per < 1) return NATRIX_OK;
    if (int rc = cg_range(B, per)) return rc;
    const bool vec = cg_vec(per, y, d);
    k_cg_axpy<<<dim3(cg_blocks(vec ? per / 2 : per, B), B), 256, 0, st>>>(y, d, num, den, sign,
                                                                           (int)per, vec);
    return launch_status();
}

int natrix_nn_cg_dir(double* d, const double* r, const double* rr_new, const double* rr_old,
                     int32_t B, int64_t per, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (B < 1 || per < 1) return NATRIX_OK;
    if (int rc = cg_range(B, per)) return rc;
    const bool vec = cg_vec(per, d, r);
    k_cg_dir<<<dim3(cg_blocks(vec ? per / 2 : per, B), B), 256, 0, st>>>(d, r, rr_new, rr_old,
                                                                          (int)per, vec);
    return launch_status();
}

int natrix_nn_cg_apply_dot(const double* d, const uint8_t* mask, int32_t B, int32_t H, int32_t W,
                           int32_t P, double* q, double* dq, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (B < 1) return NATRIX_OK;
    if (int rc = cg_range(B, (long)H * W)) return rc;
    if (cudaMemsetAsync(dq, 0, (size_t)B * sizeof(double), st) != cudaSuccess)
        return launch_status();
    k_cg_apply_dot<<<dim3(cg_rows(H, B), B), 256, 0, st>>>(d, mask, H, W, P, q, dq);
    return launch_status();
}

int natrix_nn_cg_update(double* x, double* r, const double* d, const double* q, const double* rr,
                        const double* dq, double* rr_new, int32_t B, int64_t per, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (B < 1 || per < 1) return NATRIX_OK;
    if (int rc = cg_range(B, per)) return rc;
    if (cudaMemsetAsync(rr_new, 0, (size_t)B * sizeof(double), st) != cudaSuccess)
        return launch_status();
    const bool vec = cg_vec(per, x, r) && cg_vec(per, d, q);
    k_cg_update<<<dim3(cg_blocks(vec ? per / 2 : per, B), B), 256, 0, st>>>(
        x, r, d, q, rr, dq, rr_new, (int)per, vec);
    return launch_status();
}

}  // extern "C"
