// Device-side helpers shared by the solver kernels.
//
// Arithmetic contract: the solver translation units are compiled with
// -fmad=false and IEEE division / square root (nvcc's defaults
// -prec-div=true -prec-sqrt=true), so each + - * / and sqrtf below rounds
// once, in the order written.  The order follows the reference shader text
// (natrix/core/shaders/originals/*.comp), which makes the FP32 results equal,
// bit for bit, to the oracle's float instantiation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace natrix {

// 2-D field geometry: width, height and row pitch in elements.
struct Grid {
    int W, H, P;
};

__device__ __forceinline__ float clampf(float v, float lo, float hi) {
    // GLSL clamp = min(max(x, lo), hi), in the form the oracle uses
    float m = v > lo ? v : lo;
    return m < hi ? m : hi;
}

// GLSL mix, HLSL lerp form: a + t*(b - a)
__device__ __forceinline__ float mixf(float a, float b, float t) { return a + t * (b - a); }

// Bilinear sampler of shader.AdvectVelocity.comp:38-48 (and GetVelocity in
// demo/shaders/shader.AdvectParticle.comp:21-35): corners from ceil/floor of
// the sample position clamped to the grid, the fractional delta NOT clamped
// (so positions outside the grid extrapolate linearly, as the reference does).
struct Corners {
    int lo_x, lo_y, hi_x, hi_y;
    float dx, dy;
};

// The reference clamps ceil / floor in float, then converts.  Rounding and
// converting in one instruction (cvt.rpi / cvt.rmi: saturating, NaN -> 0),
// then clamping the integer, gives the same index for every input: finite
// values round to the same integer, +-inf and out-of-range values saturate
// to the same edge, NaN becomes 0 as the float clamp makes it.
__device__ __forceinline__ int clamp_index(int v, int hi) { return min(max(v, 0), hi); }

__device__ __forceinline__ Corners corners(float fx, float fy, int W, int H) {
    Corners c;
    c.hi_x = clamp_index(__float2int_ru(fx), W - 1);
    c.hi_y = clamp_index(__float2int_ru(fy), H - 1);
    c.lo_x = clamp_index(__float2int_rd(fx), W - 1);
    c.lo_y = clamp_index(__float2int_rd(fy), H - 1);
    c.dx = fx - (float)c.lo_x;
    c.dy = fy - (float)c.lo_y;
    return c;
}

// Loads of solver fields.  A kernel that only reads a field during its
// launch takes the read-only path (ld.global.nc, CG = false); the batch step
// kernel, whose phases read fields that other CTAs wrote earlier in the same
// launch, reads through L2 (ld.global.cg, CG = true), which is coherent
// across SMs.
template <bool CG, class T>
__device__ __forceinline__ T ldf(const T* p) {
    if constexpr (CG)
        return __ldcg(p);
    else
        return __ldg(p);
}

// A plain load (CG = false) or an L2 load (CG = true): for the reads the
// per-phase kernels issue as ordinary loads.
template <bool CG, class T>
__device__ __forceinline__ T ldp(const T* p) {
    if constexpr (CG)
        return __ldcg(p);
    else
        return *p;
}

template <bool CG = false>
__device__ __forceinline__ float2 sample_vel(const float2* __restrict__ v, int P,
                                             const Corners& c) {
    // 32-bit cell offsets (grids stay below 2^31 cells)
    const int rh = c.hi_y * P, rl = c.lo_y * P;
    const float2 lt = ldf<CG>(v + (rh + c.lo_x));
    const float2 rt = ldf<CG>(v + (rh + c.hi_x));
    const float2 lb = ldf<CG>(v + (rl + c.lo_x));
    const float2 rb = ldf<CG>(v + (rl + c.hi_x));
    const float h1x = mixf(lt.x, rt.x, c.dx), h1y = mixf(lt.y, rt.y, c.dx);
    const float h2x = mixf(lb.x, rb.x, c.dx), h2y = mixf(lb.y, rb.y, c.dx);
    return make_float2(mixf(h2x, h1x, c.dy), mixf(h2y, h1y, c.dy));
}

template <bool CG = false>
__device__ __forceinline__ float sample_scalar(const float* __restrict__ s, int P,
                                               const Corners& c) {
    // 32-bit cell offsets (grids stay below 2^31 cells)
    const int rh = c.hi_y * P, rl = c.lo_y * P;
    const float lt = ldf<CG>(s + (rh + c.lo_x));
    const float rt = ldf<CG>(s + (rh + c.hi_x));
    const float lb = ldf<CG>(s + (rl + c.lo_x));
    const float rb = ldf<CG>(s + (rl + c.hi_x));
    const float h1 = mixf(lt, rt, c.dx);
    const float h2 = mixf(lb, rb, c.dx);
    return mixf(h2, h1, c.dy);
}

// exp for the Gaussian splat weight: Cody-Waite reduction x = k ln2 + r with
// ln2 = 0.693359375 - 2.12194440e-4 (k*C1 exact), degree-7 Taylor polynomial
// of exp(r) in Horner form, exact scaling by 2^k.  The oracle evaluates the
// same sequence, so the weights agree bit for bit.
__device__ __forceinline__ float nx_expf(float x) {
    x = x < -87.0f ? -87.0f : x;
    x = x > 88.0f ? 88.0f : x;
    const float kf = floorf(x * 1.44269502f + 0.5f);
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
    return ldexpf(p, (int)kf);
}

// Neighbour-substitution flags, one byte per cell, written by the divergence
// kernel and read by the Jacobi sweeps, the gradient subtraction and the
// residual.  Bit set <=> that neighbour's pressure is replaced by the centre
// pressure: the neighbour is an obstacle (shader.Poisson.comp:32-35) or lies
// beyond a wall, where the clamped index of common.sh:9-19 is the cell itself.
enum : uint8_t { NB_L = 1, NB_R = 2, NB_B = 4, NB_T = 8 };

// ------------------------------------------------------ residual arithmetic
// The residual of the pressure equation at a fluid cell, r = b - ((x1 + x2 +
// y1 + y2) - 4 pc) with the sweep's neighbour substitution, and the sums
// {n, r, r^2, b, b^2} a thread keeps over its cells.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, and plain FP32 would
// lose r to cancellation (near convergence r is tiny next to the pressures),
// so the arithmetic runs on the FP32 pipe in float-float form (a value is the
// unevaluated sum hi + lo of two floats):
//   * r is the compensated sum of the six terms b, -x1, -x2, -y1, -y2, 4 pc
//     (Ogita, Rump and Oishi's Sum2: a cascade of Knuth's TwoSum with the
//     rounding errors summed apart), kept as a pair; its error is below
//     about 1e-13 times the sum of the terms' magnitudes;
//   * squares are split exactly with a fused multiply-add (TwoProd);
//   * running sums add pairs with Dekker's add2 (TwoSum of the high parts,
//     low parts added, then renormalised).
// Warps sum their threads' pairs the same way; lane 0 converts the warp's
// pairs to FP64 once, for the block and grid sums.
struct FF {
    float h, l;
};

__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = a * b;
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const FF s = two_sum(a.h, b.h);
    const float e = s.l + (a.l + b.l);
    const float h = s.h + e;
    return {h, e - (h - s.h)};
}

struct ResidSums {
    int n = 0;
    FF r{0.0f, 0.0f}, rr{0.0f, 0.0f}, b{0.0f, 0.0f}, bb{0.0f, 0.0f};

    __device__ __forceinline__ void add(float bv, float pc, float x1, float x2, float y1,
                                        float y2) {
        FF t = two_sum(bv, -x1);
        float c = t.l;
        t = two_sum(t.h, -x2);
        c += t.l;
        t = two_sum(t.h, -y1);
        c += t.l;
        t = two_sum(t.h, -y2);
        c += t.l;
        t = two_sum(t.h, 4.0f * pc);
        c += t.l;
        const FF rv = two_sum(t.h, c);
        n += 1;
        r = ff_add(r, rv);
        FF sq = two_prod(rv.h, rv.h);
        sq.l += 2.0f * rv.h * rv.l;
        rr = ff_add(rr, sq);
        b = ff_add(b, FF{bv, 0.0f});
        bb = ff_add(bb, two_prod(bv, bv));
    }

    // Sum over the warp into lane 0, in float-float on the FP32 pipe (a
    // warp sum in FP64 would cost each thread 25 FP64 additions).
    __device__ __forceinline__ void warp_sum() {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            n += __shfl_down_sync(0xffffffffu, n, o);
            r = ff_add(r, shfl_down(r, o));
            rr = ff_add(rr, shfl_down(rr, o));
            b = ff_add(b, shfl_down(b, o));
            bb = ff_add(bb, shfl_down(bb, o));
        }
    }

    __device__ __forceinline__ static FF shfl_down(FF v, int o) {
        return {__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)};
    }

    __device__ __forceinline__ void to_double(double out[5]) const {
        out[0] = (double)n;
        out[1] = (double)r.h + (double)r.l;
        out[2] = (double)rr.h + (double)rr.l;
        out[3] = (double)b.h + (double)b.l;
        out[4] = (double)bb.h + (double)bb.l;
    }
};

// (x, y) of a linear cell index that advances by a fixed stride: one
// division when it starts, then an add and a compare per step while rows are
// at least a stride wide.
struct CellWalk {
    int x, y;
    __device__ __forceinline__ CellWalk(int lin, int W) {
        y = lin / W;
        x = lin - y * W;
    }
    __device__ __forceinline__ void advance(int stride, int W) {
        x += stride;
        if (x >= W) {
            if (W >= stride) {
                x -= W;
                ++y;
            } else {
                y += x / W;
                x %= W;
            }
        }
    }
};

// Programmatic dependent launch.  The kernels of the single-grid step are
// launched with programmatic stream serialisation, so a launch is scheduled
// while its predecessor on the stream drains instead of after it has retired.
// Every block calls pdl_enter() before anything else: it allows the next
// launch to be scheduled, then waits until the predecessor grid has completed
// and its writes are visible.  (The next launch cannot get ahead either: its
// own pdl_enter() waits for this grid, which finishes only after this wait.)
// In a kernel launched without the attribute both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// The two halves, for kernels that order them the other way round: a grid
// that triggers only after its own wait lets its successor start only once
// the grid before it has completed.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Whether step launches use programmatic dependent launch (on unless the
// environment sets NATRIX_PDL=0).
bool pdl_enabled();

// Launch `kernel` on `st`, with programmatic stream serialisation if `pdl`.
template <typename... KArgs, typename... Args>
cudaError_t launch_kernel(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                          cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace natrix
