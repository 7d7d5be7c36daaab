/* natrix_gb300 — C ABI of the learned pressure warm start (U-Net) kernels.
 *
 * No reference counterpart: natrix starts every pressure solve from zero
 * (natrix/core/fluid_simulator.py:235-248).  These entry points are the
 * building blocks the Python warm-start model (natrix_gb300/core/warmstart.py)
 * drives: tensor-core convolutions, their gradients, pooling / upsampling,
 * loss, Adam, and an FP64 conjugate-gradient solver for training targets.
 *
 * All pointers are device pointers; activations are NHWC bf16 (uint16_t
 * storage), parameters and their gradients FP32.  `stream` is a cudaStream_t
 * passed as void*.  Every function returns 0 or a negative NATRIX_E* code
 * (message in natrix_last_error()).
 */
#ifndef NATRIX_GB300_NATRIX_NN_H
#define NATRIX_GB300_NATRIX_NN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One 3x3 convolution (stride 1, zero padding 1) as an implicit GEMM on the
 * tensor cores (tcgen05, BF16 x BF16 -> FP32 in TMEM).  Input channels are
 * the concatenation of src0 (c0 channels) and src1 (c1 channels, may be 0);
 * both multiples of 8.  Output channels N: multiple of 16, at most 128.
 * Epilogue, in order: + bias, ReLU, times (gate > 0) (gate: NHWC bf16 with N
 * channels), optional 1x1 head (head_out[p] = head_b + sum_c head_w[c] y[c]);
 * channels [0, n0) go to out0 and [n0, N) to out1 (out1 NULL: all to out0;
 * a NULL output is not written). */
typedef struct natrix_nn_conv {
    const uint16_t* src0;
    int32_t c0;
    const uint16_t* src1;
    int32_t c1;
    int32_t B, H, W, N;
    const uint16_t* wpack; /* natrix_nn_pack output for this layer */
    const float* bias;
    int32_t relu;
    const uint16_t* gate;
    uint16_t* out0;
    int32_t n0;
    uint16_t* out1;
    const float* head_w;
    float head_b;
    float* head_out;
    int32_t* status; /* bit 2 set if a bounded wait ran out */
} natrix_nn_conv;

int natrix_nn_conv3x3(const natrix_nn_conv* conv, void* stream);

/* Pack FP32 weights w[cout][cin][3][3] into the bf16 operand layout the
 * convolution reads: forward (dgrad = 0: rows = cout padded to `rows`, K =
 * 9 x kc with kc = cin padded) or input-gradient (dgrad = 1: rows = cin
 * padded, kc = cout, taps flipped).  `out` holds rows * 9 * kc bf16. */
int natrix_nn_pack(const float* w, int32_t cout, int32_t cin, int32_t rows, int32_t kc,
                   int32_t dgrad, uint16_t* out, void* stream);

/* Weight and bias gradients of a 3x3 convolution, accumulated (+=) into
 * dw[cout][cin][3][3] and db[cout] (db may be NULL):
 * dw[co][ci][t] += sum_p dz[p][co] * x[p + offset(t)][ci], x = [x0, x1].
 * Channel counts are multiples of 8; with cin <= 128 and cout a multiple of
 * 16 up to 128 the sums run on the tensor cores (one FP32 partial per block,
 * added atomically), otherwise on the CUDA cores. */
int natrix_nn_wgrad(const uint16_t* dz, int32_t cout, const uint16_t* x0, int32_t c0,
                    const uint16_t* x1, int32_t c1, int32_t B, int32_t H, int32_t W, float* dw,
                    float* db, void* stream);

/* Status word of the weight-gradient kernels (bit 2 set if a bounded wait
 * ran out); read and cleared.  Synchronous. */
int natrix_nn_wgrad_status(int32_t* out);

/* Network input: x[p] = {div[p] * inv_scale[b], obstacle[p], 0 x 6} as
 * 8-channel NHWC bf16 from B pitched float / uint8 fields (mask may be NULL). */
int natrix_nn_prep(const float* div, const uint8_t* mask, const float* inv_scale, int32_t B,
                   int32_t H, int32_t W, int32_t pitch, uint16_t* x, void* stream);

/* 2x2 average pooling (H, W even) and nearest x2 upsampling, and gradients:
 * up_back: out = (sum of the 4 children of dup) * (gate > 0);
 * pool_back: out = (skip + dq[parent] / 4) * (gate > 0). */
int natrix_nn_pool(const uint16_t* in, int32_t B, int32_t H, int32_t W, int32_t C, uint16_t* out,
                   void* stream);
int natrix_nn_up(const uint16_t* in, int32_t B, int32_t H, int32_t W, int32_t C, uint16_t* out,
                 void* stream);
int natrix_nn_up_back(const uint16_t* dup, int32_t B, int32_t H, int32_t W, int32_t C,
                      const uint16_t* gate, uint16_t* out, void* stream);
int natrix_nn_pool_back(const uint16_t* skip, const uint16_t* dq, int32_t B, int32_t H, int32_t W,
                        int32_t C, const uint16_t* gate, uint16_t* out, void* stream);

/* 1x1 head (C = 16 -> 1) gradients: dhw += sum dp * d1, dhb += sum dp,
 * dz = dp * hw * (d1 > 0). */
int natrix_nn_head_back(const float* dp, const uint16_t* d1, int32_t C, int64_t n,
                        const float* hw, float* dhw, float* dhb, uint16_t* dz, void* stream);

/* Loss of B predictions p (dense B x H x W) against targets, in the
 * divergence-normalised units: per image, mean over fluid cells of the
 * squared mean-removed pressure error plus lambda times the squared residual
 * of the sweep's operator relative to the squared right-hand side.  sums
 * receives B x 6 doubles {n, sum e, sum e^2, sum r^2, sum b^2, 0}; when dp
 * is not NULL, r (scratch, B x H x W) and the gradient dp are written. */
int natrix_nn_loss(const float* p, const float* target, const float* div, const float* inv_scale,
                   const uint8_t* mask, int32_t B, int32_t H, int32_t W, int32_t pitch,
                   float lambda, double* sums, float* r, float* dp, void* stream);

/* Adam update of n FP32 parameters (step counts from 1). */
int natrix_nn_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1,
                   float b2, float eps, int32_t step, void* stream);

/* FP64 conjugate-gradient building blocks for B independent pressure systems
 * (dense vectors of H x W per image, mask rows of `pitch` bytes):
 * apply: y = -(A x) on fluid cells (0 on obstacles), A the sweep's operator;
 * dot: out[b] = sum over fluid cells of a*c (out zeroed first);
 * axpy: y += sign * (num[b] / den[b]) * d;  dir: d = r + (rr_new[b] / rr_old[b]) d.
 * B up to 65535 and H x W (per) below 2^31, else NATRIX_ERANGE. */
int natrix_nn_cg_apply(const double* x, const uint8_t* mask, int32_t B, int32_t H, int32_t W,
                       int32_t pitch, double* y, void* stream);
int natrix_nn_cg_dot(const double* a, const double* c, const uint8_t* mask, int32_t B, int32_t H,
                     int32_t W, int32_t pitch, double* out, void* stream);
int natrix_nn_cg_axpy(double* y, const double* d, const double* num, const double* den,
                      double sign, int32_t B, int64_t per, void* stream);
int natrix_nn_cg_dir(double* d, const double* r, const double* rr_new, const double* rr_old,
                     int32_t B, int64_t per, void* stream);
/* Fused steps of one CG iteration (the same arithmetic as the calls they
 * replace, fewer passes over memory):
 * apply_dot: q = -(A d) as natrix_nn_cg_apply, and dq[b] = d . q (dq zeroed
 * first; q is 0 on obstacle cells);
 * update: with alpha = rr[b] / dq[b] (0 when dq[b] is 0), x += alpha d,
 * r -= alpha q, and rr_new[b] = r . r (zeroed first).  Same limits. */
int natrix_nn_cg_apply_dot(const double* d, const uint8_t* mask, int32_t B, int32_t H, int32_t W,
                           int32_t pitch, double* q, double* dq, void* stream);
int natrix_nn_cg_update(double* x, double* r, const double* d, const double* q, const double* rr,
                        const double* dq, double* rr_new, int32_t B, int64_t per, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NATRIX_GB300_NATRIX_NN_H */
