// 3x3 convolutions (stride 1, zero padding 1) of NHWC bf16 activations as
// implicit GEMMs on the 5th-generation tensor cores: BF16 operands, FP32
// accumulation in TMEM.  Used by the U-Net warm start for the forward pass
// and, with flipped and transposed weights, for the input gradient.
//
// GEMM view: D[pixel, n] = sum over taps t and input channels c of
//     X[pixel + offset(t), c] * Wp[n, t, c]
// M = 128 pixels of one image row, N = output channels, K = 9 * C.
//
// One persistent CTA per SM, eleven warps, walking "segments": S consecutive
// output rows of one 128-pixel column strip of one image.  A segment's input
// rows stream through a ring of R stages of G rows each (G = 4, 2 or 1, as
// shared memory and TMEM allow); every input row is loaded once and serves
// the three output rows it touches, and the three horizontal taps of a row
// read the same staged row at byte offsets 0, 16 and 32 (one pixel = 16
// bytes of an 8-channel chunk; SWIZZLE_NONE rows are 16-byte granular).
// Work moves in steps of G output rows, so every barrier operation is shared
// by G rows: the single threads that issue TMA and MMA are latency-bound,
// and their per-row cost is what limits small-channel layers.
//   warp 0 lane 0  TMA producer: per stage, one 4-D box {8 channels, 136 px
//                  from x0 - 1, G rows} per 8-channel chunk (out-of-image
//                  pixels, rows and channels read as zero, which is the
//                  padding);
//   warp 1 lane 0 and warp 10 lane 0  MMA issuers: per step, G output rows
//                  (split between the two when G >= 2) x 9 taps x C/16
//                  tcgen05.mma (K = 16 each) into the step's accumulator
//                  slot (G accumulators of N columns; 2 to 4 slots in TMEM);
//                  descriptors are precomputed bases plus offsets;
//                  tcgen05.commit hands the slot to the epilogue and frees the
//                  stage no later step reads;
//   warps 2-9      epilogue, two groups of four warps taking alternate steps:
//                  tcgen05.ld of their 32-lane quarter, bias, ReLU or
//                  ReLU-gate, optional 1x1 head, bf16 NHWC stores.
// The weights (packed once per layer in the operand layout) are copied to
// shared memory once per CTA with cp.async.bulk.
//
// Operand layout (SWIZZLE_NONE K-major, see umma.cuh): a stage holds, per
// 8-channel chunk, G rows of 136 pixels x 16 bytes ([chunk][row][pixel]), so
// core matrices along M are 128 bytes apart (SBO) and chunks along K are
// G * 2176 bytes apart (LBO).  The packed weights use LBO = N/8 * 128,
// SBO = 128 with K chunks ordered (tap, channel chunk).
//
// Every wait is bounded; a role that gives up records status bit 2 and
// leaves its loop, the others then time out too, and the allocating warp
// frees TMEM before the CTA exits.
#include <cudaTypedefs.h>

#include <cstdio>

#include "../../include/natrix.h"
#include "../../include/natrix_nn.h"
#include "kernels.cuh"
#include "umma.cuh"

namespace natrix {

namespace {

constexpr int kMaxStages = 32;
constexpr int kMaxSlots = 4;     // TMEM accumulator slots (steps in flight past the MMA)
constexpr int kEpiGroups = 2;    // epilogue groups of 4 warps
constexpr int kIssuer2Warp = 2 + 4 * kEpiGroups;  // the second MMA issuer
constexpr int kThreads = 32 * (3 + 4 * kEpiGroups);
constexpr int kTileM = 128;
constexpr int kBoxW = 136;                   // pixels per box: x0 - 1 .. x0 + 128, padded
constexpr int kChunkBytes = 8 * kBoxW * 2;   // one 8-channel row: 2176 B

struct ConvParams {
    int B, H, W;
    int c0, c1;      // channels of source 0 / source 1 (multiples of 8; c1 may be 0)
    int ctot;        // c0 + c1 rounded up to a multiple of 16 (zero chunks read as padding)
    int N;           // output channels (multiple of 16, <= 128)
    const uint16_t* wpack;  // packed bf16 weights, N x 9*ctot, operand layout
    const float* bias;      // N or null
    int relu;               // 1: ReLU on the output
    const uint16_t* gate;   // NHWC bf16 with `N` channels or null: out *= (gate > 0)
    uint16_t* out0;         // NHWC bf16, channels [0, n0), or null
    int n0;
    uint16_t* out1;         // NHWC bf16, channels [n0, N), or null
    const float* head_w;    // N weights of a 1x1 head, or null
    float head_b;
    float* head_out;        // B*H*W floats, or null
    int* status;
    int tiles_x;            // 128-pixel column strips per row
    int seg_rows, n_segs;   // output rows per segment, segments per strip
    int n_units;            // B * tiles_x * n_segs
    int G;                  // output rows per step = input rows per stage (1, 2, 4)
    int stages;             // stage ring depth
    int n_slots;            // TMEM accumulator slots of G x N columns
    uint32_t stage_bytes;   // chunks x G x kChunkBytes
    uint32_t smem_w, smem_a;  // byte offsets in dynamic shared memory
    uint32_t tmem_cols;
};

struct Unit {
    int b, tx, y0, rows;
};

__device__ __forceinline__ Unit unit_of(const ConvParams& P, int u) {
    Unit r;
    r.tx = u % P.tiles_x;
    const int rest = u / P.tiles_x;
    const int seg = rest % P.n_segs;
    r.b = rest / P.n_segs;
    r.y0 = seg * P.seg_rows;
    r.rows = min(P.seg_rows, P.H - r.y0);
    return r;
}

__device__ __forceinline__ float bf16_to_f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

__device__ __forceinline__ uint16_t f_to_bf16(float f) {
    // round to nearest even
    uint32_t u = __float_as_uint(f);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// Ring position: index into a ring of n entries plus the parity of the
// pass over the ring; advanced by one entry without any division.
struct RingPos {
    uint32_t i = 0, ph = 0;
    __device__ __forceinline__ void next(uint32_t n) {
        if (++i == n) {
            i = 0;
            ph ^= 1u;
        }
    }
};

// One issuer's share of a step's MMAs: output rows [RB, RB + RC) of the G,
// x 9 taps x PAIRS (16-channel K slices), fully unrolled so every descriptor
// is a base plus a compile-time offset.  Rows past the segment's end are
// computed too (their input rows are staged and their accumulators exist);
// the epilogue does not store them.
template <int G, int RB, int RC, int PAIRS>
__device__ __forceinline__ void issue_step(uint32_t d0, uint32_t n_cols, const uint32_t* soff,
                                           uint64_t a_base, uint64_t b_base, uint32_t a_pair,
                                           uint32_t b_pair, uint32_t b_tap, uint32_t idesc) {
    constexpr uint32_t kRow16 = kChunkBytes >> 4;
#pragma unroll
    for (int r = RB; r < RB + RC; ++r) {
        const uint32_t d = d0 + (uint32_t)r * n_cols;
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            const uint64_t arow = a_base + soff[(r + dy) / G] + (uint32_t)((r + dy) % G) * kRow16;
#pragma unroll
            for (int dx = 0; dx < 3; ++dx) {
                const int tap = dy * 3 + dx;
#pragma unroll
                for (int m = 0; m < PAIRS; ++m)
                    umma::mma_bf16(d, arow + (uint32_t)dx + (uint32_t)m * a_pair,
                                   b_base + (uint32_t)tap * b_tap + (uint32_t)m * b_pair, idesc,
                                   (tap > 0 || m > 0) ? 1u : 0u);
            }
        }
    }
}

template <int G, int PAIRS>
__global__ void __launch_bounds__(kThreads, 1)
    k_conv3x3_tc(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
                 const ConvParams P) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t full[kMaxStages], empty[kMaxStages], acc_full[kMaxSlots],
        acc_empty[kMaxSlots], wbar;
    __shared__ uint32_t tmem_slot;
    // bias and 1x1-head weights, read by every epilogue thread for every
    // pixel: staged once (N <= 128)
    __shared__ __align__(16) float s_bias[128], s_head[128];
    constexpr int kLastExtra = G >= 2 ? 1 : 2;  // stages past t that step t reads
    // MMA issuers: two threads (warps 1 and kIssuer2Warp) split a step's rows
    // when G >= 2 (separate accumulators, so no ordering between them); a
    // stage is free and a slot ready after one commit from each
    constexpr int NI = G >= 2 ? 2 : 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunks = P.ctot / 8;  // 8-channel chunks per input row
    const int c0_chunks = P.c0 / 8;
    const int c1_chunks = P.c1 / 8;
    const uint32_t R = (uint32_t)P.stages;
    const uint32_t NS = (uint32_t)P.n_slots;  // 2 or 4

    if (threadIdx.x == 0) {
        for (int s = 0; s < P.stages; ++s) {
            umma::mbar_init(&full[s], 1);
            umma::mbar_init(&empty[s], NI);
        }
        for (int a = 0; a < P.n_slots; ++a) {
            umma::mbar_init(&acc_full[a], NI);
            umma::mbar_init(&acc_empty[a], 4);
        }
        umma::mbar_init(&wbar, 1);
        umma::mbar_init_fence();
    }
    if (warp == 1) umma::tmem_alloc(&tmem_slot, P.tmem_cols);
    for (int i = threadIdx.x; i < P.N; i += blockDim.x) {
        s_bias[i] = P.bias ? P.bias[i] : 0.0f;
        s_head[i] = P.head_w ? P.head_w[i] : 0.0f;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t wbytes = (uint32_t)P.N * 9u * (uint32_t)P.ctot * 2u;

    if (warp == 0 && lane == 0) {
        // weights once, then the input stages of every segment through the ring
        umma::mbar_arrive_expect_tx(&wbar, wbytes);
        for (uint32_t off = 0; off < wbytes; off += 32768u) {
            const uint32_t n = wbytes - off < 32768u ? wbytes - off : 32768u;
            umma::bulk_load(smem + P.smem_w + off, reinterpret_cast<const unsigned char*>(P.wpack) + off,
                            n, &wbar);
        }
        RingPos ps;
        bool ok = true;
        // stages armed and the parity of each one's last lap: the copies must
        // land before the CTA exits, even after a wait ran out
        uint32_t armed = 0, armed_ph = 0;
        for (int u = blockIdx.x; u < P.n_units && ok; u += gridDim.x) {
            const Unit U = unit_of(P, u);
            const int x0 = U.tx * kTileM;
            const int n_steps = (U.rows + G - 1) / G;
            const int n_stages = n_steps + kLastExtra;
            int y = U.y0 - 1;
            for (int k = 0; k < n_stages; ++k, y += G, ps.next(R)) {
                if (!umma::mbar_wait(&empty[ps.i], ps.ph ^ 1u)) {
                    ok = false;
                    break;
                }
                umma::mbar_arrive_expect_tx(&full[ps.i], P.stage_bytes);
                armed |= 1u << ps.i;
                armed_ph = (armed_ph & ~(1u << ps.i)) | (ps.ph << ps.i);
                unsigned char* d = smem + P.smem_a + ps.i * P.stage_bytes;
                for (int q = 0; q < chunks; ++q, d += G * kChunkBytes) {
                    if (q < c0_chunks || c1_chunks == 0)
                        umma::tma_load_4d(d, &tm0, 8 * q, x0 - 1, y, U.b, &full[ps.i]);
                    else
                        umma::tma_load_4d(d, &tm1, 8 * (q - c0_chunks), x0 - 1, y, U.b, &full[ps.i]);
                }
            }
        }
        if (!ok) atomicOr(P.status, 2);
        for (uint32_t i = 0; i < R; ++i)
            if ((armed >> i) & 1u) umma::mbar_wait(&full[i], (armed_ph >> i) & 1u);
    } else if ((warp == 1 || (warp == kIssuer2Warp && NI == 2)) && lane == 0) {
        const int ii = warp == 1 ? 0 : 1;  // issuer index
        bool ok = umma::mbar_wait(&wbar, 0);
        const uint32_t idesc = umma::idesc_bf16_f32(kTileM, P.N);
        const uint32_t lbo_a = (uint32_t)G * kChunkBytes;
        const uint32_t lbo_b = (uint32_t)(P.N / 8) * 128u;
        // descriptor bases; offsets (16-byte units) are added per operand
        const uint64_t a_base = umma::smem_desc(umma::smem_u32(smem + P.smem_a), lbo_a, 128);
        const uint64_t b_base = umma::smem_desc(umma::smem_u32(smem + P.smem_w), lbo_b, 128);
        const uint32_t a_pair = 2u * lbo_a >> 4;  // next 16 channels of A
        const uint32_t b_pair = 2u * lbo_b >> 4;  // next 16 channels of B
        const uint32_t b_tap = (uint32_t)chunks * lbo_b >> 4;
        const uint32_t stage16 = P.stage_bytes >> 4;
        RingPos st;    // stage of the current step t
        RingPos wt;    // next stage to wait for
        RingPos slot;  // accumulator slot of the current step
        for (int u = blockIdx.x; u < P.n_units && ok; u += gridDim.x) {
            const Unit U = unit_of(P, u);
            const int n_steps = (U.rows + G - 1) / G;
            int waited = -1;
            for (int t = 0; t < n_steps && ok; ++t, st.next(R), slot.next(NS)) {
                for (; waited < t + kLastExtra && ok; ++waited, wt.next(R))
                    ok = umma::mbar_wait(&full[wt.i], wt.ph);
                if (ok) ok = umma::mbar_wait(&acc_empty[slot.i], slot.ph ^ 1u);
                if (!ok) break;
                umma::fence_after_sync();
                // 16-byte offsets of the stages this step reads
                uint32_t soff[kLastExtra + 1];
                {
                    RingPos q = st;
#pragma unroll
                    for (int e = 0; e <= kLastExtra; ++e, q.next(R)) soff[e] = q.i * stage16;
                }
                const uint32_t d0 = tmem + slot.i * (uint32_t)G * (uint32_t)P.N;
                if (ii == 0)
                    issue_step<G, 0, G / NI, PAIRS>(d0, (uint32_t)P.N, soff, a_base, b_base,
                                                    a_pair, b_pair, b_tap, idesc);
                else
                    issue_step<G, G / NI, G / NI, PAIRS>(d0, (uint32_t)P.N, soff, a_base, b_base,
                                                         a_pair, b_pair, b_tap, idesc);
                umma::commit(&acc_full[slot.i]);
                // stage t has no later reader in this segment
                umma::commit(&empty[st.i]);
            }
            if (!ok) break;
            // the stages past the last step's own
            RingPos q = st;
            for (int e = 0; e < kLastExtra; ++e, q.next(R)) umma::commit(&empty[q.i]);
            st = q;
            wt = q;  // every stage up to here was waited for
        }
        if (!ok) atomicOr(P.status, 2);
    } else if (warp >= 2 && warp < kIssuer2Warp) {
        const int quarter = warp & 3;  // TMEM lanes this warp may read
        const int group = (warp - 2) >> 2;
        const int row = quarter * 32 + lane;
        const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
        RingPos slot;   // slot of step j
        uint32_t j = 0; // steps seen so far; this group takes j % 2 == group
        bool ok = true;
        for (int u = blockIdx.x; u < P.n_units && ok; u += gridDim.x) {
            const Unit U = unit_of(P, u);
            const int x = U.tx * kTileM + row;
            const bool inside = x < P.W;
            const int n_steps = (U.rows + G - 1) / G;
            for (int t = 0; t < n_steps; ++t, ++j, slot.next(NS)) {
                if ((int)(j & 1u) != group) continue;
                if (lane == 0) ok = umma::mbar_wait(&acc_full[slot.i], slot.ph);
                ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
                if (!ok) {
                    if (lane == 0) atomicOr(P.status, 2);
                    break;
                }
                umma::fence_after_sync();
                const int rows = min(G, U.rows - t * G);
                for (int r = 0; r < rows; ++r) {
                    const int y = U.y0 + t * G + r;
                    const size_t pix = ((size_t)U.b * P.H + y) * P.W + (inside ? x : 0);
                    const uint32_t col0 = (slot.i * (uint32_t)G + (uint32_t)r) * (uint32_t)P.N;
                    float head = P.head_b;
                    for (int c = 0; c < P.N; c += 16) {
                        float v[16];
                        umma::tmem_ld16(tmem + lane_base + col0 + (uint32_t)c, v);
                        if (!inside) continue;
                        if (P.bias) {
                            const float4* b4 = reinterpret_cast<const float4*>(s_bias + c);
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                const float4 b = b4[q];
                                v[4 * q] += b.x;
                                v[4 * q + 1] += b.y;
                                v[4 * q + 2] += b.z;
                                v[4 * q + 3] += b.w;
                            }
                        }
                        if (P.relu)
#pragma unroll
                            for (int jj = 0; jj < 16; ++jj) v[jj] = v[jj] > 0.0f ? v[jj] : 0.0f;
                        if (P.gate) {
                            const uint4* gp = reinterpret_cast<const uint4*>(P.gate + pix * P.N + c);
                            const uint4 g0 = gp[0], g1 = gp[1];
                            const uint32_t gw[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
#pragma unroll
                            for (int jj = 0; jj < 16; ++jj) {
                                const uint16_t h = (uint16_t)(gw[jj / 2] >> (16 * (jj & 1)));
                                if (!(bf16_to_f(h) > 0.0f)) v[jj] = 0.0f;
                            }
                        }
                        if (P.head_out) {
                            const float4* h4 = reinterpret_cast<const float4*>(s_head + c);
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                const float4 hw = h4[q];
                                head += hw.x * v[4 * q];
                                head += hw.y * v[4 * q + 1];
                                head += hw.z * v[4 * q + 2];
                                head += hw.w * v[4 * q + 3];
                            }
                        }
                        uint32_t packed[8];
#pragma unroll
                        for (int jj = 0; jj < 8; ++jj)
                            packed[jj] = (uint32_t)f_to_bf16(v[2 * jj]) |
                                         ((uint32_t)f_to_bf16(v[2 * jj + 1]) << 16);
                        uint16_t* dst = nullptr;
                        size_t off = 0;
                        if (c < P.n0 && P.out0) {
                            dst = P.out0;
                            off = pix * P.n0 + c;
                        } else if (c >= P.n0 && P.out1) {
                            dst = P.out1;
                            off = pix * (P.N - P.n0) + (c - P.n0);
                        }
                        if (dst) {
                            uint4* o = reinterpret_cast<uint4*>(dst + off);
                            o[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                            o[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                        }
                    }
                    if (inside && P.head_out) P.head_out[pix] = head;
                }
                umma::fence_before_sync();
                __syncwarp();
                if (lane == 0) umma::mbar_arrive(&acc_empty[slot.i]);
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 1) umma::tmem_dealloc(tmem, P.tmem_cols);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 4-D map of an NHWC bf16 tensor with an {8 channels, 136 pixels, G rows} box.
bool encode_nhwc(CUtensorMap* map, const void* base, int B, int H, int W, int C, int G) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    cuuint32_t box[4] = {8, (cuuint32_t)kBoxW, (cuuint32_t)G, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int num_sms_dev() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

}  // namespace natrix

extern "C" int natrix_nn_conv3x3(const natrix_nn_conv* c, void* stream) {
    using namespace natrix;
    if (!c || !c->src0 || !c->wpack)
        return set_last_error(NATRIX_EINVAL, "conv: NULL source or weights");
    if (c->c0 % 8 || c->c1 % 8 || c->c0 < 8 || c->N % 16 || c->N < 16 || c->N > 128 ||
        c->n0 % 16 || c->n0 > c->N || c->B < 1 || c->H < 1 || c->W < 1 || (c->c1 && !c->src1))
        return set_last_error(NATRIX_EINVAL, "conv: input channels must be multiples of 8, "
                                             "outputs multiples of 16 up to 128");
    if (c->head_out && c->N > 16)
        return set_last_error(NATRIX_EINVAL, "conv: the fused head takes 16 channels");
    ConvParams P{};
    P.B = c->B;
    P.H = c->H;
    P.W = c->W;
    P.c0 = c->c0;
    P.c1 = c->c1;
    P.ctot = (c->c0 + c->c1 + 15) / 16 * 16;
    P.N = c->N;
    P.wpack = c->wpack;
    P.bias = c->bias;
    P.relu = c->relu;
    P.gate = c->gate;
    P.out0 = c->out0;
    P.n0 = c->out1 ? c->n0 : c->N;
    P.out1 = c->out1;
    P.head_w = c->head_w;
    P.head_b = c->head_b;
    P.head_out = c->head_out;
    P.status = c->status;
    P.tiles_x = (c->W + kTileM - 1) / kTileM;
    const int sms = num_sms_dev();
    // segments: long enough that the 2 halo rows cost little, short enough
    // that every SM gets several
    int S = 64;
    auto units = [&](int rows) { return (long)c->B * P.tiles_x * ((c->H + rows - 1) / rows); };
    while (S > 8 && units(S) < 8L * sms) S /= 2;
    if (S > c->H) S = c->H;
    P.seg_rows = S;
    P.n_segs = (c->H + S - 1) / S;
    if (units(S) > 0x7fffffffL) return set_last_error(NATRIX_EINVAL, "conv: too many segments");
    P.n_units = (int)units(S);
    const uint32_t wbytes = (uint32_t)P.N * 9u * (uint32_t)P.ctot * 2u;
    P.smem_w = 0;
    P.smem_a = (wbytes + 1023u) / 1024u * 1024u;
    const uint32_t budget = 200u * 1024u;
    const long room = (long)budget - (long)P.smem_a;
    // rows per step: the largest G whose ring keeps a stage of lookahead
    // (G >= 2 reads stages t, t+1; G = 1 reads t .. t+2) and whose two
    // accumulator slots fit in TMEM
    P.G = 0;
    for (int G : {4, 2, 1}) {
        const long sb = (long)(P.ctot / 8) * G * kChunkBytes;
        const long fit = room > 0 ? room / sb : 0;
        const long need = G >= 2 ? 3 : 4;
        if (2L * G * P.N <= 512 && fit >= need && c->H >= G) {
            P.G = G;
            P.stage_bytes = (uint32_t)sb;
            P.stages = (int)(fit < kMaxStages ? fit : kMaxStages);
            break;
        }
    }
    if (!P.G)
        return set_last_error(NATRIX_EINVAL, "conv: weights + input rows exceed shared memory");
    const uint32_t smem = P.smem_a + (uint32_t)P.stages * P.stage_bytes;
    // slots: 4 when they fit in TMEM, else 2 (G is chosen so that 2 fit)
    P.n_slots = 4 * P.G * P.N <= 512 ? 4 : 2;
    uint32_t cols = 32;
    while (cols < (uint32_t)(P.n_slots * P.G * P.N)) cols *= 2;
    P.tmem_cols = cols;
    if (!P.status) return set_last_error(NATRIX_EINVAL, "conv: status word required");
    CUtensorMap tm0, tm1;
    if (!encode_nhwc(&tm0, c->src0, c->B, c->H, c->W, c->c0, P.G) ||
        !encode_nhwc(&tm1, c->src1 ? c->src1 : c->src0, c->B, c->H, c->W,
                     c->src1 ? c->c1 : c->c0, P.G))
        return set_last_error(NATRIX_ECUDA, "conv: tensor map encoding failed");
    const int grid = P.n_units < sms ? P.n_units : sms;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int pairs = P.ctot / 16;
    using Kern = void (*)(const CUtensorMap, const CUtensorMap, const ConvParams);
    Kern k = nullptr;
#define NX_CONV_CASE(GG, PP) \
    if (P.G == GG && pairs == PP) k = k_conv3x3_tc<GG, PP>;
#define NX_CONV_G(GG) \
    NX_CONV_CASE(GG, 1) NX_CONV_CASE(GG, 2) NX_CONV_CASE(GG, 3) NX_CONV_CASE(GG, 4) NX_CONV_CASE(GG, 6)
    NX_CONV_G(1) NX_CONV_G(2) NX_CONV_G(4)
#undef NX_CONV_G
#undef NX_CONV_CASE
    if (!k) return set_last_error(NATRIX_EINVAL, "conv: input channels must total 16, 32, 48, 64 or 96");
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
        cudaSuccess)
        return set_last_error(NATRIX_ECUDA, "conv: shared memory attribute");
    k<<<grid, kThreads, smem, st>>>(tm0, tm1, P);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_last_error(NATRIX_ECUDA, cudaGetErrorString(e));
    return NATRIX_OK;
}
