// Weight gradient of a 3x3 convolution on the tensor cores.
//
// For tap t = (dy, dx):  dW_t[ci][co] = sum over pixels p of
//     X[p + (dy, dx)][ci] * dZ[p][co]
// is a GEMM with M = input channels (padded to 128 rows), N = output channels
// and K = pixels.  Both operands are pixel-major (NHWC), and the tensor cores
// read them that way: MN-major operands (pixels along K), staged by TMA one
// 8-channel chunk of a row segment at a time.  A block walks "chunks" (64
// pixels of one image row); three passes cover the kernel rows dy = -1, 0, 1,
// each accumulating the three horizontal taps of its row into three TMEM
// accumulators (the taps read the same staged 66-pixel x segment at +0, +16
// and +32 bytes), and after each pass the block reads its accumulators with
// tcgen05.ld and adds them into dW with FP32 atomics (one partial sum per
// block and weight).
//
// Pixels outside the image arrive as zeros from TMA (the convolution's
// padding).  All waits are bounded; a wait that runs out sets status bit 4
// and the block skips the rest of its work after freeing TMEM.
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include "../../include/natrix.h"
#include "../../include/natrix_nn.h"
#include "kernels.cuh"
#include "umma.cuh"

namespace natrix {

namespace {

constexpr int kChunkPix = 64;  // pixels (K) per chunk
constexpr int kRowsA = 128;    // M: input channels, padded
constexpr int kXBox = kChunkPix + 2;  // x segment: x0 - 1 .. x0 + 64

__device__ __forceinline__ float bfw(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

// The tensor cores read both operands MN-major (pixels along K, channels
// along M / N), which is exactly how NHWC data lands in shared memory when
// TMA copies one 8-channel chunk of a row segment ([chunk][pixel][8
// channels], 16-byte pixel rows): core matrix = 8 pixels x 8 channels, 128
// bytes; for this layout the descriptor's LBO is the 128 bytes between core
// matrices along K and its SBO the chunk slot between core matrices along
// M / N.  No register transposes: warp 0 lane 0 issues the TMA copies of a
// stage (the 66-pixel x segments of every input chunk, the 64-pixel dZ
// segments); warp 1 lane 0 and, when two accumulator sets fit in TMEM
// (6 cout <= 512), warp 6 lane 0 issue the 3 x 4 MMAs of alternate chunks
// (M = 128 channel rows, N = cout, K = 16 pixels) into their own three
// accumulators of the pass; warps 2-5 read the accumulators out after each
// pass and add the two sets.  Channel rows past
// cin read whatever their chunk slots hold; those accumulator rows are never
// read.

// Position in a ring of n stages plus the parity of the pass over the ring.
struct RingPos {
    uint32_t i = 0, ph = 0;
    __device__ __forceinline__ void next(uint32_t n) {
        if (++i == n) {
            i = 0;
            ph ^= 1u;
        }
    }
};

constexpr int kMnThreads = 224;
constexpr int kIssuer2 = 6;  // warp of the second MMA issuer
constexpr int kXSlot = 1152;                  // 66 pixels x 16 B, padded to 128 B
constexpr int kXSlot3 = 3200;                 // three rows of 66 pixels x 16 B, padded
constexpr int kZSlot = kChunkPix * 16;        // 64 pixels x 16 B
constexpr int kASlots = kRowsA / 8;           // channel chunks of M = 128
constexpr int kMnMaxStages = 12;

struct WgMnParams {
    int cout, c0, c1, B, H, W;
    int cpr, n_chunks;
    float* dw;
    float* db;  // bias gradient from the ones slot, or null (separate kernel)
    int* status;
    uint32_t tmem_cols;
    uint32_t a_bytes;      // X part of a stage (the dZ segments follow it)
    uint32_t stage_bytes;  // a_bytes + cout / 8 x kZSlot
    int stages;
    int issuers;  // 1 or 2 (two accumulator sets of 3 cout columns)
};

// kNine: one pass with all nine taps (needs 9 x cout x issuers TMEM
// columns: cout 16).  Each input chunk arrives as one three-row box (rows
// y - 1 .. y + 1, slot stride kXSlot3) and dZ once per chunk, a third of the
// copies of the three-pass form; tap (dy, dx) reads row dy + 1 at +16 dx bytes.
// Only the slots that hold channels (and the ones slot) are part of a stage;
// the A operand's other M rows read whatever follows (the next stages or the
// slack past the last one) and are never read back.
template <bool kNine>
__global__ void __launch_bounds__(kMnThreads, 1)
    k_wgrad_mn(const __grid_constant__ CUtensorMap tx0, const __grid_constant__ CUtensorMap tx1,
               const __grid_constant__ CUtensorMap tdz, const WgMnParams P) {
    constexpr int kPasses = kNine ? 1 : 3;
    constexpr int kTaps = kNine ? 9 : 3;
    constexpr int kXRows = kNine ? 3 : 1;
    constexpr uint32_t kSlot = kNine ? kXSlot3 : kXSlot;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t full[kMnMaxStages], empty[kMnMaxStages], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int cin = P.c0 + P.c1, cout = P.cout;
    const int q0 = P.c0 / 8, q1 = P.c1 / 8, qz = cout / 8;
    const uint32_t R = (uint32_t)P.stages;
    const uint32_t a_bytes = P.a_bytes;
    const uint32_t tx_bytes =
        (uint32_t)(q0 + q1) * kXBox * 16u * kXRows + (uint32_t)qz * kZSlot;

    if (tid == 0) {
        for (int i = 0; i < P.stages; ++i) {
            umma::mbar_init(&full[i], 1);
            umma::mbar_init(&empty[i], 1);
        }
        umma::mbar_init(&done, (uint32_t)P.issuers);
        umma::mbar_init_fence();
        s_ok = 1;
    }
    // Bias gradient for free: the first chunk slot past the input channels
    // holds bf16 ones in every stage (TMA never writes it), so its
    // accumulator rows sum dZ over the chunk's pixels.
    const int q_ones = q0 + q1;
    if (P.db) {
        const uint32_t ones = 0x3F803F80u;  // two bf16 1.0
        for (int s = 0; s < P.stages; ++s) {
            uint32_t* slot = reinterpret_cast<uint32_t*>(smem + s * P.stage_bytes + q_ones * kSlot);
            for (int k = tid; k < kXBox * 4 * kXRows; k += kMnThreads) slot[k] = ones;
        }
        umma::fence_smem_to_async();
    }
    if (warp == 1) umma::tmem_alloc(&tmem_slot, P.tmem_cols);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_slot;

    const int per = (P.n_chunks + gridDim.x - 1) / gridDim.x;
    const int ch0 = blockIdx.x * per;
    const int ch1 = min(ch0 + per, P.n_chunks);
    RingPos ps, ms;  // producer / MMA positions in the stage ring (continue across passes)
    // stages the producer has armed, and the parity of each one's last lap:
    // before the CTA exits it waits for those copies to land
    uint32_t armed = 0, armed_ph = 0;
    bool ok = true;

    for (int pass = 0; pass < kPasses && ch0 < ch1; ++pass) {
        const int dy = kNine ? 0 : pass - 1;  // kNine: rows y - 1 .. y + 1 in one box
        if (warp == 0 && lane == 0) {
            for (int ch = ch0; ch < ch1 && ok; ++ch, ps.next(R)) {
                ok = umma::mbar_wait(&empty[ps.i], ps.ph ^ 1u);
                if (!ok) break;
                const int row = ch / P.cpr, x0 = (ch - row * P.cpr) * kChunkPix;
                const int y = row % P.H, b = row / P.H;
                unsigned char* st = smem + ps.i * P.stage_bytes;
                umma::mbar_arrive_expect_tx(&full[ps.i], tx_bytes);
                armed |= 1u << ps.i;
                armed_ph = (armed_ph & ~(1u << ps.i)) | (ps.ph << ps.i);
                const int ty = kNine ? y - 1 : y + dy;
                for (int q = 0; q < q0; ++q)
                    umma::tma_load_4d(st + q * kSlot, &tx0, 8 * q, x0 - 1, ty, b, &full[ps.i]);
                for (int q = 0; q < q1; ++q)
                    umma::tma_load_4d(st + (q0 + q) * kSlot, &tx1, 8 * q, x0 - 1, ty, b,
                                      &full[ps.i]);
                for (int q = 0; q < qz; ++q)
                    umma::tma_load_4d(st + a_bytes + q * kZSlot, &tdz, 8 * q, x0, y, b, &full[ps.i]);
            }
            if (!ok) s_ok = 0;
        } else if ((warp == 1 || (warp == kIssuer2 && P.issuers == 2)) && lane == 0) {
            const int ii = warp == 1 ? 0 : 1;  // this issuer takes chunks it % issuers == ii
            const uint32_t acc = tmem + (uint32_t)(ii * kTaps * cout);
            // both operands MN-major (instruction descriptor bits 15, 16)
            const uint32_t idesc = umma::idesc_bf16_f32(kRowsA, cout) | (1u << 15) | (1u << 16);
            // MN-major without swizzling: LBO = 128 B between 8-pixel groups
            // (along K), SBO = one chunk slot between 8-channel groups (M / N)
            const uint64_t a0 = umma::smem_desc(umma::smem_u32(smem), 128, kSlot);
            const uint64_t b0 = umma::smem_desc(umma::smem_u32(smem + a_bytes), 128, kZSlot);
            const uint32_t stage16 = P.stage_bytes >> 4;
            int it = 0;
            bool first = true;  // this issuer's first chunk of the pass
            for (int ch = ch0; ch < ch1 && ok; ++ch, ++it, ms.next(R)) {
                if (it % P.issuers != ii) continue;
                ok = umma::mbar_wait(&full[ms.i], ms.ph);
                if (!ok) break;
                umma::fence_after_sync();
                const uint64_t ab = a0 + ms.i * stage16, bb = b0 + ms.i * stage16;
#pragma unroll
                for (int t = 0; t < kTaps; ++t) {
                    // row t / 3 of the box (66 pixels = 66 units of 16 B), pixel shift t % 3
                    const uint32_t aoff = (uint32_t)((t / 3) * kXBox + t % 3);
#pragma unroll
                    for (int m = 0; m < kChunkPix / 16; ++m)
                        umma::mma_bf16(acc + (uint32_t)(t * cout), ab + aoff + (uint32_t)m * 16u,
                                       bb + (uint32_t)m * 16u, idesc,
                                       (!first || m > 0) ? 1u : 0u);
                }
                first = false;
                umma::commit(&empty[ms.i]);
            }

            umma::commit(&done);
            if (!ok) s_ok = 0;
        } else if (warp >= 2 && warp < kIssuer2) {
            // the pass's accumulators: wait for the last commit, then read
            bool w = true;
            if (lane == 0) w = umma::mbar_wait(&done, (uint32_t)pass & 1u);
            w = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
            if (!w) {
                if (lane == 0) s_ok = 0;
            } else {
                umma::fence_after_sync();
                const int quarter = warp & 3;
                const int ci = quarter * 32 + lane;
                for (int c = 0; c < kTaps * cout; c += 16) {
                    float v[16];
                    umma::tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, v);
                    // the second set holds a sum only when the second issuer
                    // had a chunk (the block has at least two)
                    if (P.issuers == 2 && ch1 - ch0 >= 2) {
                        float v2[16];
                        umma::tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) +
                                            (uint32_t)(kTaps * cout + c),
                                        v2);
#pragma unroll
                        for (int j = 0; j < 16; ++j) v[j] += v2[j];
                    }
                    // tap t of column c: kernel row (kNine ? t / 3 : dy + 1), column t % 3
                    constexpr int kCentre = kNine ? 4 : 1;
                    if (ci < cin) {
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const int col = c + j, t = col / cout, co = col % cout;
                            const int ky = kNine ? t / 3 : dy + 1;
                            atomicAdd(P.dw + ((size_t)co * cin + ci) * 9 + ky * 3 + t % 3, v[j]);
                        }
                    } else if (ci == cin && P.db && dy == 0 && c >= kCentre * cout &&
                               c < (kCentre + 1) * cout) {
                        // the ones row of the centre tap: sum of dZ per output channel
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            atomicAdd(P.db + (c - kCentre * cout + j), v[j]);
                    }
                }
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (!s_ok) {
            ok = false;
            break;
        }
    }
    if (tid == 0) {
        // every copy this CTA issued has landed before it exits (on a normal
        // run these phases completed long ago; after a wait ran out they may
        // still be in flight)
        for (uint32_t i = 0; i < R; ++i)
            if ((armed >> i) & 1u) umma::mbar_wait(&full[i], (armed_ph >> i) & 1u);
        if (!ok || !s_ok) atomicOr(P.status, 4);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 1) umma::tmem_dealloc(tmem, P.tmem_cols);
}

// db[co] += sum over pixels of dZ[p][co]: 8 channels per thread, block
// partial sums in shared memory, one atomic per block and channel
__global__ void __launch_bounds__(256) k_bias_grad(const uint16_t* __restrict__ dz, int cout,
                                                   int npix, float* __restrict__ db) {
    __shared__ float part[128];
    for (int i = threadIdx.x; i < cout; i += 256) part[i] = 0.0f;
    __syncthreads();
    const int cz8 = cout / 8;
    const int groups = 256 / cz8;  // pixels per block step (cout <= 128)
    const int g = threadIdx.x % cz8, lanep = threadIdx.x / cz8;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (lanep < groups) {
        for (int p = blockIdx.x * groups + lanep; p < npix; p += gridDim.x * groups) {
            const uint4 u = *reinterpret_cast<const uint4*>(dz + (size_t)p * cout + 8 * g);
            const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] += bfw((uint16_t)(w[j >> 1] >> (16 * (j & 1))));
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) atomicAdd(&part[8 * g + j], acc[j]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < cout; i += 256) atomicAdd(db + i, part[i]);
}

int wg_fail(int code, const char* msg) { return set_last_error(code, msg); }

PFN_cuTensorMapEncodeTiled_v12000 wg_encode_fn() {
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

// 4-D map of an NHWC bf16 tensor whose box is one 8-channel chunk of box_h
// row segments: {8 channels, box_w pixels, box_h rows, 1 image}.
bool encode_chunks(CUtensorMap* map, const void* base, int B, int H, int W, int C, int box_w,
                   int box_h = 1) {
    auto fn = wg_encode_fn();
    if (!fn) return false;
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    cuuint32_t box[4] = {8, (cuuint32_t)box_w, (cuuint32_t)box_h, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// status word of the weight-gradient kernels (bit 2: a bounded wait ran out)
__device__ int g_wgrad_status;

}  // namespace

// Tensor-core path of natrix_nn_wgrad (unet_kernels.cu dispatches here when
// the shapes allow it: cin <= 128, cout a multiple of 16 up to 128).
int wgrad_tc(const uint16_t* dz, int cout, const uint16_t* x0, int c0, const uint16_t* x1, int c1,
             int B, int H, int W, float* dw, float* db, cudaStream_t st) {
    const long npix = (long)B * H * W;
    if (npix <= 0) return NATRIX_OK;
    static int* status = nullptr;
    if (!status && cudaGetSymbolAddress(reinterpret_cast<void**>(&status), g_wgrad_status) !=
                       cudaSuccess)
        return wg_fail(NATRIX_ECUDA, "wgrad: status word");
    WgMnParams P{};
    P.cout = cout;
    P.c0 = c0;
    P.c1 = c1;
    P.B = B;
    P.H = H;
    P.W = W;
    P.cpr = (W + kChunkPix - 1) / kChunkPix;
    if ((long)B * H * P.cpr >= (1L << 31)) return wg_fail(NATRIX_EINVAL, "wgrad: too many rows");
    P.n_chunks = B * H * P.cpr;
    P.dw = dw;
    // the ones slot needs a free 8-channel slot of the 128 M rows
    P.db = (db && c0 + c1 + 8 <= kRowsA) ? db : nullptr;
    P.status = status;
    // nine taps in one pass when two issuers' accumulators fit (cout 16)
    const bool nine = 2 * 9 * cout <= 512;
    const int taps = nine ? 9 : 3;
    P.issuers = 2 * taps * cout <= 512 ? 2 : 1;
    uint32_t cols = 32;
    while (cols < (uint32_t)(taps * cout * P.issuers)) cols *= 2;
    P.tmem_cols = cols;
    // kNine: the channel slots plus the ones slot; the A operand's other M
    // rows reach up to 15 slots + the last tap's rows past a stage's start
    // (51,168 bytes), covered by the reach below.  Three passes: all 16 slots.
    P.a_bytes = nine ? (uint32_t)((c0 + c1) / 8 + 1) * kXSlot3 : (uint32_t)kASlots * kXSlot;
    P.stage_bytes = P.a_bytes + (uint32_t)(cout / 8) * kZSlot;
    const uint32_t reach = nine ? 51200u : 8192u;
    const uint32_t budget = (nine ? 220u : 200u) * 1024u;
    P.stages = (int)((budget - (nine ? reach : 0u)) / P.stage_bytes);
    if (P.stages > kMnMaxStages) P.stages = kMnMaxStages;
    // Two issuers take alternate chunks; with an even ring every stage's
    // chunks share one parity, so each stage is only ever consumed by one
    // issuer, lap after lap in order.  (With an odd ring an issuer could wait
    // for a stage's next lap before the current lap had landed, and the
    // parity test would match the lap before.)
    if (P.issuers == 2 && (P.stages & 1)) --P.stages;
    if (P.stages < 2) return wg_fail(NATRIX_EINVAL, "wgrad: stage does not fit");
    // slack past the last stage: every descriptor read stays inside the
    // allocation whichever of its two strides runs along K
    const uint32_t smem = (uint32_t)P.stages * P.stage_bytes + reach;
    const int rows = nine ? 3 : 1;
    CUtensorMap tx0, tx1, tdz;
    if (!encode_chunks(&tx0, x0, B, H, W, c0, kXBox, rows) ||
        !encode_chunks(&tx1, c1 ? x1 : x0, B, H, W, c1 ? c1 : c0, kXBox, rows) ||
        !encode_chunks(&tdz, dz, B, H, W, cout, kChunkPix))
        return wg_fail(NATRIX_ECUDA, "wgrad: tensor map encoding failed");
    auto kernel = nine ? k_wgrad_mn<true> : k_wgrad_mn<false>;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return wg_fail(NATRIX_ECUDA, "wgrad: shared memory attribute");
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = P.n_chunks < sms ? P.n_chunks : sms;
    kernel<<<grid, kMnThreads, smem, st>>>(tx0, tx1, tdz, P);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return wg_fail(NATRIX_ECUDA, cudaGetErrorString(e));
    if (db && !P.db) {
        const int groups = 256 / (cout / 8);
        long blocks = (npix + groups - 1) / groups;
        blocks = blocks < 1024 ? blocks : 1024;
        k_bias_grad<<<(unsigned)blocks, 256, 0, st>>>(dz, cout, (int)npix, db);
        if ((e = cudaGetLastError()) != cudaSuccess) return wg_fail(NATRIX_ECUDA, cudaGetErrorString(e));
    }
    return NATRIX_OK;
}

}  // namespace natrix

extern "C" int natrix_nn_wgrad_status(int32_t* out) {
    using namespace natrix;
    if (!out) return set_last_error(NATRIX_EINVAL, "NULL argument");
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_wgrad_status, sizeof v);
    if (e == cudaSuccess && v) {
        const int z = 0;
        e = cudaMemcpyToSymbol(g_wgrad_status, &z, sizeof z);
    }
    if (e != cudaSuccess) return set_last_error(NATRIX_ECUDA, cudaGetErrorString(e));
    *out = v;
    return NATRIX_OK;
}
