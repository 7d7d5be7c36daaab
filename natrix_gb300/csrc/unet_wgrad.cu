// Weight gradient of a 3x3 convolution on the tensor cores.
//
// For tap t = (dy, dx):  dW_t[ci][co] = sum over pixels p of
//     X[p + (dy, dx)][ci] * dZ[p][co]
// is a GEMM with M = input channels (padded to 128 rows), N = output channels
// and K = pixels.  Both operands arrive pixel-major (NHWC): a producer warp
// fetches each chunk (64 pixels of one image row, plus one pixel either side
// of the input rows) with TMA, and eight warps transpose it, 8 x 8 blocks in
// registers, into the K-major SWIZZLE_NONE operand layout the forward
// convolution uses (core matrices of 8 rows x 8 pixels, 16-byte rows; SBO =
// 128 between row groups, LBO between 8-pixel groups): A_dx for
// the three horizontal taps of one kernel row and B = dZ^T.  One thread issues
// the 3 x 4 tcgen05.mma (M = 128, N = cout, K = 16) of a chunk into three
// TMEM accumulators of cout columns; staging and MMAs alternate between two
// buffers (the MMA commit of a buffer's last use guards its restaging).
// Three passes cover the kernel rows dy = -1, 0, 1; after each pass the block
// reads its accumulators with tcgen05.ld and adds them into dW with FP32
// atomics (one partial sum per block and weight).
//
// Pixels outside the image arrive as zeros from TMA (the convolution's
// padding).  All
// waits are bounded; a wait that runs out sets status bit 4 and the block
// skips the rest of its work after freeing TMEM.
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include "../../include/natrix.h"
#include "../../include/natrix_nn.h"
#include "kernels.cuh"
#include "umma.cuh"

namespace natrix {

namespace {

constexpr int kWgThreads = 256;
constexpr int kChunkPix = 64;                     // pixels (K) per chunk
constexpr int kRowsA = 128;                       // M: input channels, padded
constexpr int kALbo = (kRowsA / 8) * 128;         // 2048 B between 8-pixel groups
constexpr int kABytes = kRowsA * kChunkPix * 2;   // 16 KB per tap

__device__ __forceinline__ float bfw(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

// K-major SWIZZLE_NONE operand: element (row, k) sits at
// (row / 8) * 128 + (k / 8) * LBO + (row % 8) * 16 + (k % 8) * 2 bytes.

// 8 x 8 transpose of 16-bit values across the 8 lanes of an aligned lane
// group: lane kk enters holding the 8 channels of pixel kk (4 words of two
// channels) and leaves holding channel kk of pixels 0..7, so each lane then
// writes one 16-byte core-matrix row (bank-conflict free) instead of eight
// scattered 2-byte values.  Three butterfly stages: word pairs (distance 4),
// words (distance 2), 16-bit halves (distance 1).
__device__ __forceinline__ void transpose8(uint32_t (&w)[4], int kk) {
    const unsigned FULL = 0xffffffffu;
    uint32_t s0 = (kk & 4) ? w[0] : w[2], s1 = (kk & 4) ? w[1] : w[3];
    uint32_t r0 = __shfl_xor_sync(FULL, s0, 4), r1 = __shfl_xor_sync(FULL, s1, 4);
    if (kk & 4) {
        w[0] = r0;
        w[1] = r1;
    } else {
        w[2] = r0;
        w[3] = r1;
    }
    s0 = (kk & 2) ? w[0] : w[1];
    s1 = (kk & 2) ? w[2] : w[3];
    r0 = __shfl_xor_sync(FULL, s0, 2);
    r1 = __shfl_xor_sync(FULL, s1, 2);
    if (kk & 2) {
        w[0] = r0;
        w[2] = r1;
    } else {
        w[1] = r0;
        w[3] = r1;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint32_t part = __shfl_xor_sync(FULL, w[i], 1);
        w[i] = (kk & 1) ? __byte_perm(part, w[i], 0x7632) : __byte_perm(w[i], part, 0x5410);
    }
}

struct WgParams {
    const uint16_t* dz;
    const uint16_t* x0;
    const uint16_t* x1;
    int cout, c0, c1, B, H, W;
    int cpr;       // chunks per image row: ceil(W / 64)
    int n_chunks;  // B * H * cpr (each chunk: 64 pixels of one image row)
    float* dw;
    int* status;
    uint32_t tmem_cols;
    uint32_t buf_bytes;  // 3 A tiles + B tile
    uint32_t raw_bytes;  // x0, x1 and dZ segments of one chunk
};

// Warp roles: warp 9 lane 0 fetches each chunk's raw rows with TMA (the
// 66-pixel x segment of every input source, the 64-pixel dZ segment; out of
// image pixels and rows arrive as zeros) into one of two raw buffers; warps
// 0-7 transpose a raw buffer into one of two operand buffers; warp 8 lane 0
// issues the MMAs.  Barriers: rawfull (TMA bytes), rawempty (8 warps done
// reading), full (8 warps done writing), empty (MMA commit), done (a pass's
// last commit, before the accumulator read-out).
constexpr int kStageWarps = 8;
constexpr int kXBox = kChunkPix + 2;  // x0 - 1 .. x0 + 64
constexpr int kWgAllThreads = kWgThreads + 64;

__global__ void __launch_bounds__(kWgAllThreads, 1)
    k_wgrad_tc(const __grid_constant__ CUtensorMap tx0, const __grid_constant__ CUtensorMap tx1,
               const __grid_constant__ CUtensorMap tdz, const WgParams P) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t full[2], empty[2], rawfull[2], rawempty[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int cin = P.c0 + P.c1, cout = P.cout;
    const int b_lbo = (cout / 8) * 128;
    const uint32_t b_off = 3u * kABytes;
    const uint32_t raw0 = 2u * P.buf_bytes;  // raw buffers after the operand buffers
    // TMA destinations start on 128-byte boundaries
    const uint32_t x1_off = (uint32_t)(kXBox * P.c0 * 2 + 127) / 128 * 128;
    const uint32_t dz_off = x1_off + (uint32_t)(kXBox * P.c1 * 2 + 127) / 128 * 128;
    const uint32_t raw_tx = (uint32_t)(kXBox * cin * 2 + kChunkPix * cout * 2);

    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            umma::mbar_init(&full[b], kStageWarps);
            umma::mbar_init(&empty[b], 1);
            umma::mbar_init(&rawfull[b], 1);
            umma::mbar_init(&rawempty[b], kStageWarps);
        }
        umma::mbar_init(&done, 1);
        umma::mbar_init_fence();
        s_ok = 1;
    }
    // operand rows >= cin stay zero for the whole kernel
    for (uint32_t i = tid * 16; i < 2 * P.buf_bytes; i += kWgAllThreads * 16)
        *reinterpret_cast<uint4*>(smem + i) = make_uint4(0, 0, 0, 0);
    if (warp == kStageWarps) umma::tmem_alloc(&tmem_slot, P.tmem_cols);
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_slot;

    // this block's chunks
    const int per = (P.n_chunks + gridDim.x - 1) / gridDim.x;
    const int ch0 = blockIdx.x * per;
    const int ch1 = min(ch0 + per, P.n_chunks);
    uint32_t fills[2] = {0, 0};  // operand buffer uses (staging warps / MMA warp)
    uint32_t raws[2] = {0, 0};   // raw buffer uses (producer / staging warps)
    uint32_t done_phase = 0;
    bool ok = true;

    for (int pass = 0; pass < 3 && ch0 < ch1; ++pass) {
        const int dy = pass - 1;
        if (warp == kStageWarps + 1) {
            if (lane == 0 && ok) {
                int it = 0;
                for (int ch = ch0; ch < ch1 && ok; ++ch, ++it) {
                    const int rb = it & 1;
                    if (raws[rb] > 0) ok = umma::mbar_wait(&rawempty[rb], (raws[rb] - 1) & 1u);
                    if (!ok) break;
                    const int row = ch / P.cpr, x0 = (ch - row * P.cpr) * kChunkPix;
                    const int y = row % P.H, b = row / P.H;
                    unsigned char* r = smem + raw0 + (uint32_t)rb * P.raw_bytes;
                    umma::mbar_arrive_expect_tx(&rawfull[rb], raw_tx);
                    umma::tma_load_4d(r, &tx0, 0, x0 - 1, y + dy, b, &rawfull[rb]);
                    if (P.c1) umma::tma_load_4d(r + x1_off, &tx1, 0, x0 - 1, y + dy, b, &rawfull[rb]);
                    umma::tma_load_4d(r + dz_off, &tdz, 0, x0, y, b, &rawfull[rb]);
                    ++raws[rb];
                }
                if (!ok) s_ok = 0;
            }
        } else if (warp == kStageWarps) {
            if (lane == 0 && ok) {
                const uint32_t idesc = umma::idesc_bf16_f32(kRowsA, cout);
                const uint64_t a_desc = umma::smem_desc(umma::smem_u32(smem), kALbo, 128);
                const uint64_t b_desc = umma::smem_desc(umma::smem_u32(smem + b_off), b_lbo, 128);
                const uint32_t buf16 = P.buf_bytes >> 4, a16 = kABytes >> 4;
                const uint32_t a_k = (2u * kALbo) >> 4, b_k = (2u * (uint32_t)b_lbo) >> 4;
                int it = 0;
                for (int ch = ch0; ch < ch1 && ok; ++ch, ++it) {
                    const int buf = it & 1;
                    ok = umma::mbar_wait(&full[buf], fills[buf] & 1u);
                    if (!ok) break;
                    umma::fence_after_sync();
                    const uint64_t ab = a_desc + (uint32_t)buf * buf16, bb = b_desc + (uint32_t)buf * buf16;
#pragma unroll
                    for (int dxi = 0; dxi < 3; ++dxi) {
#pragma unroll
                        for (int m = 0; m < kChunkPix / 16; ++m)
                            umma::mma_bf16(tmem + (uint32_t)(dxi * cout),
                                           ab + (uint32_t)dxi * a16 + (uint32_t)m * a_k,
                                           bb + (uint32_t)m * b_k,
                                           idesc, (it > 0 || m > 0) ? 1u : 0u);
                    }
                    umma::commit(&empty[buf]);
                    ++fills[buf];
                }
                umma::commit(&done);
                if (!ok) s_ok = 0;
            }
        } else {
            const int cz8 = cout / 8, ci8 = cin / 8, c08 = P.c0 / 8;
            int it = 0;
            for (int ch = ch0; ch < ch1; ++ch, ++it) {
                const int buf = it & 1;
                unsigned char* base = smem + (uint32_t)buf * P.buf_bytes;
                const unsigned char* r = smem + raw0 + (uint32_t)buf * P.raw_bytes;
                bool w = true;
                if (lane == 0) {
                    w = umma::mbar_wait(&rawfull[buf], raws[buf] & 1u);
                    // the MMAs that read this operand buffer's previous chunk must be done
                    if (w && fills[buf] > 0) w = umma::mbar_wait(&empty[buf], (fills[buf] - 1) & 1u);
                }
                w = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
                if (!w) {
                    ok = false;
                    break;
                }
                // B = dZ^T: a lane group of 8 reads 8 pixels' 8-channel groups
                // and transposes them into 8 rows of 8 pixels
                for (int i = tid; i < kChunkPix * cz8; i += kWgThreads) {  // multiple of 32
                    const int kk = i & 7, rest = i >> 3;
                    const int g = rest % cz8, kg = rest / cz8;
                    const uint4 u = *reinterpret_cast<const uint4*>(
                        r + dz_off + (uint32_t)(((8 * kg + kk) * cout + 8 * g) * 2));
                    uint32_t wv[4] = {u.x, u.y, u.z, u.w};
                    transpose8(wv, kk);
                    *reinterpret_cast<uint4*>(base + b_off + (uint32_t)(g * 128 + kg * b_lbo + kk * 16)) =
                        make_uint4(wv[0], wv[1], wv[2], wv[3]);
                }
                // A_dx = X shifted by (dy, dx): pixel k + dx of the 66-pixel segment
                for (int i = tid; i < 3 * kChunkPix * ci8; i += kWgThreads) {  // multiple of 32
                    const int kk = i & 7, rest = i >> 3;
                    const int g = rest % ci8, rest2 = rest / ci8;
                    const int kg = rest2 & 7, dxi = rest2 >> 3;
                    const int px = 8 * kg + kk + dxi;
                    const uint4 u = g < c08
                        ? *reinterpret_cast<const uint4*>(r + (uint32_t)((px * P.c0 + 8 * g) * 2))
                        : *reinterpret_cast<const uint4*>(r + x1_off +
                                                          (uint32_t)((px * P.c1 + 8 * (g - c08)) * 2));
                    uint32_t wv[4] = {u.x, u.y, u.z, u.w};
                    transpose8(wv, kk);
                    *reinterpret_cast<uint4*>(base + (uint32_t)dxi * kABytes +
                                              (uint32_t)(g * 128 + kg * kALbo + kk * 16)) =
                        make_uint4(wv[0], wv[1], wv[2], wv[3]);
                }
                umma::fence_smem_to_async();
                __syncwarp();
                if (lane == 0) {
                    umma::mbar_arrive(&rawempty[buf]);
                    umma::mbar_arrive(&full[buf]);
                }
                ++fills[buf];
                ++raws[buf];
            }
        }
        // the pass's accumulators: wait for the last commit, then read
        if (warp < kStageWarps) {
            bool w = ok;
            if (lane == 0 && w) w = umma::mbar_wait(&done, done_phase);
            w = __shfl_sync(0xffffffffu, w ? 1 : 0, 0) != 0;
            if (!w) ok = false;
        }
        done_phase ^= 1u;
        if (!ok) s_ok = 0;
        __syncthreads();
        if (!s_ok) {
            ok = false;
            break;
        }
        umma::fence_after_sync();
        if (warp < kStageWarps) {
            // warps w and w + 4 share TMEM lane quarter w % 4 and split the columns
            const int quarter = warp & 3, half = warp >> 2;
            const int ci = quarter * 32 + lane;
            const int ncol = 3 * cout;
            for (int c = half * 16; c < ncol; c += 32) {
                float v[16];
                umma::tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, v);
                if (ci < cin) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int col = c + j, dxi = col / cout, co = col % cout;
                        atomicAdd(P.dw + ((size_t)co * cin + ci) * 9 + (dy + 1) * 3 + dxi, v[j]);
                    }
                }
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    }
    if (tid == 0 && (!ok || !s_ok)) atomicOr(P.status, 4);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == kStageWarps) umma::tmem_dealloc(tmem, P.tmem_cols);
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

// 4-D map of an NHWC bf16 tensor whose box is one row segment: {all C
// channels, box_w pixels, 1 row, 1 image} (C * 2 bytes <= 256 elements' worth)
bool encode_rows(CUtensorMap* map, const void* base, int B, int H, int W, int C, int box_w) {
    auto fn = wg_encode_fn();
    if (!fn) return false;
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    cuuint32_t box[4] = {(cuuint32_t)C, (cuuint32_t)box_w, 1, 1};
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
    WgParams P{};
    P.dz = dz;
    P.x0 = x0;
    P.x1 = x1;
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
    P.status = status;
    uint32_t cols = 32;
    while (cols < (uint32_t)(3 * cout)) cols *= 2;
    P.tmem_cols = cols;
    P.buf_bytes = 3u * kABytes + (uint32_t)cout * kChunkPix * 2u;
    P.raw_bytes = (uint32_t)(kXBox * c0 * 2 + 127) / 128 * 128 +
                  (uint32_t)(kXBox * c1 * 2 + 127) / 128 * 128 + (uint32_t)kChunkPix * cout * 2u;
    P.raw_bytes = (P.raw_bytes + 127u) / 128u * 128u;
    const uint32_t smem = 2u * P.buf_bytes + 2u * P.raw_bytes;
    CUtensorMap tx0, tx1, tdz;
    if (!encode_rows(&tx0, x0, B, H, W, c0, kXBox) ||
        !encode_rows(&tx1, c1 ? x1 : x0, B, H, W, c1 ? c1 : c0, kXBox) ||
        !encode_rows(&tdz, dz, B, H, W, cout, kChunkPix))
        return wg_fail(NATRIX_ECUDA, "wgrad: tensor map encoding failed");
    if (cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return wg_fail(NATRIX_ECUDA, "wgrad: shared memory attribute");
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = P.n_chunks < sms ? P.n_chunks : sms;
    k_wgrad_tc<<<grid, kWgAllThreads, smem, st>>>(tx0, tx1, tdz, P);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return wg_fail(NATRIX_ECUDA, cudaGetErrorString(e));
    if (db) {
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
