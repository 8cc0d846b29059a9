// Learned denoiser kernels: a kernel-predicting CNN (8 conv3x3 layers of 48
// channels, ReLU, a 5x5 per-pixel filter from a softmax over 25 logits),
// trained on pairs of low-spp frames (radiance + albedo, normal, depth
// G-buffers) and high-spp targets rendered by this path tracer.  No
// reference counterpart: vk_cinematic has no denoiser.
//
// Tensors are NHWC.  Activations and weights are BF16, accumulation FP32.
//  * conv3x3 forward / data gradient: implicit GEMM on the tensor cores,
//    M = pixels, N = output channels, K = 9 taps x input channels, with
//    mma.sync m16n8k16 BF16.  CTAs are persistent: each loads the layer's
//    weights into shared memory once (padded rows, conflict-free fragment
//    loads) and then walks 64-pixel row segments.
//  * weight gradient: FP32 outer products over pixel chunks, one tap per
//    CTA, reduced with atomics.
//  * filter, loss and Adam: elementwise FP32.

#include <cstdint>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <atomic>
#include <mutex>

#include "gbsp_internal.h"

namespace gbsp {
namespace dn {

constexpr int kTileP = 64;   // pixels per row segment
constexpr int kThreads = 128;

__device__ __forceinline__ void mma_bf16_16816(float *c, uint32_t a0, uint32_t a1, uint32_t a2,
    uint32_t a3, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// Activations and their gradients use a channel-group-planar layout,
// [B][H][C/8][W][8]: each 8-channel group of an image row is a contiguous
// plane of W x 16 bytes (BF16), so that one TMA box of a row's pixels is one
// contiguous read.  Element (row = b H + y, x, c):
__device__ __forceinline__ size_t cg_index(size_t row, int x, int c, int W, int C)
{
    return ((row * (size_t)(C / 8) + (size_t)(c / 8)) * (size_t)W + (size_t)x) * 8 + (size_t)(c % 8);
}

// 3: FP32 logits + bias fed straight into the 5x5 kernel-prediction filter
enum Epilogue : int { kEpiBf16BiasRelu = 0, kEpiF32Bias = 1, kEpiF32 = 2, kEpiFilter = 3 };

// out[p][co] = sum_{tap, ci} in[p + off(tap)][ci] * w[tap][co][ci] (+ bias, ReLU)
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(kThreads) k_conv3x3(const __nv_bfloat16 *__restrict__ in, int B,
    int H, int W, const __nv_bfloat16 *__restrict__ w, const float *__restrict__ bias,
    __nv_bfloat16 *__restrict__ outB, float *__restrict__ outF)
{
    static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel padding");
    constexpr int SIN = CIN + 8;  // padded element stride per pixel (bank-conflict free)
    constexpr int SPX = kTileP + 2;
    extern __shared__ __align__(128) unsigned char smemRaw[];
    __nv_bfloat16 *sW = reinterpret_cast<__nv_bfloat16 *>(smemRaw);   // [9][COUT][SIN]
    __nv_bfloat16 *sIn = sW + 9 * COUT * SIN;                          // [3][SPX][SIN]
    const int tid = threadIdx.x;
    for (int i = tid; i < 9 * COUT * (CIN / 2); i += kThreads) {
        int row = i / (CIN / 2), c2 = i % (CIN / 2);
        reinterpret_cast<uint32_t *>(sW + row * SIN)[c2] =
            reinterpret_cast<const uint32_t *>(w)[(size_t)row * (CIN / 2) + c2];
    }
    const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int tilesPerRow = (W + kTileP - 1) / kTileP;
    const int numTiles = tilesPerRow * B * H;
    for (int tile = blockIdx.x; tile < numTiles; tile += gridDim.x) {
        const int row = tile / tilesPerRow;  // b * H + y
        const int x0 = (tile % tilesPerRow) * kTileP;
        const int b = row / H, y = row % H;
        __syncthreads();  // previous tile's reads of sIn are done (and sW is loaded)
        for (int i = tid; i < 3 * SPX * (CIN / 2); i += kThreads) {
            int c2 = i % (CIN / 2);
            int px = (i / (CIN / 2)) % SPX;
            int ry = i / ((CIN / 2) * SPX);
            int gy = y + ry - 1, gx = x0 + px - 1;
            uint32_t v = 0;
            if (gy >= 0 && gy < H && gx >= 0 && gx < W)
                v = reinterpret_cast<const uint32_t *>(in)[cg_index((size_t)(b * H + gy), gx, 2 * c2, W, CIN) / 2];
            reinterpret_cast<uint32_t *>(sIn + (ry * SPX + px) * SIN)[c2] = v;
        }
        __syncthreads();
        float acc[COUT / 8][4];
#pragma unroll
        for (int n = 0; n < COUT / 8; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
        const int m0 = warp * 16;
#pragma unroll 1
        for (int tap = 0; tap < 9; tap++) {
            const int ty = tap / 3, tx = tap % 3;
            const __nv_bfloat16 *aBase = sIn + (ty * SPX + m0 + tx) * SIN;
            const __nv_bfloat16 *bBase = sW + tap * COUT * SIN;
#pragma unroll
            for (int kc = 0; kc < CIN; kc += 16) {
                uint32_t a0 = *reinterpret_cast<const uint32_t *>(aBase + g * SIN + kc + 2 * t);
                uint32_t a1 = *reinterpret_cast<const uint32_t *>(aBase + (g + 8) * SIN + kc + 2 * t);
                uint32_t a2 = *reinterpret_cast<const uint32_t *>(aBase + g * SIN + kc + 2 * t + 8);
                uint32_t a3 = *reinterpret_cast<const uint32_t *>(aBase + (g + 8) * SIN + kc + 2 * t + 8);
#pragma unroll
                for (int n = 0; n < COUT / 8; n++) {
                    const __nv_bfloat16 *bp = bBase + (n * 8 + g) * SIN + kc + 2 * t;
                    uint32_t b0 = *reinterpret_cast<const uint32_t *>(bp);
                    uint32_t b1 = *reinterpret_cast<const uint32_t *>(bp + 8);
                    mma_bf16_16816(acc[n], a0, a1, a2, a3, b0, b1);
                }
            }
        }
        // epilogue: rows g and g+8 of the warp's slab, columns 2t, 2t+1 of each n tile
#pragma unroll
        for (int half = 0; half < 2; half++) {
            int x = x0 + m0 + g + 8 * half;
            if (x >= W) continue;
            size_t p = (size_t)row * W + x;  // logits (FP32, NHWC)
#pragma unroll
            for (int n = 0; n < COUT / 8; n++) {
                int co = n * 8 + 2 * t;
                float v0 = acc[n][2 * half], v1 = acc[n][2 * half + 1];
                if (EPI != kEpiF32) {
                    v0 += bias[co];
                    v1 += bias[co + 1];
                }
                if (EPI == kEpiBf16BiasRelu) {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                    reinterpret_cast<uint32_t *>(outB)[cg_index(row, x, co, W, COUT) / 2] =
                        pack_bf16(v0, v1);
                } else if (EPI == kEpiF32Bias) {
                    *reinterpret_cast<float2 *>(outF + p * COUT + co) = make_float2(v0, v1);
                } else {
                    *reinterpret_cast<float2 *>(outF + cg_index(row, x, co, W, COUT)) =
                        make_float2(v0, v1);
                }
            }
        }
    }
}

template <int CIN, int COUT, int EPI>
int launch_conv(cudaStream_t s, int smCount, const void *in, int B, int H, int W, const void *w,
    const float *bias, void *outB, float *outF)
{
    constexpr int SIN = CIN + 8;
    size_t smem = (size_t)(9 * COUT + 3 * (kTileP + 2)) * SIN * 2;
    auto kern = k_conv3x3<CIN, COUT, EPI>;
    GBSP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int tiles = ((W + kTileP - 1) / kTileP) * B * H;
    int grid = smCount * 3;
    if (grid > tiles) grid = tiles;
    kern<<<grid, kThreads, smem, s>>>(reinterpret_cast<const __nv_bfloat16 *>(in), B, H, W,
        reinterpret_cast<const __nv_bfloat16 *>(w), bias, reinterpret_cast<__nv_bfloat16 *>(outB),
        outF);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

// ---------------------------------------------------------------------------
// conv3x3 on the 5th-generation tensor cores (tcgen05).
//
// GEMM: M = 128 pixels of one image row, K = 9 taps x CIN, and the G =
// kTcGroupRows output rows y .. y + G - 1 of a group side by side along N
// (row y + j in accumulator columns [j COUT, (j + 1) COUT)).  One elected
// thread issues tcgen05.mma.cta_group::1.kind::f16 (BF16 x BF16 -> FP32) per
// (input row, horizontal tap, 16-channel slice): input row y - 1 + k feeds
// every output row j of the group with k - j in 0..2 at once, with the
// matching tap rows of the [ty 2 | ty 1 | ty 0] weight stack as a
// contiguous B slice (N = COUT, 2 COUT or 3 COUT).  An M = 128 MMA costs
// about the same up to N = 96 and runs at the dense rate from N = 128, so
// G = 4 takes 6 instead of 12 MMAs per (tap, slice) for 4 rows.  Both
// operands are read straight from shared memory through matrix descriptors,
// so the 3x3 neighbourhood is never expanded: a horizontal tap is a
// 16-byte-granular offset of the A descriptor into a staged input row.
//
// Shared memory holds the operands in the canonical no-swizzle K-major
// layout: 8 x 16-byte core matrices (8 rows of 8 BF16 channels), rows
// contiguous.  Input rows: ring slots of [CIN/8 channel groups][kTcPlane
// pixels][16 B] (a core matrix = 8 consecutive pixels of one channel group,
// so a pixel shift moves the start by 16 B); weights: [3 taps][CIN/8
// groups][3 tap rows x COUT][16 B].  Descriptor strides: leading (K) = next
// channel group, stride (M or N) = next 8 rows = 128 B.
//
// One persistent CTA per SM walks vertical strips (one 128-pixel column
// segment, a run of rows) with its warps specialised and coupled only by
// mbarriers:
//   * lane 0 of warp 1 (producer) loads input rows into a ring of kTcRing
//     slots with TMA (cp.async.bulk.tensor: one box of 130 pixels x every
//     channel group per row, which in the channel-group-planar activation
//     layout is CIN/8 contiguous 2,080-byte runs; zero outside the image),
//     as many rows in flight as the ring allows; a row lands on its rowFull
//     barrier by transaction count, and its slot is reused once the MMAs of
//     the last row group that reads it have completed (rowEmpty, signalled
//     by tcgen05.commit);
//   * lane 0 of warp 0 issues, per group of kTcGroupRows output rows, the
//     (kTcGroupRows + 2) x 3 x CIN/16 MMAs reading its input rows into one
//     TMEM accumulator, then commits to that accumulator's accFull and to the
//     rowEmpty of the input rows no later group reads;
//   * warps 4-11 are two epilogue groups taking alternate row groups (warp
//     w owns TMEM lanes 32 (w % 4) .. + 31 = pixels): wait on accFull, read
//     the accumulator with tcgen05.ld, apply bias / ReLU / BF16 packing (or
//     the fused filter), and release it on accEmpty, while the tensor core
//     already works on the next group.
// Every wait is bounded; a timeout raises a shared abort flag that ends the
// other roles' waits, and sets g_dnStatus.
// ---------------------------------------------------------------------------
constexpr int kTcTileP = 128;
// One CTA per SM: warp 0 issues the MMAs, lane 0 of warp 1 loads rows, warps 4-11 are
// two epilogue groups that take alternate row groups.
constexpr int kTcThreads = 384;
constexpr int kTcEpiGroups = 2;
constexpr int kTcAccSlots = 4;  // at most; accumulator a is drained by epilogue group a % 2
constexpr int kTcSpx = kTcTileP + 2;     // staged pixels per row: x0 - 1 .. x0 + 128
constexpr int kTcPlane = kTcSpx;         // pixels per channel-group plane of a ring slot
constexpr int kTcGroupRows = 4;  // output rows per accumulator
constexpr int kTcRing = 14;  // input row slots: 6 read by a row group's MMAs, the rest in flight
constexpr uint32_t kTcWaitLimit = 1u << 26;

__device__ uint32_t g_dnStatus;

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Bounded mbarrier wait (at most kTcWaitLimit polls and kTcWaitNs of
// wall time) that also gives up when another role has aborted.
constexpr uint64_t kTcWaitNs = 2000000000ull;

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, volatile uint32_t *abortFlag)
{
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < kTcWaitLimit; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
        if (*abortFlag) return false;
        if ((it & 255u) == 255u && global_ns() - t0 > kTcWaitNs) break;
    }
    *abortFlag = 1u;
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(bar) : "memory");
}

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), leading-dimension
// byte offset >> 4 (16-29), stride-dimension byte offset >> 4 (32-45),
// descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
        ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
template <int M, int N>
__device__ __forceinline__ uint32_t instr_desc_bf16()
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
        ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void softmax25(const float *l, float *w)
{
    float m = l[0];
#pragma unroll
    for (int k = 1; k < 25; k++) m = fmaxf(m, l[k]);
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 25; k++) {
        w[k] = __expf(l[k] - m);
        s += w[k];
    }
    float inv = 1.0f / s;
#pragma unroll
    for (int k = 0; k < 25; k++) w[k] *= inv;
}

__device__ __forceinline__ uint64_t tap_pixel(uint64_t p, int x, int y, int W, int H, int k)
{
    int gx = min(max(x + k % 5 - 2, 0), W - 1), gy = min(max(y + k / 5 - 2, 0), H - 1);
    return p - (uint64_t)x - (uint64_t)y * W + (uint64_t)gy * W + gx;
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// One tcgen05.mma.cta_group::1.kind::f16 (BF16 x BF16 -> FP32 in tensor
// memory); accumulate = 0 overwrites the accumulator.
__device__ __forceinline__ void tc_mma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc,
    uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :: "r"(dTmem), "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate));
}

// Bias / ReLU / BF16 packing of one pixel's COUT accumulators and the store:
// BF16 activations and FP32 gradients channel-group-planar, FP32 logits NHWC.
template <int COUT, int EPI>
__device__ __forceinline__ void conv_store(const uint32_t (&r)[COUT], size_t row, int x, int W,
    const float *__restrict__ bias, __nv_bfloat16 *__restrict__ outB, float *__restrict__ outF)
{
#pragma unroll
    for (int c = 0; c < COUT; c += 8) {
        float v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = __uint_as_float(r[c + k]);
            if (EPI != kEpiF32) v[k] += bias[c + k];
            if (EPI == kEpiBf16BiasRelu) v[k] = fmaxf(v[k], 0.0f);
        }
        if (EPI == kEpiBf16BiasRelu) {
            *reinterpret_cast<uint4 *>(outB + cg_index(row, x, c, W, COUT)) = make_uint4(
                pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                pack_bf16(v[6], v[7]));
        } else {
            float4 *o = reinterpret_cast<float4 *>(
                EPI == kEpiF32Bias ? outF + (row * W + x) * COUT + c : outF + cg_index(row, x, c, W, COUT));
            o[0] = make_float4(v[0], v[1], v[2], v[3]);
            o[1] = make_float4(v[4], v[5], v[6], v[7]);
        }
    }
}

// Softmax of the 25 kernel logits (accumulators + bias) and the 5x5 filter of
// the noisy radiance around pixel p = (x, y): the same arithmetic as k_filter
// on stored logits, so the fused and unfused results are bit-identical.
template <int COUT>
__device__ __forceinline__ void conv_filter_store(const uint32_t (&r)[COUT], size_t p, int x, int y,
    int W, int H, const float *__restrict__ bias, const float4 *__restrict__ noisy,
    float4 *__restrict__ out)
{
    static_assert(COUT >= 25, "kernel logits");
    float l[25], wk[25];
#pragma unroll
    for (int k = 0; k < 25; k++) l[k] = __uint_as_float(r[k]) + bias[k];
    softmax25(l, wk);
    float3 o = make_float3(0, 0, 0);
#pragma unroll
    for (int k = 0; k < 25; k++) {
        float4 c = __ldg(noisy + tap_pixel(p, x, y, W, H, k));
        o.x += wk[k] * c.x;
        o.y += wk[k] * c.y;
        o.z += wk[k] * c.z;
    }
    out[p] = make_float4(o.x, o.y, o.z, 1.0f);
}

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(kTcThreads, 1) k_conv3x3_tc(const __grid_constant__ CUtensorMap tmIn,
    int B, int H, int W, int rowsPerStrip, int reverseStrips, const __nv_bfloat16 *__restrict__ w,
    const float *__restrict__ bias, __nv_bfloat16 *__restrict__ outB, float *__restrict__ outF,
    const float4 *__restrict__ noisy, float4 *__restrict__ outFilt)
{
    constexpr int G = kTcGroupRows;
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && 3 * COUT <= 256, "tcgen05 tile shape");
    constexpr int KG = CIN / 8;  // 16-byte channel groups
    constexpr int ACC_COLS = G * COUT <= 128 ? 128 : 256;  // G output rows side by side
    static_assert(G * COUT <= ACC_COLS, "accumulator");
    // an even number of accumulators: accumulator a is always drained by epilogue group a % 2
    constexpr int SLOTS = 512 / ACC_COLS >= kTcAccSlots ? kTcAccSlots : 512 / ACC_COLS;
    static_assert(SLOTS % kTcEpiGroups == 0, "accumulator slots");
    constexpr int TMEM_COLS = 512;
    extern __shared__ __align__(128) unsigned char smemRaw[];
    uint4 *sW = reinterpret_cast<uint4 *>(smemRaw);  // [3][KG][3 COUT]
    // ring slots of [KG][kTcPlane] 16-byte pixels, each slot 128-byte aligned for TMA
    constexpr uint32_t kSlotBytes = (uint32_t)((KG * kTcPlane * 16 + 127) / 128 * 128);
    const uint32_t ringAddr = (smem_u32(sW + 9 * KG * COUT) + 127u) & ~127u;
    __shared__ __align__(8) uint64_t rowFull[kTcRing], rowEmpty[kTcRing];
    __shared__ __align__(8) uint64_t accFull[SLOTS], accEmpty[SLOTS], drain;
    __shared__ uint32_t tmemBase;
    __shared__ volatile uint32_t abortFlag;
    __shared__ __align__(16) float sBias[COUT];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid < COUT) sBias[tid] = EPI != kEpiF32 ? bias[tid] : 0.0f;

    // weights -> stacked canonical layout: block (tx, kg) holds 3 COUT rows of 16 B, the
    // tap rows ty = 2, 1, 0 one after the other, each row w[3 ty + tx][co][8 kg .. 8 kg + 7]
    for (int i = tid; i < 9 * KG * COUT; i += kTcThreads) {
        const int r = i % (3 * COUT), blk = i / (3 * COUT);
        const int kg = blk % KG, tx = blk / KG;
        const int ty = 2 - r / COUT, co = r % COUT;
        sW[i] = reinterpret_cast<const uint4 *>(w)[((size_t)(3 * ty + tx) * COUT + co) * KG + kg];
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmemBase)), "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < kTcRing; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&rowFull[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&rowEmpty[i])));
        }
        for (int i = 0; i < SLOTS; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&accFull[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" :: "r"(smem_u32(&accEmpty[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&drain)));
        abortFlag = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmemBase;

    const int segs = (W + kTcTileP - 1) / kTcTileP;
    const int stripsPerCol = (H + rowsPerStrip - 1) / rowsPerStrip;
    const int numStrips = B * segs * stripsPerCol;
    // strip geometry: segment origin x0, output rows [y0, y1) in P groups of G rows
    // (the last group may reach past the image); staged input rows y0 - 1 .. y0 + G P
#define GBSP_STRIP_GEOMETRY(strip)                                                       \
    const int st = reverseStrips ? numStrips - 1 - (strip) : (strip);                     \
    const int sy = st % stripsPerCol, seg = (st / stripsPerCol) % segs;                  \
    const int b = st / (stripsPerCol * segs);                                             \
    const int x0 = seg * kTcTileP, y0 = sy * rowsPerStrip;                                \
    const int y1 = min(H, y0 + rowsPerStrip);                                             \
    const int P = (y1 - y0 + G - 1) / G;                                                  \
    (void)b;                                                                              \
    (void)x0;                                                                             \
    (void)y1

    if (warp == 0) {
        if (lane == 0) {
            // ---- MMA issue.  Input row gy of a strip has sequence number qBase + gy - y0 + 1.
            // Group (y .. y + G - 1) accumulates its G output rows side by side (row y + j in
            // columns [j COUT, (j + 1) COUT)).  Input row y - 1 + k feeds output rows
            // j = max(0, k - 2) .. min(G - 1, k) through tap rows ty = k - j: one MMA whose
            // B operand is the contiguous slice of the [ty 2 | ty 1 | ty 0] weight stack.
            uint32_t idesc[4];
            idesc[1] = instr_desc_bf16<kTcTileP, COUT>();
            idesc[2] = instr_desc_bf16<kTcTileP, 2 * COUT>();
            idesc[3] = instr_desc_bf16<kTcTileP, 3 * COUT>();
            const uint64_t aDesc0 = smem_desc(ringAddr, kTcPlane * 16, 128);
            const uint64_t bDesc0 = smem_desc(smem_u32(sW), 3 * COUT * 16, 128);
            // issue order per (tx, kc): k = 2 and k = G + 1 first (their outputs tile all G
            // rows, so they can start the accumulator), then the rest
            static_assert(G == 4, "issue order below is for groups of 4 rows");
            constexpr int kOrder[G + 2] = {2, 5, 0, 1, 3, 4};
            uint32_t qBase = 0, groupCount = 0;
            bool ok = true;
            for (int strip = blockIdx.x; strip < numStrips && ok; strip += gridDim.x) {
                GBSP_STRIP_GEOMETRY(strip);
                for (int p = 0; p < P && ok; p++) {
                    const uint32_t q0 = qBase + (uint32_t)(G * p);  // input row y - 1
                    for (uint32_t q = q0; q < q0 + G + 2 && ok; q++)
                        ok = tc_wait(smem_u32(&rowFull[q % kTcRing]), (q / kTcRing) & 1u,
                            &abortFlag);
                    if (!ok) break;
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    const uint32_t acc = groupCount % SLOTS, use = groupCount / SLOTS;
                    if (use > 0 && !tc_wait(smem_u32(&accEmpty[acc]), (use - 1u) & 1u, &abortFlag)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t dAcc = tmem + acc * (uint32_t)ACC_COLS;
#pragma unroll
                    for (int tx = 0; tx < 3; tx++) {
#pragma unroll
                        for (int kc = 0; kc < CIN / 16; kc++) {
#pragma unroll
                            for (int o = 0; o < G + 2; o++) {
                                const int k = kOrder[o];
                                const int jlo = k - 2 > 0 ? k - 2 : 0, jhi = k < G - 1 ? k : G - 1;
                                const uint32_t slot = (q0 + (uint32_t)k) % kTcRing;
                                // 16-byte units: slot row, channel group 2 kc, pixel tx
                                const uint64_t aDesc = aDesc0 +
                                    (uint64_t)(slot * (kSlotBytes / 16) + 2 * kc * kTcPlane + tx);
                                // weight block (tx, 2 kc), starting at tap row ty = k - jlo
                                const uint64_t bDesc = bDesc0 +
                                    (uint64_t)((tx * KG + 2 * kc) * 3 * COUT + (2 - k + jlo) * COUT);
                                const uint32_t accumulate = (tx | kc) || o >= 2 ? 1u : 0u;
                                tc_mma(dAcc + (uint32_t)(jlo * COUT), aDesc, bDesc,
                                    idesc[jhi - jlo + 1], accumulate);
                            }
                        }
                    }
                    tc_commit(smem_u32(&accFull[acc]));
                    // input rows y - 1 .. y + G - 2 have no later reader
                    for (int k = 0; k < G; k++)
                        tc_commit(smem_u32(&rowEmpty[(q0 + (uint32_t)k) % kTcRing]));
                    groupCount++;
                }
                if (!ok) break;
                // the strip's last two input rows are free once its last MMAs finish
                const uint32_t qLast = qBase + (uint32_t)(G * P) + 1u;
                tc_commit(smem_u32(&rowEmpty[(qLast - 1u) % kTcRing]));
                tc_commit(smem_u32(&rowEmpty[qLast % kTcRing]));
                qBase = qLast + 1u;
            }
            // every MMA issued has finished before the accumulators are freed
            // (waited for even after an abort: the tensor memory is freed below)
            tc_commit(smem_u32(&drain));
            volatile uint32_t never = 0u;
            if (!tc_wait(smem_u32(&drain), 0u, &never)) abortFlag = 1u;
            if (!ok) abortFlag = 1u;
        }
        __syncwarp();
    } else if (warp < 4) {
        // ---- producer (lane 0 of warp 1): input rows y0 - 1 .. y0 + G P of every strip,
        // one TMA box per row (8 channels x 130 pixels x every channel group, zero outside
        // the image, landing as [group][pixel][8 channels]), completing the row's rowFull
        // transaction count
        if (warp == 1 && lane == 0) {
            constexpr uint32_t kRowBytes = (uint32_t)(KG * kTcSpx * 16);
            uint32_t q = 0;
            bool ok = true;
            for (int strip = blockIdx.x; strip < numStrips && ok; strip += gridDim.x) {
                GBSP_STRIP_GEOMETRY(strip);
                for (int gy = y0 - 1; gy <= y0 + G * P; gy++, q++) {
                    const uint32_t slot = q % kTcRing, use = q / kTcRing;
                    if (use > 0 && !tc_wait(smem_u32(&rowEmpty[slot]), (use - 1u) & 1u, &abortFlag)) {
                        ok = false;
                        break;
                    }
                    const uint32_t bar = smem_u32(&rowFull[slot]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                                 :: "r"(bar), "r"(kRowBytes) : "memory");
                    const uint32_t dst = ringAddr + slot * kSlotBytes;
                    asm volatile(
                        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
                        :: "r"(dst), "l"(reinterpret_cast<uint64_t>(&tmIn)), "r"(0), "r"(x0 - 1),
                           "r"(0), "r"(gy), "r"(b), "r"(bar)
                        : "memory");
                }
            }
            // every box issued has landed before the CTA's shared memory is released
            volatile uint32_t never = 0u;
            for (uint32_t s0 = 0; s0 < kTcRing && s0 < q; s0++) {
                const uint32_t lastUse = (q - 1u - ((q - 1u - s0) % kTcRing)) / kTcRing;
                if (!tc_wait(smem_u32(&rowFull[s0]), lastUse & 1u, &never)) abortFlag = 1u;
            }
            if (!ok) abortFlag = 1u;
        }
        __syncwarp();
    } else {
        // ---- epilogue: group g = (warp - 4) / 4 takes the row groups with groupCount % 2 == g;
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 (pixels)
        const int quarter = warp & 3, group = (warp - 4) >> 2;
        uint32_t groupCount = 0;
        bool ok = true;
        for (int strip = blockIdx.x; strip < numStrips && ok; strip += gridDim.x) {
            GBSP_STRIP_GEOMETRY(strip);
            for (int p = 0; p < P; p++, groupCount++) {
                if ((int)(groupCount % kTcEpiGroups) != group) continue;
                const uint32_t acc = groupCount % SLOTS, use = groupCount / SLOTS;
                ok = tc_wait(smem_u32(&accFull[acc]), use & 1u, &abortFlag);
                __syncwarp();
                if (!__all_sync(0xFFFFFFFFu, ok)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t cols = tmem + ((uint32_t)(quarter * 32) << 16) + acc * (uint32_t)ACC_COLS;
                const int x = x0 + quarter * 32 + lane;
#pragma unroll 1
                for (int j = 0; j < G; j++) {
                    const int y = y0 + G * p + j;
                    uint32_t r[COUT];
#pragma unroll
                    for (int c = 0; c < COUT; c += 16)
                        tmem_ld16(cols + (uint32_t)(j * COUT + c), *reinterpret_cast<uint32_t(*)[16]>(r + c));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (x < W && y < y1) {
                        const size_t row = (size_t)(b * H + y);
                        if constexpr (EPI == kEpiFilter)
                            conv_filter_store<COUT>(r, row * W + x, x, y, W, H, sBias, noisy,
                                outFilt);
                        else
                            conv_store<COUT, EPI>(r, row, x, W, sBias, outB, outF);
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;");
                mbar_arrive(smem_u32(&accEmpty[acc]));
            }
        }
    }
#undef GBSP_STRIP_GEOMETRY
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && abortFlag) atomicOr(&g_dnStatus, 1u);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :: "r"(tmem), "r"(TMEM_COLS));
}

// Rate probe for the MMA shape the convolutions use: one CTA, `issuers`
// threads (lane 0 of warps 0..issuers-1) each issue `iters` back-to-back
// 128 x N x 16 BF16 MMAs from zeroed shared memory into their own TMEM
// accumulator, then wait for completion.  The A operand starts aOff16 16-byte
// units past a 1,024-byte boundary (a pixel-shifted view of a staged row).
// cycles[k] = clock64 cycles of issuer k from its first issue to the
// completion of its last MMA.
template <int N>
__global__ void __launch_bounds__(64) k_tc_rate(int iters, int issuers, int aOff16,
    unsigned long long *cycles)
{
    __shared__ __align__(1024) uint4 sA[2 * 128 + 64];
    __shared__ __align__(1024) uint4 sB[2 * 256];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmemBase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 2 * 128 + 64; i += 64) sA[i] = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < 2 * 256; i += 64) sB[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmemBase)), "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < 2; i++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar[i])));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmemBase;
    if (lane == 0 && warp < issuers) {
        const uint32_t idesc = instr_desc_bf16<128, N>();
        const uint64_t a = smem_desc(smem_u32(sA + aOff16), 128 * 16, 128);
        const uint64_t b = smem_desc(smem_u32(sB), N * 16, 128);
        const uint32_t d = tmem + (uint32_t)(256 * warp);
        const long long t0 = clock64();
        for (int i = 0; i < iters; i++) {
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                :: "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(i ? 1u : 0u));
        }
        tc_commit(smem_u32(&bar[warp]));
        volatile uint32_t never = 0u;
        const bool done = tc_wait(smem_u32(&bar[warp]), 0u, &never);
        cycles[warp] = done ? (unsigned long long)(clock64() - t0) : 0ull;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(512));
}

// tcgen05 convolutions launched so far (all shapes): its parity picks the strip order.
static std::atomic<unsigned> g_convLaunches{0};

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link-time dependency on libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// TMA map of a channel-group-planar BF16 activation tensor [B][H][cin/8][W][8]
// (dimension order: 8 channels, pixel, channel group, row, image): one box =
// 8 channels x boxPixels pixels x every channel group of one row, i.e. cin/8
// contiguous runs of 16 boxPixels bytes, written to shared memory as
// [group][pixel][8 channels], zero outside the tensor.  input_tensor_map: the
// forward convolution's boxes of kTcSpx pixels.
static int planar_tensor_map(CUtensorMap *map, const void *in, int B, int H, int W, int cin,
    int boxPixels)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return set_error(GBSP_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)cin / 8, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[4] = {16, (cuuint64_t)W * 16, (cuuint64_t)W * cin * 2,
        (cuuint64_t)H * W * cin * 2};
    const cuuint32_t box[5] = {8, (cuuint32_t)boxPixels, (cuuint32_t)cin / 8, 1, 1};
    const cuuint32_t elem[5] = {1, 1, 1, 1, 1};
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(in), dims,
        strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return set_error(GBSP_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return GBSP_OK;
}

// The same tensor seen as 32-bit words [B][H][cin/8][W * 4] (dimension order:
// word, channel group, row, image): one box = boxPixels * 4 words (boxPixels
// <= 64) of every channel group of one row, landing as the same
// [group][pixel][8 channels] bytes in one 16 boxPixels-byte run per group.
// x coordinates are pixel * 4 (16-byte aligned, negative allowed).
static int planar_words_tensor_map(CUtensorMap *map, const void *in, int B, int H, int W, int cin,
    int boxPixels)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return set_error(GBSP_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    if (boxPixels < 1 || boxPixels > 64)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "box of %d pixels", boxPixels);
    const cuuint64_t dims[4] = {(cuuint64_t)W * 4, (cuuint64_t)cin / 8, (cuuint64_t)H,
        (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)W * 16, (cuuint64_t)W * cin * 2,
        (cuuint64_t)H * W * cin * 2};
    const cuuint32_t box[4] = {(cuuint32_t)boxPixels * 4, (cuuint32_t)cin / 8, 1, 1};
    const cuuint32_t elem[4] = {1, 1, 1, 1};
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, const_cast<void *>(in), dims,
        strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return set_error(GBSP_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return GBSP_OK;
}

static int input_tensor_map(CUtensorMap *map, const void *in, int B, int H, int W, int cin)
{
    return planar_tensor_map(map, in, B, H, W, cin, kTcSpx);
}

template <int CIN, int COUT, int EPI>
int launch_conv_tc(cudaStream_t s, int smCount, const void *in, int B, int H, int W, const void *w,
    const float *bias, void *outB, float *outF, const float4 *noisy = nullptr,
    float4 *outFilt = nullptr)
{
    // weights, then the ring (rounded up to a 128-byte boundary inside the kernel)
    size_t smem = (size_t)9 * (CIN / 8) * COUT * 16 +
        (size_t)kTcRing * (((CIN / 8) * kTcPlane * 16 + 127) / 128 * 128) + 128;
    auto kern = k_conv3x3_tc<CIN, COUT, EPI>;
    GBSP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUtensorMap map;
    int rc = input_tensor_map(&map, in, B, H, W, CIN);
    if (rc) return rc;
    const int ctas = smCount;  // one CTA per SM (the row ring takes most of shared memory)
    const int cols = B * ((W + kTcTileP - 1) / kTcTileP);
    // rows per strip: about six strips per CTA (strips go round-robin, so
    // the last round is nearly full), at least 4 rows
    int rows = (int)(((int64_t)cols * H + 6 * ctas - 1) / (6 * ctas));
    rows = rows < 4 ? 4 : (rows > H ? H : rows);
    rows = (rows + kTcGroupRows - 1) / kTcGroupRows * kTcGroupRows;  // whole row groups
    int strips = cols * ((H + rows - 1) / rows);
    int grid = strips < ctas ? strips : ctas;
    // consecutive convolutions walk the strips in opposite orders, so a layer
    // starts on the rows its predecessor wrote last (still in L2)
    const int reverse = (int)(g_convLaunches.fetch_add(1, std::memory_order_relaxed) & 1u);
    kern<<<grid, kTcThreads, smem, s>>>(map, B, H, W, rows, reverse,
        reinterpret_cast<const __nv_bfloat16 *>(w), bias, reinterpret_cast<__nv_bfloat16 *>(outB),
        outF, noisy, outFilt);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

// Input features: log(1 + radiance), albedo, normal, depth/(1 + depth),
// zero-padded to 16 channels.
__global__ void k_features(const float4 *__restrict__ rad, const float4 *__restrict__ aov,
    uint64_t n, int W, __nv_bfloat16 *__restrict__ out)
{
    uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    float4 r = rad[p];
    float4 a = aov[2 * p], nn = aov[2 * p + 1];
    float d = fmaxf(a.w, 0.0f);
    float f[16] = {log1pf(fmaxf(r.x, 0.0f)), log1pf(fmaxf(r.y, 0.0f)), log1pf(fmaxf(r.z, 0.0f)),
        a.x, a.y, a.z, nn.x, nn.y, nn.z, d / (1.0f + d), 0, 0, 0, 0, 0, 0};
    const size_t row = p / (uint64_t)W;
    const int x = (int)(p % (uint64_t)W);
#pragma unroll
    for (int g = 0; g < 2; g++)
        *reinterpret_cast<uint4 *>(out + cg_index(row, x, 8 * g, W, 16)) = make_uint4(
            pack_bf16(f[8 * g], f[8 * g + 1]), pack_bf16(f[8 * g + 2], f[8 * g + 3]),
            pack_bf16(f[8 * g + 4], f[8 * g + 5]), pack_bf16(f[8 * g + 6], f[8 * g + 7]));
}

// w'[8 - tap][ci][co] = w[tap][co][ci]: weights of the data-gradient conv.
__global__ void k_flip_transpose(const __nv_bfloat16 *w, int cout, int cin, __nv_bfloat16 *wt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * cout * cin) return;
    int tap = i / (cout * cin), r = i % (cout * cin), co = r / cin, ci = r % cin;
    wt[((8 - tap) * cin + ci) * cout + co] = w[i];
}

// d = dAct * (act > 0) as BF16 (ReLU backward).
__global__ void k_relu_bwd(const float *__restrict__ dAct, const __nv_bfloat16 *__restrict__ act,
    uint64_t n, __nv_bfloat16 *__restrict__ out)
{
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a = __bfloat162float(act[i]);
    out[i] = __float2bfloat16_rn(a > 0.0f ? dAct[i] : 0.0f);
}

// dW[tap][co][ci] += sum_p d[p][co] * in[p + off(tap)][ci]; dBias[co] += sum_p d[p][co].
// CTA = (pixel chunk, tap); 128 threads, each owns a (COUT/8 x CIN/16) block.
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3x3_wgrad(const __nv_bfloat16 *__restrict__ in,
    const __nv_bfloat16 *__restrict__ d, int B, int H, int W, int chunk, float *dW, float *dBias)
{
    constexpr int TC = COUT / 8, TI = CIN / 16;  // 8 x 16 thread grid
    constexpr int STAGE = 32;                    // pixels staged per iteration
    __shared__ float sD[STAGE][COUT];
    __shared__ float sI[STAGE][CIN];
    const int tap = blockIdx.y, dy = tap / 3 - 1, dx = tap % 3 - 1;
    const uint64_t N = (uint64_t)B * H * W;
    const uint64_t p0 = (uint64_t)blockIdx.x * chunk;
    const int tco = threadIdx.x / 16, tci = threadIdx.x % 16;
    float acc[TC][TI];
#pragma unroll
    for (int a = 0; a < TC; a++)
#pragma unroll
        for (int c = 0; c < TI; c++) acc[a][c] = 0.0f;
    float bacc = 0.0f;
    for (int base = 0; base < chunk; base += STAGE) {
        __syncthreads();
        for (int i = threadIdx.x; i < STAGE * COUT; i += 128) {
            int k = i / COUT, co = i % COUT;
            uint64_t p = p0 + base + k;
            sD[k][co] = p < N ? __bfloat162float(d[cg_index(p / W, (int)(p % W), co, W, COUT)]) : 0.0f;
        }
        for (int i = threadIdx.x; i < STAGE * CIN; i += 128) {
            int k = i / CIN, ci = i % CIN;
            uint64_t p = p0 + base + k;
            float v = 0.0f;
            if (p < N) {
                int x = (int)(p % W), y = (int)((p / W) % H);
                int gx = x + dx, gy = y + dy;
                if (gx >= 0 && gx < W && gy >= 0 && gy < H)
                    v = __bfloat162float(in[cg_index(p / W + dy, gx, ci, W, CIN)]);
            }
            sI[k][ci] = v;
        }
        __syncthreads();
        for (int k = 0; k < STAGE; k++) {
            float dv[TC], iv[TI];
#pragma unroll
            for (int a = 0; a < TC; a++) dv[a] = sD[k][tco * TC + a];
#pragma unroll
            for (int c = 0; c < TI; c++) iv[c] = sI[k][tci * TI + c];
#pragma unroll
            for (int a = 0; a < TC; a++)
#pragma unroll
                for (int c = 0; c < TI; c++) acc[a][c] += dv[a] * iv[c];
            if (tap == 4 && threadIdx.x < COUT) bacc += sD[k][threadIdx.x];
        }
    }
#pragma unroll
    for (int a = 0; a < TC; a++)
#pragma unroll
        for (int c = 0; c < TI; c++)
            atomicAdd(&dW[((size_t)tap * COUT + tco * TC + a) * CIN + tci * TI + c], acc[a][c]);
    if (tap == 4 && threadIdx.x < COUT) atomicAdd(&dBias[threadIdx.x], bacc);
}

// Weight gradient on the tensor cores (mma.sync m16n8k16, BF16 in, FP32
// accumulate): per tap, dW[tap][co][ci] = sum_p d[p][co] * x[p + off(tap)][ci]
// is a GEMM with M = COUT, N = CIN and K = pixels.  A CTA of 9 warps (warp =
// tap) walks 64-pixel row segments: it stages d transposed ([co][pixel]) and
// the three input rows around the segment transposed ([row][ci][pixel], one
// pixel of halo on each side), then every warp multiplies its tap's shifted
// view, holding all COUT/16 x CIN/8 accumulator tiles in registers.  Each CTA
// writes its partial sums (and the bias gradient sum_p d[p][co]) to its own
// slice of a scratch buffer; k_wgrad_reduce adds the slices in a fixed order,
// so the result is deterministic.
constexpr int kWgTile = 64;
constexpr int kWgStride = kWgTile + 8;  // padded pixel stride of the staged rows

template <int CIN, int COUT>
__global__ void __launch_bounds__(288) k_conv3x3_wgrad_tc(const __nv_bfloat16 *__restrict__ in,
    const __nv_bfloat16 *__restrict__ d, int B, int H, int W, float *__restrict__ partial)
{
    static_assert(CIN % 8 == 0 && COUT % 16 == 0, "tile shape");
    constexpr int MT = COUT / 16, NT = CIN / 8;
    __shared__ __align__(16) __nv_bfloat16 sD[COUT][kWgStride];
    __shared__ __align__(16) __nv_bfloat16 sX[3][CIN][kWgStride];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int tap = warp, ty = tap / 3, tx = tap % 3;
    float acc[MT][NT][4];
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
        for (int n = 0; n < NT; n++) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.0f;
    float bacc = 0.0f;  // threads 0..COUT-1: bias gradient of channel tid
    const int segs = (W + kWgTile - 1) / kWgTile;
    const int tiles = segs * B * H;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int row = tile / segs, x0 = (tile % segs) * kWgTile;
        const int b = row / H, y = row % H;
        __syncthreads();
        // staging: one 16-byte load per (pixel, 8-channel group) of the planar
        // tensors (consecutive threads take consecutive pixels of one plane),
        // spread over the transposed [channel][pixel] tiles
        for (int i = tid; i < kWgTile * (COUT / 8); i += 288) {
            const int k = i % kWgTile, cg = i / kWgTile, x = x0 + k;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (x < W) v = *reinterpret_cast<const uint4 *>(d + cg_index((size_t)row, x, 8 * cg, W, COUT));
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int j = 0; j < 8; j++) sD[8 * cg + j][k] = e[j];
        }
        for (int i = tid; i < 3 * (kWgTile + 2) * (CIN / 8); i += 288) {
            const int px = i % (kWgTile + 2), cg = (i / (kWgTile + 2)) % (CIN / 8);
            const int ry = i / ((kWgTile + 2) * (CIN / 8));
            const int gy = y + ry - 1, gx = x0 + px - 1;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (gy >= 0 && gy < H && gx >= 0 && gx < W)
                v = *reinterpret_cast<const uint4 *>(in + cg_index((size_t)(b * H + gy), gx, 8 * cg, W, CIN));
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int j = 0; j < 8; j++) sX[ry][8 * cg + j][px] = e[j];
        }
        __syncthreads();
        if (tid < COUT) {
            for (int k = 0; k < kWgTile; k++) bacc += __bfloat162float(sD[tid][k]);
        }
#pragma unroll
        for (int k0 = 0; k0 < kWgTile; k0 += 16) {
            uint32_t a[MT][4];
#pragma unroll
            for (int m = 0; m < MT; m++) {
                const __nv_bfloat16 *r0 = &sD[m * 16 + g][k0 + 2 * t];
                const __nv_bfloat16 *r1 = &sD[m * 16 + g + 8][k0 + 2 * t];
                a[m][0] = *reinterpret_cast<const uint32_t *>(r0);
                a[m][1] = *reinterpret_cast<const uint32_t *>(r1);
                a[m][2] = *reinterpret_cast<const uint32_t *>(r0 + 8);
                a[m][3] = *reinterpret_cast<const uint32_t *>(r1 + 8);
            }
#pragma unroll
            for (int n = 0; n < NT; n++) {
                // B[k][ci] = x[pixel k + tx - 1 of the segment][ci]: the staged row ty
                // at halo index k + tx (odd for tx = 1: two 16-bit loads per pair)
                const __nv_bfloat16 *c = &sX[ty][n * 8 + g][k0 + 2 * t + tx];
                __nv_bfloat162 p0, p1;
                p0.x = c[0];
                p0.y = c[1];
                p1.x = c[8];
                p1.y = c[9];
                uint32_t b0 = *reinterpret_cast<uint32_t *>(&p0);
                uint32_t b1 = *reinterpret_cast<uint32_t *>(&p1);
#pragma unroll
                for (int m = 0; m < MT; m++)
                    mma_bf16_16816(acc[m][n], a[m][0], a[m][1], a[m][2], a[m][3], b0, b1);
            }
        }
    }
    // C fragment: rows g / g + 8 (co), columns 2t, 2t + 1 (ci) of each tile
    float *out = partial + (size_t)blockIdx.x * (9 * COUT * CIN + COUT);
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
        for (int n = 0; n < NT; n++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                int co = m * 16 + g + 8 * h, ci = n * 8 + 2 * t;
                float *o = out + ((size_t)tap * COUT + co) * CIN + ci;
                o[0] = acc[m][n][2 * h];
                o[1] = acc[m][n][2 * h + 1];
            }
    if (tid < COUT) out[9 * COUT * CIN + tid] = bacc;
}

// dW[i] += sum over CTA slices of partial[slice][i], slices in order; the
// last COUT entries of a slice are the bias gradient.
__global__ void k_wgrad_reduce(const float *__restrict__ partial, int slices, int perSlice,
    int wCount, float *dW, float *dBias)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= perSlice) return;
    float sum = 0.0f;
    for (int k = 0; k < slices; k++) sum += partial[(size_t)k * perSlice + i];
    if (i < wCount)
        dW[i] += sum;
    else
        dBias[i - wCount] += sum;
}

// ---------------------------------------------------------------------------
// Weight gradient on the 5th-generation tensor cores (tcgen05), fed by TMA.
//
// dW[ty 3 + tx][co][ci] = sum_p d[y][p][co] x[y + ty - 1][p + tx - 1][ci] over
// every output pixel (b, y, p).  Substituting the input pixel q = p + tx - 1,
// one GEMM per input-row chunk gives all nine taps at once:
//   D[(ty, ci)][(tx, co)] = sum_q x[y + ty - 1][q][ci] d[y][q - tx + 1][co],
// M = 3 CIN rows (two M = 128 MMAs when CIN = 48, one when CIN = 16), N = 3
// COUT, K = 64 input pixels q of a chunk (4 MMAs of K = 16 per M block).
//
// Both operands are MN-major, which is the channel-group-planar layout
// itself: a core matrix (8 pixels along K x 8 channels along M or N, one
// 16-byte row per pixel) is 128 contiguous bytes of one channel group, so the
// leading (K) byte offset is 128 and the stride (M / N) byte offset is one
// 8-channel block.  A chunk's operands are six TMA boxes of [group][64
// pixels][8 channels] (the tensor seen as 32-bit words, so that a box is one
// 1 KB run per channel group): the three input rows (A, one 1 KB block per
// (ty, group)) and three copies of the output-gradient row shifted by one pixel
// each (B, one block per (tx, group)), zero outside the tensor; nothing is
// transposed in registers.  A block of ones after the input rows makes
// accumulator row 3 CIN the sum of d over the chunk: with column block
// tx = 1, the bias gradient.
//
// One persistent CTA per SM walks its chunks (b, y, 64-pixel segment) through
// a ring of kWtStages stages: lane 0 of warp 0 waits for a free stage (its
// `empty` barrier, committed by the MMAs that read it) and issues the six
// loads against the stage's `full` transaction count; lane 0 of warp 1 waits
// on `full` and issues the MMAs into FP32 accumulators in tensor memory that
// persist over all of the CTA's chunks.  At the end the warps read the
// accumulators and write the CTA's partial sums to its slice of a scratch
// buffer; k_wgrad_reduce adds the slices in a fixed order (deterministic).
// Every wait is bounded and raises g_dnStatus on timeout.
// ---------------------------------------------------------------------------
constexpr int kWtPx = 64;
constexpr int kWtStages = 4;
constexpr int kWtThreads = 256;

template <int CIN, int COUT>
struct WtShape {
    static constexpr int KGI = CIN / 8, KGO = COUT / 8;
    static constexpr int MROWS = 3 * CIN, N = 3 * COUT;
    static constexpr int MB = (MROWS + 8 + 127) / 128;          // M = 128 blocks, with the ones
    static constexpr uint32_t kBlock = kWtPx * 16;              // 8 rows x 64 pixels: 1 KB
    static constexpr uint32_t kBOff = (3 * KGI + 1) * kBlock;   // input rows, then the ones
    static constexpr uint32_t kBBytes = 3 * KGO * kBlock;
    static constexpr uint32_t kAExtent = MB * 16 * kBlock;      // what the M = 128 MMAs read
    static constexpr uint32_t kStage =
        ((kBOff + kBBytes > kAExtent ? kBOff + kBBytes : kAExtent) + 1023u) / 1024u * 1024u;
    static constexpr uint32_t kTxBytes = (uint32_t)(3 * KGI + 3 * KGO) * kBlock;
    static constexpr int TMEM_COLS = MB * N <= 256 ? 256 : 512;
    static_assert(CIN % 8 == 0 && COUT % 16 == 0 && N <= 256 && MB * N <= 512, "tile shape");
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(kWtThreads, 1) k_conv3x3_wgrad_tma(
    const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmD, int B, int H,
    int W, float *__restrict__ partial)
{
    using S = WtShape<CIN, COUT>;
    constexpr int N = S::N, MB = S::MB, MROWS = S::MROWS;
    // the ring starts at the first 1 KB boundary (the launch adds 1 KB of slack)
    extern __shared__ __align__(128) unsigned char smemRaw[];
    const uint32_t base = (smem_u32(smemRaw) + 1023u) & ~1023u;
    __shared__ __align__(8) uint64_t full[kWtStages], empty[kWtStages], done;
    __shared__ uint32_t tmemBase;
    __shared__ volatile uint32_t abortFlag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // the ones block of every stage (BF16 1.0 pairs), written once
    for (int k = tid; k < kWtStages * (int)(S::kBlock / 4); k += kWtThreads) {
        const uint32_t st = (uint32_t)k / (S::kBlock / 4), w = (uint32_t)k % (S::kBlock / 4);
        asm volatile("st.shared.u32 [%0], %1;" :: "r"(base + st * S::kStage + (uint32_t)(3 * S::KGI) *
            S::kBlock + 4u * w), "r"(0x3F803F80u) : "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmemBase)), "r"(S::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < kWtStages; i++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&full[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&empty[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&done)));
        abortFlag = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmemBase;
    const int segs = (W + kWtPx - 1) / kWtPx;
    const int chunks = B * H * segs;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t i = 0;
            bool ok = true;
            for (int c = blockIdx.x; c < chunks && ok; c += gridDim.x, i++) {
                const uint32_t st = i % kWtStages, use = i / kWtStages;
                if (use > 0 && !(ok = tc_wait(smem_u32(&empty[st]), (use - 1u) & 1u, &abortFlag)))
                    break;
                const int seg = c % segs, row = c / segs;
                const int b = row / H, y = row % H, x0 = seg * kWtPx;
                const uint32_t bar = smem_u32(&full[st]), sb = base + st * S::kStage;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                             :: "r"(bar), "r"(S::kTxBytes) : "memory");
#pragma unroll
                // word coordinates: pixel * 4 (a 16-byte multiple)
                for (int t = 0; t < 3; t++) {
                    asm volatile(
                        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4, %5}], [%6];"
                        :: "r"(sb + (uint32_t)(t * S::KGI) * S::kBlock),
                           "l"(reinterpret_cast<uint64_t>(&tmX)), "r"(4 * x0), "r"(0),
                           "r"(y + t - 1), "r"(b), "r"(bar)
                        : "memory");
                    asm volatile(
                        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4, %5}], [%6];"
                        :: "r"(sb + S::kBOff + (uint32_t)(t * S::KGO) * S::kBlock),
                           "l"(reinterpret_cast<uint64_t>(&tmD)), "r"(4 * (x0 + 1 - t)), "r"(0),
                           "r"(y), "r"(b), "r"(bar)
                        : "memory");
                }
            }
            // every box issued has landed before the CTA's shared memory is released
            volatile uint32_t never = 0u;
            for (uint32_t s0 = 0; s0 < (uint32_t)kWtStages && s0 < i; s0++) {
                const uint32_t lastUse = (i - 1u - ((i - 1u - s0) % kWtStages)) / kWtStages;
                if (!tc_wait(smem_u32(&full[s0]), lastUse & 1u, &never)) abortFlag = 1u;
            }
            if (!ok) abortFlag = 1u;
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // A and B MN-major (instruction descriptor bits 15 and 16)
            const uint32_t idesc = instr_desc_bf16<128, N>() | (1u << 15) | (1u << 16);
            uint32_t i = 0;
            bool ok = true;
            for (int c = blockIdx.x; c < chunks && ok; c += gridDim.x, i++) {
                const uint32_t st = i % kWtStages, use = i / kWtStages;
                if (!(ok = tc_wait(smem_u32(&full[st]), use & 1u, &abortFlag))) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t aAddr = base + st * S::kStage, bAddr = aAddr + S::kBOff;
#pragma unroll
                for (int kk = 0; kk < kWtPx / 16; kk++) {
                    // K-adjacent core matrices (8 pixels) 128 B apart, M- or N-adjacent
                    // ones (8 channels) one block apart
                    const uint64_t bDesc = smem_desc(bAddr + (uint32_t)kk * 256u, 128, S::kBlock);
#pragma unroll
                    for (int mb = 0; mb < MB; mb++) {
                        const uint64_t aDesc = smem_desc(aAddr + (uint32_t)(mb * 16) * S::kBlock +
                            (uint32_t)kk * 256u, 128, S::kBlock);
                        tc_mma(tmem + (uint32_t)(mb * N), aDesc, bDesc, idesc,
                            (i > 0 || kk > 0) ? 1u : 0u);
                    }
                }
                tc_commit(smem_u32(&empty[st]));
            }
            // every MMA issued has finished before the accumulators are read
            // or freed (waited for even after an abort)
            tc_commit(smem_u32(&done));
            volatile uint32_t never = 0u;
            if (!tc_wait(smem_u32(&done), 0u, &never)) abortFlag = 1u;
            if (!ok) abortFlag = 1u;
        }
        __syncwarp();
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // ---- epilogue: warp w < 4 MB reads TMEM lanes 32 (w % 4) .. + 31 of M block w / 4:
    // accumulator row R = (ty, ci), or MROWS for the bias; column n = (tx, co)
    float *out = partial + (size_t)blockIdx.x * (9 * COUT * CIN + COUT);
    if (blockIdx.x >= chunks) {
        // no chunk: nothing accumulated (the launch sizes the grid to avoid this)
        for (int k = tid; k < 9 * COUT * CIN + COUT; k += kWtThreads) out[k] = 0.0f;
    } else if (!abortFlag && warp < 4 * MB) {
        const int mb = warp >> 2, quarter = warp & 3;
        const int R = mb * 128 + quarter * 32 + lane;
        const int ty = R / CIN, ci = R % CIN;
#pragma unroll 1
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t v[16];
            tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(mb * N + c0), v);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (R < MROWS) {
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int n = c0 + k, tx = n / COUT, co = n % COUT;
                    out[((size_t)(3 * ty + tx) * COUT + co) * CIN + ci] = __uint_as_float(v[k]);
                }
            } else if (R == MROWS) {
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int n = c0 + k;
                    if (n / COUT == 1) out[9 * COUT * CIN + n % COUT] = __uint_as_float(v[k]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && abortFlag) atomicOr(&g_dnStatus, 1u);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :: "r"(tmem), "r"(S::TMEM_COLS));
}

// Per-pixel 5x5 filter from softmax(logits[0..24]) applied to the noisy
// radiance (clamped to the image edge).
__global__ void k_filter(const float *__restrict__ logits, const float4 *__restrict__ noisy, int B,
    int H, int W, float4 *__restrict__ out)
{
    uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (p >= (uint64_t)B * H * W) return;
    int x = (int)(p % W), y = (int)((p / W) % H);
    float l[25], w[25];
#pragma unroll
    for (int k = 0; k < 25; k++) l[k] = logits[p * 32 + k];
    softmax25(l, w);
    float3 o = make_float3(0, 0, 0);
#pragma unroll
    for (int k = 0; k < 25; k++) {
        float4 c = noisy[tap_pixel(p, x, y, W, H, k)];
        o.x += w[k] * c.x;
        o.y += w[k] * c.y;
        o.z += w[k] * c.z;
    }
    out[p] = make_float4(o.x, o.y, o.z, 1.0f);
}

// Per-tile error check of a denoised frame against the plain path tracer.
// A (the denoiser's input) and C are two independent plain renders with the
// same spp, D the denoised A.  For unbiased plain estimates with variance s^2,
// E[(D - C)^2] = (D - mu)^2 + s^2 and E[(A - C)^2] = 2 s^2, so per pixel and
// channel (D - C)^2 - (A - C)^2 / 2 estimates the denoiser's squared error;
// divided by D^2 + 0.01 and averaged over a tile it estimates the tile's
// relMSE.  The per-pixel terms are noisy at low spp, so a tile falls back
// only when the bound lies below the estimate by more than kFallbackZ
// standard errors of the tile mean (a one-sided test at about 98%): then it
// is served from the plain samples, (A + C) / 2; the others keep D.  One CTA of 256 threads per tile
// (tile <= 16 x 16).  tileErr[t] receives the estimate, flags[t] 1 when the
// tile fell back.
constexpr float kFallbackZ = 2.0f;

__global__ void __launch_bounds__(256) k_tile_fallback(const float4 *__restrict__ D,
    const float4 *__restrict__ A, const float4 *__restrict__ C, int B, int H, int W, int tile,
    float bound, float4 *__restrict__ out, float *__restrict__ tileErr, uint32_t *__restrict__ flags)
{
    const int tilesX = (W + tile - 1) / tile, tilesY = (H + tile - 1) / tile;
    const int t = blockIdx.x;
    const int b = t / (tilesX * tilesY), ty = (t / tilesX) % tilesY, tx = t % tilesX;
    const int lx = threadIdx.x % tile, ly = threadIdx.x / tile;
    const int x = tx * tile + lx, y = ty * tile + ly;
    const bool in = threadIdx.x < tile * tile && x < W && y < H;
    const size_t p = ((size_t)b * H + y) * W + x;
    float e = 0.0f, e2 = 0.0f, n = 0.0f;
    float4 d = make_float4(0, 0, 0, 0), a = d, c = d;
    if (in) {
        d = D[p];
        a = A[p];
        c = C[p];
        float dv[3] = {d.x, d.y, d.z}, av[3] = {a.x, a.y, a.z}, cv[3] = {c.x, c.y, c.z};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float dc = dv[k] - cv[k], ac = av[k] - cv[k];
            const float term = (dc * dc - 0.5f * ac * ac) / (dv[k] * dv[k] + 0.01f);
            e += term;
            e2 += term * term;
        }
        n = 3.0f;
    }
    __shared__ float sE[8], sE2[8], sN[8];
    for (int off = 16; off; off >>= 1) {
        e += __shfl_xor_sync(0xFFFFFFFFu, e, off);
        e2 += __shfl_xor_sync(0xFFFFFFFFu, e2, off);
        n += __shfl_xor_sync(0xFFFFFFFFu, n, off);
    }
    if ((threadIdx.x & 31) == 0) {
        sE[threadIdx.x >> 5] = e;
        sE2[threadIdx.x >> 5] = e2;
        sN[threadIdx.x >> 5] = n;
    }
    __syncthreads();
    float te = 0.0f, te2 = 0.0f, tn = 0.0f;
    for (int k = 0; k < 8; k++) {
        te += sE[k];
        te2 += sE2[k];
        tn += sN[k];
    }
    const float est = tn > 0.0f ? te / tn : 0.0f;
    // standard error of the tile mean from the spread of its per-pixel terms
    const float var = tn > 1.0f ? fmaxf(te2 - te * est, 0.0f) / (tn - 1.0f) : 0.0f;
    const float se = tn > 0.0f ? sqrtf(var / tn) : 0.0f;
    const bool fallback = est - kFallbackZ * se > bound;
    if (threadIdx.x == 0) {
        tileErr[t] = est;
        flags[t] = fallback ? 1u : 0u;
    }
    if (in)
        out[p] = fallback ? make_float4(0.5f * (a.x + c.x), 0.5f * (a.y + c.y), 0.5f * (a.z + c.z), 1.0f)
                          : d;
}

// Served-output check of a denoised frame D against the plain path tracer,
// per tile x tile block.  A: the plain render D was denoised from (sppA
// samples per pixel); C: an independent plain render (sppC).  Per value v
// (pixel and RGB channel), with sigma^2 the per-sample variance of the
// pixel's estimator:
//   E[(D - C)^2] = (D - mu)^2 + sigma^2 / sppC,
//   E[(A - C)^2] = sigma^2 (1 / sppA + 1 / sppC),
// so (D - C)^2 - (A - C)^2 * sppA / (sppA + sppC) estimates D's squared error
// without bias, and (A - C)^2 * sppA * sppC / (sppA + sppC) estimates
// sigma^2.  tileErr = the tile mean of the first over (D^2 + 0.01); the tile
// is flagged when that estimate exceeds `bound` by more than kFallbackZ
// standard errors of the mean.  needSpp = the plain samples per pixel that
// reach `bound` on the tile, margin x mean(sigma^2 / (M^2 + 0.01)) / bound
// with M the pooled plain mean (margin > 1 covers the noise of the variance
// estimate), at least 1 and at most maxSpp.
__global__ void __launch_bounds__(256) k_tile_check(const float4 *__restrict__ D,
    const float4 *__restrict__ A, float sppA, const float4 *__restrict__ C, float sppC, int B,
    int H, int W, int tile, float bound, float margin, uint32_t maxSpp, float *__restrict__ tileErr,
    uint32_t *__restrict__ flags, uint32_t *__restrict__ needSpp)
{
    const int tilesX = (W + tile - 1) / tile, tilesY = (H + tile - 1) / tile;
    const int t = blockIdx.x;
    const int b = t / (tilesX * tilesY), ty = (t / tilesX) % tilesY, tx = t % tilesX;
    const int lx = threadIdx.x % tile, ly = threadIdx.x / tile;
    const int x = tx * tile + lx, y = ty * tile + ly;
    const bool in = threadIdx.x < tile * tile && x < W && y < H;
    const float wVarC = sppA / (sppA + sppC), wVar = sppA * sppC / (sppA + sppC);
    const float wA = sppA / (sppA + sppC), wC = sppC / (sppA + sppC);
    float e = 0.0f, e2 = 0.0f, n = 0.0f, r1 = 0.0f;
    if (in) {
        const size_t p = ((size_t)b * H + y) * W + x;
        const float4 d = D[p], a = A[p], c = C[p];
        float dv[3] = {d.x, d.y, d.z}, av[3] = {a.x, a.y, a.z}, cv[3] = {c.x, c.y, c.z};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float dc = dv[k] - cv[k], ac = av[k] - cv[k];
            const float term = (dc * dc - wVarC * ac * ac) / (dv[k] * dv[k] + 0.01f);
            e += term;
            e2 += term * term;
            const float m = wA * av[k] + wC * cv[k];
            r1 += wVar * ac * ac / (m * m + 0.01f);
        }
        n = 3.0f;
    }
    __shared__ float sE[8], sE2[8], sN[8], sR[8];
    for (int off = 16; off; off >>= 1) {
        e += __shfl_xor_sync(0xFFFFFFFFu, e, off);
        e2 += __shfl_xor_sync(0xFFFFFFFFu, e2, off);
        n += __shfl_xor_sync(0xFFFFFFFFu, n, off);
        r1 += __shfl_xor_sync(0xFFFFFFFFu, r1, off);
    }
    if ((threadIdx.x & 31) == 0) {
        sE[threadIdx.x >> 5] = e;
        sE2[threadIdx.x >> 5] = e2;
        sN[threadIdx.x >> 5] = n;
        sR[threadIdx.x >> 5] = r1;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    float te = 0.0f, te2 = 0.0f, tn = 0.0f, tr = 0.0f;
    for (int k = 0; k < 8; k++) {
        te += sE[k];
        te2 += sE2[k];
        tn += sN[k];
        tr += sR[k];
    }
    const float est = tn > 0.0f ? te / tn : 0.0f;
    const float var = tn > 1.0f ? fmaxf(te2 - te * est, 0.0f) / (tn - 1.0f) : 0.0f;
    const float se = tn > 0.0f ? sqrtf(var / tn) : 0.0f;
    tileErr[t] = est;
    flags[t] = est - kFallbackZ * se > bound ? 1u : 0u;
    const float need = tn > 0.0f ? margin * (tr / tn) / bound : 1.0f;
    needSpp[t] = need >= (float)maxSpp ? maxSpp : (uint32_t)fmaxf(1.0f, ceilf(need));
}

// Served frame: D on unflagged tiles; on flagged tiles the mean of every
// plain sample of the pixel, (sppA A + sppC C + sppF[t] F) / (sppA + sppC +
// sppF[t]) with F the fallback render of the tile (sppF[t] = 0: none).
__global__ void __launch_bounds__(256) k_tile_merge(const float4 *__restrict__ D,
    const float4 *__restrict__ A, float sppA, const float4 *__restrict__ C, float sppC,
    const float4 *__restrict__ F, const uint32_t *__restrict__ sppF, int B, int H, int W,
    int tile, const uint32_t *__restrict__ flags, float4 *__restrict__ out)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (size_t)B * H * W) return;
    const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((size_t)W * H));
    const int tilesX = (W + tile - 1) / tile, tilesY = (H + tile - 1) / tile;
    const int t = (b * tilesY + y / tile) * tilesX + x / tile;
    if (!flags[t]) {
        out[p] = D[p];
        return;
    }
    const float f = F ? (float)sppF[t] : 0.0f;
    const float inv = 1.0f / (sppA + sppC + f);
    const float4 a = A[p], c = C[p];
    const float4 g = f > 0.0f ? F[p] : make_float4(0, 0, 0, 0);
    out[p] = make_float4((sppA * a.x + sppC * c.x + f * g.x) * inv,
        (sppA * a.y + sppC * c.y + f * g.y) * inv, (sppA * a.z + sppC * c.z + f * g.z) * inv, 1.0f);
}

// relMSE = mean over pixels and channels of (out - ref)^2 / (ref^2 + 0.01);
// writes dLogits (BF16, 32 channels, zeros beyond 25) and adds the loss sum.
__global__ void k_relmse_bwd(const float *__restrict__ logits, const float4 *__restrict__ noisy,
    const float4 *__restrict__ target, int B, int H, int W, float invCount,
    __nv_bfloat16 *__restrict__ dLogits, float *lossSum)
{
    uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    float loss = 0.0f;
    if (p < (uint64_t)B * H * W) {
        int x = (int)(p % W), y = (int)((p / W) % H);
        float l[25], w[25];
#pragma unroll
        for (int k = 0; k < 25; k++) l[k] = logits[p * 32 + k];
        softmax25(l, w);
        float3 o = make_float3(0, 0, 0);
        uint64_t tp[25];
#pragma unroll
        for (int k = 0; k < 25; k++) {
            tp[k] = tap_pixel(p, x, y, W, H, k);
            float4 c = noisy[tp[k]];
            o.x += w[k] * c.x;
            o.y += w[k] * c.y;
            o.z += w[k] * c.z;
        }
        float4 r = target[p];
        float ex = o.x - r.x, ey = o.y - r.y, ez = o.z - r.z;
        float nx = 1.0f / (r.x * r.x + 0.01f), ny = 1.0f / (r.y * r.y + 0.01f),
              nz = 1.0f / (r.z * r.z + 0.01f);
        loss = ex * ex * nx + ey * ey * ny + ez * ez * nz;
        float gx = 2.0f * ex * nx * invCount, gy = 2.0f * ey * ny * invCount,
              gz = 2.0f * ez * nz * invCount;
        float gk[25], dot = 0.0f;
#pragma unroll
        for (int k = 0; k < 25; k++) {
            float4 c = noisy[tp[k]];
            gk[k] = gx * c.x + gy * c.y + gz * c.z;
            dot += w[k] * gk[k];
        }
        const size_t row = p / (uint64_t)W;
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
            float v0 = k < 25 ? w[k] * (gk[k] - dot) : 0.0f;
            float v1 = k + 1 < 25 ? w[k + 1] * (gk[k + 1] - dot) : 0.0f;
            reinterpret_cast<uint32_t *>(dLogits)[cg_index(row, x, k, W, 32) / 2] = pack_bf16(v0, v1);
        }
    }
    for (int off = 16; off; off >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(lossSum, loss);
}

__global__ void k_adam(float *param, __nv_bfloat16 *paramBf16, const float *grad, float *m,
    float *v, uint64_t n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = grad[i];
    float mi = b1 * m[i] + (1.0f - b1) * g;
    float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float p = param[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    param[i] = p;
    if (paramBf16) paramBf16[i] = __float2bfloat16_rn(p);
}

inline unsigned blocks(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace dn
}  // namespace gbsp

using namespace gbsp;
using namespace gbsp::dn;

template <int CIN, int COUT>
static int launch_wgrad_tc(cudaStream_t s, const __nv_bfloat16 *in, const __nv_bfloat16 *d, int B,
    int H, int W, float *dW, float *dBias)
{
    const int tiles = ((W + kWgTile - 1) / kWgTile) * B * H;
    int perSm = 1;
    GBSP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm,
        k_conv3x3_wgrad_tc<CIN, COUT>, 288, 0));
    int grid = sm_count() * (perSm > 0 ? perSm : 1);
    if (grid > tiles) grid = tiles;
    const int perSlice = 9 * COUT * CIN + COUT;
    float *partial = nullptr;
    GBSP_CUDA_TRY(cudaMallocAsync((void **)&partial, sizeof(float) * (size_t)grid * perSlice, s));
    k_conv3x3_wgrad_tc<CIN, COUT><<<grid, 288, 0, s>>>(in, d, B, H, W, partial);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_wgrad_reduce<<<(perSlice + 255) / 256, 256, 0, s>>>(partial, grid, perSlice,
            9 * COUT * CIN, dW, dBias);
        e = cudaGetLastError();
    }
    cudaFreeAsync(partial, s);
    if (e != cudaSuccess) return cuda_error(e, "weight gradient");
    return GBSP_OK;
}

template <int CIN, int COUT>
static int launch_wgrad_tma(cudaStream_t s, const __nv_bfloat16 *in, const __nv_bfloat16 *d, int B,
    int H, int W, float *dW, float *dBias)
{
    using S = WtShape<CIN, COUT>;
    const int chunks = ((W + kWtPx - 1) / kWtPx) * B * H;
    int grid = sm_count();
    if (grid > chunks) grid = chunks;
    const size_t smem = 1024 + (size_t)kWtStages * S::kStage;
    auto kern = k_conv3x3_wgrad_tma<CIN, COUT>;
    GBSP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUtensorMap mapX, mapD;
    int rc;
    if ((rc = planar_words_tensor_map(&mapX, in, B, H, W, CIN, kWtPx)) ||
        (rc = planar_words_tensor_map(&mapD, d, B, H, W, COUT, kWtPx)))
        return rc;
    const int perSlice = 9 * COUT * CIN + COUT;
    float *partial = nullptr;
    GBSP_CUDA_TRY(cudaMallocAsync((void **)&partial, sizeof(float) * (size_t)grid * perSlice, s));
    kern<<<grid, kWtThreads, smem, s>>>(mapX, mapD, B, H, W, partial);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_wgrad_reduce<<<(perSlice + 255) / 256, 256, 0, s>>>(partial, grid, perSlice,
            9 * COUT * CIN, dW, dBias);
        e = cudaGetLastError();
    }
    cudaFreeAsync(partial, s);
    if (e != cudaSuccess) return cuda_error(e, "TMA-fed weight gradient");
    return GBSP_OK;
}

extern "C" {

int gbsp_dn_features(void *stream, const float *radiance, const float *aov, uint64_t pixels,
    uint32_t width, uint16_t *out)
{
    if (!radiance || !aov || !out) return set_error(GBSP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!pixels) return GBSP_OK;
    if (!width || pixels % width)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "pixels must be whole rows of `width`");
    k_features<<<blocks(pixels, 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(radiance), reinterpret_cast<const float4 *>(aov), pixels,
        (int)width, reinterpret_cast<__nv_bfloat16 *>(out));
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_conv3x3_forward(void *stream, const uint16_t *in, uint32_t B, uint32_t H, uint32_t W,
    uint32_t cin, const uint16_t *weights, const float *bias, uint32_t cout, int epilogue,
    uint16_t *outBf16, float *outF32)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!in || !weights || !B || !H || !W) return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad conv args");
    int sm = sm_count();
    if (epilogue == kEpiBf16BiasRelu && !outBf16) return set_error(GBSP_ERR_INVALID_ARGUMENT, "outBf16");
    if (epilogue != kEpiBf16BiasRelu && !outF32) return set_error(GBSP_ERR_INVALID_ARGUMENT, "outF32");
    if (epilogue != kEpiF32 && !bias) return set_error(GBSP_ERR_INVALID_ARGUMENT, "bias");
#define GBSP_CONV_CASE(CI, CO, EP)                                                               \
    if (cin == CI && cout == CO && epilogue == EP)                                               \
        return launch_conv<CI, CO, EP>(s, sm, in, B, H, W, weights, bias, outBf16, outF32);
    GBSP_CONV_CASE(16, 48, kEpiBf16BiasRelu)
    GBSP_CONV_CASE(48, 48, kEpiBf16BiasRelu)
    GBSP_CONV_CASE(48, 32, kEpiF32Bias)
    GBSP_CONV_CASE(48, 48, kEpiF32)
    GBSP_CONV_CASE(32, 48, kEpiF32)
#undef GBSP_CONV_CASE
    return set_error(GBSP_ERR_INVALID_ARGUMENT, "conv3x3 %u->%u epilogue %d not instantiated", cin,
        cout, epilogue);
}

int gbsp_dn_conv3x3_forward_tc(void *stream, const uint16_t *in, uint32_t B, uint32_t H,
    uint32_t W, uint32_t cin, const uint16_t *weights, const float *bias, uint32_t cout,
    int epilogue, uint16_t *outBf16, float *outF32)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!in || !weights || !B || !H || !W) return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad conv args");
    int sm = sm_count();
    if (epilogue == kEpiBf16BiasRelu && !outBf16) return set_error(GBSP_ERR_INVALID_ARGUMENT, "outBf16");
    if (epilogue != kEpiBf16BiasRelu && !outF32) return set_error(GBSP_ERR_INVALID_ARGUMENT, "outF32");
    if (epilogue != kEpiF32 && !bias) return set_error(GBSP_ERR_INVALID_ARGUMENT, "bias");
    if (((uintptr_t)in | (uintptr_t)weights | (uintptr_t)outBf16 | (uintptr_t)outF32) & 15u)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "conv tensors must be 16-byte aligned");
#define GBSP_CONV_CASE(CI, CO, EP)                                                               \
    if (cin == CI && cout == CO && epilogue == EP)                                               \
        return launch_conv_tc<CI, CO, EP>(s, sm, in, B, H, W, weights, bias, outBf16, outF32);
    GBSP_CONV_CASE(16, 48, kEpiBf16BiasRelu)
    GBSP_CONV_CASE(48, 48, kEpiBf16BiasRelu)
    GBSP_CONV_CASE(48, 32, kEpiF32Bias)
    GBSP_CONV_CASE(48, 48, kEpiF32)
    GBSP_CONV_CASE(32, 48, kEpiF32)
#undef GBSP_CONV_CASE
    return set_error(GBSP_ERR_INVALID_ARGUMENT, "conv3x3 %u->%u epilogue %d not instantiated", cin,
        cout, epilogue);
}

int gbsp_dn_conv3x3_filter_tc(void *stream, const uint16_t *in, uint32_t B, uint32_t H,
    uint32_t W, uint32_t cin, const uint16_t *weights, const float *bias, const float *noisy,
    float *out)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!in || !weights || !bias || !noisy || !out || !B || !H || !W)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad fused conv/filter args");
    if (((uintptr_t)in | (uintptr_t)weights | (uintptr_t)noisy | (uintptr_t)out) & 15u)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "conv tensors must be 16-byte aligned");
    if (cin != 48)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "fused conv/filter %u->32 not instantiated", cin);
    return launch_conv_tc<48, 32, kEpiFilter>(s, sm_count(), in, (int)B, (int)H, (int)W, weights,
        bias, nullptr, nullptr, reinterpret_cast<const float4 *>(noisy),
        reinterpret_cast<float4 *>(out));
}

int gbsp_dn_tc_rate(uint32_t n, uint32_t iters, uint32_t issuers, uint32_t aOffset16,
    double *cyclesPerMma)
{
    if (!cyclesPerMma || !iters || issuers < 1 || issuers > 2 || aOffset16 > 64)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad MMA rate probe args");
    unsigned long long *d = nullptr;
    GBSP_CUDA_TRY(cudaMalloc((void **)&d, 2 * sizeof(unsigned long long)));
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    switch (n) {
    case 16: k_tc_rate<16><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    case 32: k_tc_rate<32><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    case 48: k_tc_rate<48><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    case 64: k_tc_rate<64><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    case 96: k_tc_rate<96><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    case 128: k_tc_rate<128><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    case 144: k_tc_rate<144><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    case 256: k_tc_rate<256><<<1, 64>>>((int)iters, (int)issuers, (int)aOffset16, d); break;
    default:
        cudaFree(d);
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "MMA rate probe: N = %u not instantiated", n);
    }
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    GBSP_CUDA_TRY(e);
    for (uint32_t k = 0; k < issuers; k++) cyclesPerMma[k] = (double)h[k] / (double)iters;
    return h[0] ? GBSP_OK : set_error(GBSP_ERR_DEVICE_STATUS, "MMA rate probe timed out");
}

int gbsp_dn_status(uint32_t *status)
{
    if (!status) return set_error(GBSP_ERR_INVALID_ARGUMENT, "status is NULL");
    GBSP_CUDA_TRY(cudaMemcpyFromSymbol(status, g_dnStatus, sizeof(uint32_t)));
    uint32_t zero = 0;
    GBSP_CUDA_TRY(cudaMemcpyToSymbol(g_dnStatus, &zero, sizeof(uint32_t)));
    return *status ? set_error(GBSP_ERR_DEVICE_STATUS, "denoiser device status 0x%x", *status)
                   : GBSP_OK;
}

int gbsp_dn_flip_transpose(void *stream, const uint16_t *w, uint32_t cout, uint32_t cin,
    uint16_t *wt)
{
    uint32_t n = 9 * cout * cin;
    k_flip_transpose<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const __nv_bfloat16 *>(w), (int)cout, (int)cin,
        reinterpret_cast<__nv_bfloat16 *>(wt));
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_relu_backward(void *stream, const float *dAct, const uint16_t *act, uint64_t n,
    uint16_t *out)
{
    if (!n) return GBSP_OK;
    k_relu_bwd<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(dAct,
        reinterpret_cast<const __nv_bfloat16 *>(act), n, reinterpret_cast<__nv_bfloat16 *>(out));
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_conv3x3_weight_grad_tc(void *stream, const uint16_t *in, const uint16_t *dOut,
    uint32_t B, uint32_t H, uint32_t W, uint32_t cin, uint32_t cout, float *dW, float *dBias)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!in || !dOut || !dW || !dBias || !B || !H || !W)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad weight-gradient args");
    const __nv_bfloat16 *i16 = reinterpret_cast<const __nv_bfloat16 *>(in);
    const __nv_bfloat16 *d16 = reinterpret_cast<const __nv_bfloat16 *>(dOut);
    if (cin == 16 && cout == 48) return launch_wgrad_tc<16, 48>(s, i16, d16, B, H, W, dW, dBias);
    if (cin == 48 && cout == 48) return launch_wgrad_tc<48, 48>(s, i16, d16, B, H, W, dW, dBias);
    if (cin == 48 && cout == 32) return launch_wgrad_tc<48, 32>(s, i16, d16, B, H, W, dW, dBias);
    return set_error(GBSP_ERR_INVALID_ARGUMENT, "weight grad %u->%u not instantiated", cin, cout);
}

int gbsp_dn_conv3x3_weight_grad_tcgen05(void *stream, const uint16_t *in, const uint16_t *dOut,
    uint32_t B, uint32_t H, uint32_t W, uint32_t cin, uint32_t cout, float *dW, float *dBias)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!in || !dOut || !dW || !dBias || !B || !H || !W)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad weight-gradient args");
    if (((uintptr_t)in | (uintptr_t)dOut) & 15u)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "weight-gradient tensors must be 16-byte aligned");
    const __nv_bfloat16 *i16 = reinterpret_cast<const __nv_bfloat16 *>(in);
    const __nv_bfloat16 *d16 = reinterpret_cast<const __nv_bfloat16 *>(dOut);
    if (cin == 16 && cout == 48) return launch_wgrad_tma<16, 48>(s, i16, d16, B, H, W, dW, dBias);
    if (cin == 48 && cout == 48) return launch_wgrad_tma<48, 48>(s, i16, d16, B, H, W, dW, dBias);
    if (cin == 48 && cout == 32) return launch_wgrad_tma<48, 32>(s, i16, d16, B, H, W, dW, dBias);
    return set_error(GBSP_ERR_INVALID_ARGUMENT, "weight grad %u->%u not instantiated", cin, cout);
}

int gbsp_dn_conv3x3_weight_grad(void *stream, const uint16_t *in, const uint16_t *dOut,
    uint32_t B, uint32_t H, uint32_t W, uint32_t cin, uint32_t cout, float *dW, float *dBias)
{
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t n = (uint64_t)B * H * W;
    int chunk = 2048;
    dim3 grid(blocks(n, chunk), 9);
    const __nv_bfloat16 *i16 = reinterpret_cast<const __nv_bfloat16 *>(in);
    const __nv_bfloat16 *d16 = reinterpret_cast<const __nv_bfloat16 *>(dOut);
    if (cin == 16 && cout == 48)
        k_conv3x3_wgrad<16, 48><<<grid, 128, 0, s>>>(i16, d16, B, H, W, chunk, dW, dBias);
    else if (cin == 48 && cout == 48)
        k_conv3x3_wgrad<48, 48><<<grid, 128, 0, s>>>(i16, d16, B, H, W, chunk, dW, dBias);
    else if (cin == 48 && cout == 32)
        k_conv3x3_wgrad<48, 32><<<grid, 128, 0, s>>>(i16, d16, B, H, W, chunk, dW, dBias);
    else
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "weight grad %u->%u not instantiated", cin, cout);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_filter(void *stream, const float *logits, const float *noisy, uint32_t B, uint32_t H,
    uint32_t W, float *out)
{
    uint64_t n = (uint64_t)B * H * W;
    k_filter<<<blocks(n, 128), 128, 0, (cudaStream_t)stream>>>(logits,
        reinterpret_cast<const float4 *>(noisy), B, H, W, reinterpret_cast<float4 *>(out));
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_tile_check(void *stream, const float *denoised, const float *plainA, uint32_t sppA,
    const float *plainC, uint32_t sppC, uint32_t B, uint32_t H, uint32_t W, uint32_t tile,
    float bound, float margin, uint32_t maxSpp, float *tileErr, uint32_t *flags, uint32_t *needSpp)
{
    if (!denoised || !plainA || !plainC || !tileErr || !flags || !needSpp || !B || !H || !W ||
        !sppA || !sppC || !maxSpp || !(bound > 0.0f) || !(margin > 0.0f))
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad tile check args");
    if (tile < 1 || tile > 16) return set_error(GBSP_ERR_INVALID_ARGUMENT, "tile must be 1..16");
    const uint64_t tiles = (uint64_t)B * ((H + tile - 1) / tile) * ((W + tile - 1) / tile);
    if (tiles > 0x7FFFFFFFull) return set_error(GBSP_ERR_CAPACITY, "too many tiles");
    k_tile_check<<<(unsigned)tiles, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(denoised), reinterpret_cast<const float4 *>(plainA),
        (float)sppA, reinterpret_cast<const float4 *>(plainC), (float)sppC, (int)B, (int)H, (int)W,
        (int)tile, bound, margin, maxSpp, tileErr, flags, needSpp);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_tile_merge(void *stream, const float *denoised, const float *plainA, uint32_t sppA,
    const float *plainC, uint32_t sppC, const float *fallback, const uint32_t *sppF, uint32_t B,
    uint32_t H, uint32_t W, uint32_t tile, const uint32_t *flags, float *out)
{
    if (!denoised || !plainA || !plainC || !flags || !out || !B || !H || !W || !sppA || !sppC ||
        (fallback && !sppF))
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad tile merge args");
    if (tile < 1 || tile > 16) return set_error(GBSP_ERR_INVALID_ARGUMENT, "tile must be 1..16");
    const uint64_t n = (uint64_t)B * H * W;
    k_tile_merge<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(denoised), reinterpret_cast<const float4 *>(plainA),
        (float)sppA, reinterpret_cast<const float4 *>(plainC), (float)sppC,
        reinterpret_cast<const float4 *>(fallback), sppF, (int)B, (int)H, (int)W, (int)tile, flags,
        reinterpret_cast<float4 *>(out));
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_tile_fallback(void *stream, const float *denoised, const float *plainA,
    const float *plainC, uint32_t B, uint32_t H, uint32_t W, uint32_t tile, float bound,
    float *out, float *tileErr, uint32_t *flags)
{
    if (!denoised || !plainA || !plainC || !out || !tileErr || !flags || !B || !H || !W)
        return set_error(GBSP_ERR_INVALID_ARGUMENT, "bad fallback args");
    if (tile < 1 || tile > 16) return set_error(GBSP_ERR_INVALID_ARGUMENT, "tile must be 1..16");
    uint64_t tiles = (uint64_t)B * ((H + tile - 1) / tile) * ((W + tile - 1) / tile);
    k_tile_fallback<<<(unsigned)tiles, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(denoised), reinterpret_cast<const float4 *>(plainA),
        reinterpret_cast<const float4 *>(plainC), (int)B, (int)H, (int)W, (int)tile, bound,
        reinterpret_cast<float4 *>(out), tileErr, flags);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_relmse_backward(void *stream, const float *logits, const float *noisy,
    const float *target, uint32_t B, uint32_t H, uint32_t W, uint16_t *dLogits, float *lossSum)
{
    uint64_t n = (uint64_t)B * H * W;
    k_relmse_bwd<<<blocks(n, 128), 128, 0, (cudaStream_t)stream>>>(logits,
        reinterpret_cast<const float4 *>(noisy), reinterpret_cast<const float4 *>(target), B, H, W,
        1.0f / (3.0f * (float)n), reinterpret_cast<__nv_bfloat16 *>(dLogits), lossSum);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_dn_adam(void *stream, float *param, uint16_t *paramBf16, const float *grad, float *m,
    float *v, uint64_t n, float lr, float beta1, float beta2, float eps, uint32_t step)
{
    float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(param,
        reinterpret_cast<__nv_bfloat16 *>(paramBf16), grad, m, v, n, lr, beta1, beta2, eps, c1, c2);
    GBSP_CUDA_TRY(cudaGetLastError());
    return GBSP_OK;
}

}  // extern "C"
