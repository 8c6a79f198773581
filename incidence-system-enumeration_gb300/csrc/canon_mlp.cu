// canon_mlp.cu -- the learned search order: a BF16 MLP 64 -> 128 -> 128 -> 1 that
// scores every row of a matrix as the first row of the canonical labeling.
//
// Inference and the forward pass of training run on the 5th-generation tensor cores
// (tcgen05.mma, BF16 operands, FP32 accumulators in tensor memory, 128 rows per CTA:
// mlp_forward_tc_kernel).  The earlier warp-level path (mma.sync m16n8k16, one warp per
// 16 rows, the hidden activations kept in registers as A fragments) stays as the
// context option CANON_OPT_MLP_WARP_MMA.  The backward pass propagates through the same layers (the hidden
// gradient dH1 = dH2 * W2 also on the tensor cores), the weight gradients are
// tiled FP32 reductions over the batch, and Adam keeps FP32 master weights from
// which the BF16 copies are refreshed after every step.  No counterpart in the
// reference.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "canon_internal.h"

namespace canon {

namespace {

constexpr int IN = 64, HID = 128;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
    return (uint32_t)__bfloat16_as_ushort(l) | ((uint32_t)__bfloat16_as_ushort(h) << 16);
}

__device__ __forceinline__ float bf_lo(uint32_t v) { return __bfloat162float(__ushort_as_bfloat16((unsigned short)(v & 0xFFFFu))); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __bfloat162float(__ushort_as_bfloat16((unsigned short)(v >> 16))); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// two consecutive bf16 of a row-major matrix as one 32-bit word (0 outside the rows)
__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16 *m, long rows, long row, int ld, int col) {
    if (row >= rows)
        return 0u;
    return *reinterpret_cast<const uint32_t *>(m + row * ld + col);
}

struct MlpDev {
    const __nv_bfloat16 *w1;   // [128][64]
    const float *b1;           // [128]
    const __nv_bfloat16 *w2;   // [128][128]
    const float *b2;           // [128]
    const __nv_bfloat16 *w3;   // [128]
    const float *b3;           // [1]
};

// The weights staged in shared memory once per block: W1 and W2 with their rows
// padded by 8 BF16 (4 words), so that the 8 rows a B fragment load touches fall in 8
// different banks; biases and w3 beside them.
constexpr int W1_LD = IN + 8, W2_LD = HID + 8;
constexpr size_t FWD_SMEM = (size_t)HID * W1_LD * 2 + (size_t)HID * W2_LD * 2 + (size_t)HID * 4 * 3 + 16;

// two consecutive bf16 of a row of a staged matrix (leading dimension ld)
__device__ __forceinline__ uint32_t lds2(const __nv_bfloat16 *m, int row, int ld, int col) {
    return *reinterpret_cast<const uint32_t *>(m + row * ld + col);
}

// Forward pass of 16 rows per warp, the warps of a block sharing the staged weights.
// Writes logits; when h1/h2 are given also the (BF16, post-ReLU) hidden activations
// for the backward pass.
__global__ void __launch_bounds__(128) mlp_forward_kernel(long n, const __nv_bfloat16 *__restrict__ x, MlpDev wg,
                                                          float *__restrict__ y, __nv_bfloat16 *__restrict__ h1out,
                                                          __nv_bfloat16 *__restrict__ h2out) {
    extern __shared__ __align__(16) unsigned char fwd_smem[];
    __nv_bfloat16 *sw1 = reinterpret_cast<__nv_bfloat16 *>(fwd_smem);
    __nv_bfloat16 *sw2 = sw1 + HID * W1_LD;
    float *sb1 = reinterpret_cast<float *>(sw2 + HID * W2_LD);
    float *sb2 = sb1 + HID;
    float *sw3 = sb2 + HID;
    for (int i = threadIdx.x; i < HID * IN / 2; i += blockDim.x) {
        const int r = i / (IN / 2), c = 2 * (i % (IN / 2));
        *reinterpret_cast<uint32_t *>(sw1 + r * W1_LD + c) = *reinterpret_cast<const uint32_t *>(wg.w1 + r * IN + c);
    }
    for (int i = threadIdx.x; i < HID * HID / 2; i += blockDim.x) {
        const int r = i / (HID / 2), c = 2 * (i % (HID / 2));
        *reinterpret_cast<uint32_t *>(sw2 + r * W2_LD + c) = *reinterpret_cast<const uint32_t *>(wg.w2 + r * HID + c);
    }
    for (int i = threadIdx.x; i < HID; i += blockDim.x) {
        sb1[i] = wg.b1[i];
        sb2[i] = wg.b2[i];
        sw3[i] = __bfloat162float(wg.w3[i]);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
    const long tiles = (n + 15) / 16;
    for (long tile = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile < tiles;
         tile += (long)gridDim.x * (blockDim.x >> 5)) {
        const long r0 = tile * 16;
        uint32_t a[4][4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            a[t][0] = ld2(x, n, r0 + g, IN, 16 * t + 2 * tg);
            a[t][1] = ld2(x, n, r0 + g + 8, IN, 16 * t + 2 * tg);
            a[t][2] = ld2(x, n, r0 + g, IN, 16 * t + 8 + 2 * tg);
            a[t][3] = ld2(x, n, r0 + g + 8, IN, 16 * t + 8 + 2 * tg);
        }
        // layer 1: 16 x 128 = relu(X W1^T + b1), kept as packed BF16 A fragments of layer 2
        uint32_t h1[16][2];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const uint32_t b0 = lds2(sw1, 8 * j + g, W1_LD, 16 * t + 2 * tg);
                const uint32_t b1 = lds2(sw1, 8 * j + g, W1_LD, 16 * t + 8 + 2 * tg);
                mma_bf16(acc, a[t], b0, b1);
            }
            const float bb0 = sb1[8 * j + 2 * tg], bb1 = sb1[8 * j + 2 * tg + 1];
            h1[j][0] = pack_bf16(fmaxf(acc[0] + bb0, 0.f), fmaxf(acc[1] + bb1, 0.f));
            h1[j][1] = pack_bf16(fmaxf(acc[2] + bb0, 0.f), fmaxf(acc[3] + bb1, 0.f));
            if (h1out) {
                if (r0 + g < n)
                    *reinterpret_cast<uint32_t *>(h1out + (r0 + g) * HID + 8 * j + 2 * tg) = h1[j][0];
                if (r0 + g + 8 < n)
                    *reinterpret_cast<uint32_t *>(h1out + (r0 + g + 8) * HID + 8 * j + 2 * tg) = h1[j][1];
            }
        }
        // layer 2 and the output layer, one 8-wide tile at a time
        float part0 = 0.f, part1 = 0.f;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const uint32_t af[4] = {h1[2 * t][0], h1[2 * t][1], h1[2 * t + 1][0], h1[2 * t + 1][1]};
                const uint32_t b0 = lds2(sw2, 8 * j + g, W2_LD, 16 * t + 2 * tg);
                const uint32_t b1 = lds2(sw2, 8 * j + g, W2_LD, 16 * t + 8 + 2 * tg);
                mma_bf16(acc, af, b0, b1);
            }
            const float bb0 = sb2[8 * j + 2 * tg], bb1 = sb2[8 * j + 2 * tg + 1];
            const uint32_t p0 = pack_bf16(fmaxf(acc[0] + bb0, 0.f), fmaxf(acc[1] + bb1, 0.f));
            const uint32_t p1 = pack_bf16(fmaxf(acc[2] + bb0, 0.f), fmaxf(acc[3] + bb1, 0.f));
            if (h2out) {
                if (r0 + g < n)
                    *reinterpret_cast<uint32_t *>(h2out + (r0 + g) * HID + 8 * j + 2 * tg) = p0;
                if (r0 + g + 8 < n)
                    *reinterpret_cast<uint32_t *>(h2out + (r0 + g + 8) * HID + 8 * j + 2 * tg) = p1;
            }
            const float w30 = sw3[8 * j + 2 * tg], w31 = sw3[8 * j + 2 * tg + 1];
            part0 += bf_lo(p0) * w30 + bf_hi(p0) * w31;
            part1 += bf_lo(p1) * w30 + bf_hi(p1) * w31;
        }
        part0 += __shfl_xor_sync(0xFFFFFFFFu, part0, 1);
        part0 += __shfl_xor_sync(0xFFFFFFFFu, part0, 2);
        part1 += __shfl_xor_sync(0xFFFFFFFFu, part1, 1);
        part1 += __shfl_xor_sync(0xFFFFFFFFu, part1, 2);
        if (tg == 0) {
            if (r0 + g < n)
                y[r0 + g] = part0 + wg.b3[0];
            if (r0 + g + 8 < n)
                y[r0 + g + 8] = part1 + wg.b3[0];
        }
    }
}

// ---- the forward pass on the 5th-generation tensor cores -------------------
// One CTA (4 warps) takes 128 rows at a time.  Both layers are tcgen05.mma
// (kind::f16: BF16 operands, FP32 accumulators in tensor memory) issued by one
// thread: D1[128 x 128] = X[128 x 64] W1^T, then D2[128 x 128] = H1[128 x 128] W2^T.
// The operands sit in shared memory in the K-major layout without swizzle, as 8-row x
// 16-byte core matrices.  X arrives by TMA (cp.async.bulk.tensor): eight boxes of 128
// rows x 8 elements, each 2 KB with its rows 16 bytes apart, so the core matrices of
// an 8-row group are 128 bytes apart (stride byte offset) and those along K 2 KB apart
// (leading byte offset); the next tile's X is requested as soon as this tile's first
// MMAs are done, and arrives while the rest of the tile runs.  W1, W2 and H1 use
// 8-row groups (K/8) x 128 bytes apart and K neighbours 128 bytes apart.  Each
// thread owns one row of the accumulators (tensor-memory lane = row): it reads its
// row with tcgen05.ld, adds the bias, applies the ReLU and rounds to BF16 -- H1 goes
// back to shared memory as layer 2's A operand, H2 meets w3 in a per-thread dot
// product.  W1 and W2 are staged once per CTA.  Every wait for the tensor cores is
// bounded by time: past it the kernel raises *err, stops, frees its tensor memory
// and returns.
constexpr int TC_ROWS = 128;
constexpr uint32_t TC_TMEM_COLS = 256;                  // D1 in columns 0-127, D2 in 128-255
constexpr uint32_t TC_W1 = 0, TC_W2 = TC_W1 + HID * IN * 2, TC_X = TC_W2 + HID * HID * 2,
                   TC_H1 = TC_X + TC_ROWS * IN * 2, TC_PAR = TC_H1 + TC_ROWS * HID * 2,
                   TC_BAR = TC_PAR + 3 * HID * 4, TC_END = TC_BAR + 32;
// in the barrier block: the MMA barrier at +0, the tensor-memory address at +8, the TMA barrier at +16
constexpr uint32_t TC_X_CHUNK = TC_ROWS * 16;           // one TMA box: 128 rows x 16 bytes
constexpr size_t TC_SMEM = TC_END + 1024;               // + the alignment of the base to 1 KB
// instruction descriptor, kind::f16: FP32 accumulator (bit 4), BF16 A (bits 7-9 = 1) and
// B (bits 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(HID >> 3) << 17) |
                              ((uint32_t)(TC_ROWS >> 4) << 24);
constexpr unsigned long long TC_WAIT_NS = 1000000000ull;   // 1 s: far beyond any tile's MMAs

// byte offset of the 16-byte chunk (row r, K elements 8*k8 .. 8*k8+7) of a K-major tile
// whose rows hold kdim elements
__device__ __forceinline__ uint32_t core_off(int r, int k8, int kdim) {
    return (uint32_t)((r >> 3) * (kdim / 8) * 128 + k8 * 128 + (r & 7) * 16);
}

// shared-memory matrix descriptor: start, leading and stride byte offsets (>> 4), the
// descriptor version (1 at bit 46), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ unsigned long long tc_now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// waits for the phase of the given parity of the barrier; false after TC_WAIT_NS
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = tc_now();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok)
            return true;
        if (tc_now() - t0 > TC_WAIT_NS)
            return false;
    }
}

// 32 consecutive FP32 accumulator columns of this thread's row (the warp's 32 lanes)
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&f)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i)
        f[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void async_proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// the X rows [row0, row0 + 128) as eight TMA boxes (columns 8k .. 8k+7 each) into the
// tile, all counted on the TMA barrier; rows past the tensor's end arrive as zeros
__device__ __forceinline__ void tc_load_x(const CUtensorMap *tmap, uint32_t dst, uint32_t bar, long row0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(TC_ROWS * IN * 2)
                 : "memory");
#pragma unroll
    for (int k8 = 0; k8 < IN / 8; ++k8)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
            "[%4];" ::"r"(dst + k8 * TC_X_CHUNK),
            "l"(reinterpret_cast<uint64_t>(tmap)), "r"(8 * k8), "r"((int)row0), "r"(bar)
            : "memory");
}

__global__ void __launch_bounds__(128, 1) mlp_forward_tc_kernel(long n, const __grid_constant__ CUtensorMap xmap,
                                                                MlpDev wg, float *__restrict__ y,
                                                                __nv_bfloat16 *__restrict__ h1out,
                                                                __nv_bfloat16 *__restrict__ h2out, unsigned *err) {
    extern __shared__ __align__(16) unsigned char tc_smem_raw[];
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(tc_smem_raw);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    unsigned char *sm = tc_smem_raw + pad;
    const uint32_t sbase = raw + pad;
    float *sb1 = reinterpret_cast<float *>(sm + TC_PAR), *sb2 = sb1 + HID, *sw3 = sb2 + HID;
    const uint32_t bar = sbase + TC_BAR, tbar = sbase + TC_BAR + 16;
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(sm + TC_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // tensor memory: one warp allocates (and at the end frees) the accumulator columns
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + TC_BAR + 8),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    const long tiles = (n + TC_ROWS - 1) / TC_ROWS;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the first tile's X, while the weights are staged
        if ((long)blockIdx.x < tiles)
            tc_load_x(&xmap, sbase + TC_X, tbar, (long)blockIdx.x * TC_ROWS);
    }
    // the weights (K-major core-matrix layout) and the biases, once
    for (int i = tid; i < HID * (IN / 8); i += blockDim.x) {
        const int r = i / (IN / 8), k8 = i % (IN / 8);
        *reinterpret_cast<uint4 *>(sm + TC_W1 + core_off(r, k8, IN)) =
            *reinterpret_cast<const uint4 *>(wg.w1 + r * IN + k8 * 8);
    }
    for (int i = tid; i < HID * (HID / 8); i += blockDim.x) {
        const int r = i / (HID / 8), k8 = i % (HID / 8);
        *reinterpret_cast<uint4 *>(sm + TC_W2 + core_off(r, k8, HID)) =
            *reinterpret_cast<const uint4 *>(wg.w2 + r * HID + k8 * 8);
    }
    for (int i = tid; i < HID; i += blockDim.x) {
        sb1[i] = wg.b1[i];
        sb2[i] = wg.b2[i];
        sw3[i] = __bfloat162float(wg.w3[i]);
    }
    async_proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t d1 = tmem, d2 = tmem + HID;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;    // this warp's 32 tensor-memory lanes
    const float b3 = wg.b3[0];
    // the parity each barrier completes next; what is in flight and the parity it completes on
    uint32_t phase = 0, tphase = 0, mma_parity = 0, x_parity = 0;
    bool failed = false, x_pending = (long)blockIdx.x < tiles, mma_pending = false;
    for (long tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const long r0 = tile * TC_ROWS;
        // this tile's X (requested one tile earlier)
        x_parity = tphase;
        bool ok = tc_wait(tbar, tphase);
        tphase ^= 1u;
        x_pending = !ok;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < IN / 16; ++ks)
                tc_mma(d1, tc_desc(sbase + TC_X + ks * 2 * TC_X_CHUNK, TC_X_CHUNK, 128),
                       tc_desc(sbase + TC_W1 + ks * 256, 128, (IN / 8) * 128), ks > 0);
            tc_commit(bar);
        }
        mma_parity = phase;
        ok = tc_wait(bar, phase);
        phase ^= 1u;
        mma_pending = !ok;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        // the X tile is read: request the next one now
        if (tile + gridDim.x < tiles) {
            if (tid == 0)
                tc_load_x(&xmap, sbase + TC_X, tbar, (tile + gridDim.x) * TC_ROWS);
            x_pending = true;
            x_parity = tphase;
        }
        tc_fence_after();
        // layer-1 epilogue: H1 = relu(D1 + b1) in BF16, this thread's row
        const int row = 32 * warp + lane;
        const long grow = r0 + row;
#pragma unroll 1
        for (int c = 0; c < HID / 32; ++c) {
            float f[32];
            tc_ld32(d1 + lane_base + 32 * c, f);
            uint32_t pk[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = 32 * c + 2 * j;
                pk[j] = pack_bf16(fmaxf(f[2 * j] + sb1[col], 0.f), fmaxf(f[2 * j + 1] + sb1[col + 1], 0.f));
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 v = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
                *reinterpret_cast<uint4 *>(sm + TC_H1 + core_off(row, 4 * c + q, HID)) = v;
                if (h1out && grow < n)
                    *reinterpret_cast<uint4 *>(h1out + grow * HID + (4 * c + q) * 8) = v;
            }
        }
        tc_fence_before();
        async_proxy_fence();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < HID / 16; ++ks)
                tc_mma(d2, tc_desc(sbase + TC_H1 + ks * 256, 128, (HID / 8) * 128),
                       tc_desc(sbase + TC_W2 + ks * 256, 128, (HID / 8) * 128), ks > 0);
            tc_commit(bar);
        }
        mma_parity = phase;
        ok = tc_wait(bar, phase);
        phase ^= 1u;
        mma_pending = !ok;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();
        // layer-2 epilogue: H2 = relu(D2 + b2) in BF16, and the logit H2 . w3 + b3
        float acc = 0.f;
#pragma unroll 1
        for (int c = 0; c < HID / 32; ++c) {
            float f[32];
            tc_ld32(d2 + lane_base + 32 * c, f);
            uint32_t pk[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = 32 * c + 2 * j;
                pk[j] = pack_bf16(fmaxf(f[2 * j] + sb2[col], 0.f), fmaxf(f[2 * j + 1] + sb2[col + 1], 0.f));
                acc += bf_lo(pk[j]) * sw3[col] + bf_hi(pk[j]) * sw3[col + 1];
            }
            if (h2out && grow < n) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    *reinterpret_cast<uint4 *>(h2out + grow * HID + (4 * c + q) * 8) =
                        make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
            }
        }
        if (grow < n)
            y[grow] = acc + b3;
        tc_fence_before();
        __syncthreads();
    }
    if (failed) {
        if (tid == 0)
            atomicExch(err, 1u);
        // what is still in flight (the MMAs the barrier waited for, a requested X tile):
        // once more, bounded, before the tensor memory and the shared memory are given up
        if (mma_pending)
            (void)tc_wait(bar, mma_parity);
        if (x_pending)
            (void)tc_wait(tbar, x_parity);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
    }
}

// The backward pass on tcgen05, 128 rows per CTA, one row per thread: dy and the BCE loss
// of the row, dH2 = dy w3 [H2 > 0] (FP32 to global memory for the weight gradients, BF16
// into shared memory as the A operand), then dH1 = (dH2 W2) [H1 > 0] as 8 MMAs of
// 128 x 128 x 16 into 128 tensor-memory columns, with W2 transposed ([in][out], K-major
// for B) staged once per CTA.  The same operand layouts, descriptors and bounded waits as
// mlp_forward_tc_kernel.
constexpr uint32_t TB_W2T = 0, TB_A = TB_W2T + HID * HID * 2, TB_W3 = TB_A + TC_ROWS * HID * 2,
                   TB_BAR = TB_W3 + HID * 4, TB_END = TB_BAR + 16;
constexpr size_t TB_SMEM = TB_END + 1024;
constexpr uint32_t TB_TMEM_COLS = 128;

__global__ void __launch_bounds__(128, 1) mlp_backward_tc_kernel(long n, const float *__restrict__ logit,
                                                                 const float *__restrict__ label,
                                                                 const __nv_bfloat16 *__restrict__ h1,
                                                                 const __nv_bfloat16 *__restrict__ h2,
                                                                 const __nv_bfloat16 *__restrict__ w3,
                                                                 const __nv_bfloat16 *__restrict__ w2t,
                                                                 float *__restrict__ dy, float *__restrict__ dh2,
                                                                 float *__restrict__ dh1, float *__restrict__ loss_sum,
                                                                 unsigned *err) {
    extern __shared__ __align__(16) unsigned char tb_smem_raw[];
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(tb_smem_raw);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    unsigned char *sm = tb_smem_raw + pad;
    const uint32_t sbase = raw + pad;
    float *sw3 = reinterpret_cast<float *>(sm + TB_W3);
    const uint32_t bar = sbase + TB_BAR;
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(sm + TB_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + TB_BAR + 8),
                     "r"(TB_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < HID * (HID / 8); i += blockDim.x) {
        const int r = i / (HID / 8), k8 = i % (HID / 8);
        *reinterpret_cast<uint4 *>(sm + TB_W2T + core_off(r, k8, HID)) =
            *reinterpret_cast<const uint4 *>(w2t + r * HID + k8 * 8);
    }
    for (int i = tid; i < HID; i += blockDim.x)
        sw3[i] = __bfloat162float(w3[i]);
    async_proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    const float inv_n = 1.f / (float)n;
    uint32_t phase = 0, mma_parity = 0;
    bool failed = false, mma_pending = false;
    const long tiles = (n + TC_ROWS - 1) / TC_ROWS;
    for (long tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const int row = 32 * warp + lane;
        const long r = tile * TC_ROWS + row;
        const bool in = r < n;
        // dy and the loss of this row (rows past n contribute nothing)
        float d = 0.f, l = 0.f;
        if (in) {
            const float z = logit[r], t = label[r];
            d = (1.f / (1.f + __expf(-z)) - t) * inv_n;
            l = fmaxf(z, 0.f) - z * t + log1pf(__expf(-fabsf(z)));
            dy[r] = d;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            l += __shfl_xor_sync(0xFFFFFFFFu, l, o);
        if (lane == 0 && l != 0.f)
            atomicAdd(loss_sum, l);
        // dH2 of this row: FP32 out, BF16 into the A tile
#pragma unroll 1
        for (int k8 = 0; k8 < HID / 8; ++k8) {
            uint4 hv = make_uint4(0u, 0u, 0u, 0u);
            if (in)
                hv = *reinterpret_cast<const uint4 *>(h2 + r * HID + k8 * 8);
            const uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
            float g[8];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = k8 * 8 + 2 * j;
                g[2 * j] = bf_lo(hw[j]) > 0.f ? d * sw3[c] : 0.f;
                g[2 * j + 1] = bf_hi(hw[j]) > 0.f ? d * sw3[c + 1] : 0.f;
            }
            if (in) {
                float4 *dst = reinterpret_cast<float4 *>(dh2 + r * HID + k8 * 8);
                dst[0] = make_float4(g[0], g[1], g[2], g[3]);
                dst[1] = make_float4(g[4], g[5], g[6], g[7]);
            }
            *reinterpret_cast<uint4 *>(sm + TB_A + core_off(row, k8, HID)) =
                make_uint4(pack_bf16(g[0], g[1]), pack_bf16(g[2], g[3]), pack_bf16(g[4], g[5]),
                           pack_bf16(g[6], g[7]));
        }
        tc_fence_before();
        async_proxy_fence();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < HID / 16; ++ks)
                tc_mma(tmem, tc_desc(sbase + TB_A + ks * 256, 128, (HID / 8) * 128),
                       tc_desc(sbase + TB_W2T + ks * 256, 128, (HID / 8) * 128), ks > 0);
            tc_commit(bar);
        }
        mma_parity = phase;
        const bool ok = tc_wait(bar, phase);
        phase ^= 1u;
        mma_pending = !ok;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        tc_fence_after();
        // dH1 = (dH2 W2) [H1 > 0]
#pragma unroll 1
        for (int c = 0; c < HID / 32; ++c) {
            float f[32];
            tc_ld32(tmem + lane_base + 32 * c, f);
            if (in) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint4 hv = *reinterpret_cast<const uint4 *>(h1 + r * HID + 32 * c + 8 * q);
                    const uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
                    float o[8];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        o[2 * j] = bf_lo(hw[j]) > 0.f ? f[8 * q + 2 * j] : 0.f;
                        o[2 * j + 1] = bf_hi(hw[j]) > 0.f ? f[8 * q + 2 * j + 1] : 0.f;
                    }
                    float4 *dst = reinterpret_cast<float4 *>(dh1 + r * HID + 32 * c + 8 * q);
                    dst[0] = make_float4(o[0], o[1], o[2], o[3]);
                    dst[1] = make_float4(o[4], o[5], o[6], o[7]);
                }
            }
        }
        tc_fence_before();
        __syncthreads();
    }
    if (failed) {
        if (tid == 0)
            atomicExch(err, 1u);
        if (mma_pending)
            (void)tc_wait(bar, mma_parity);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TB_TMEM_COLS)
                     : "memory");
    }
}

// Weight gradients on tcgen05: G[o][i] = sum over rows of dh[row][o] * act[row][i], the
// batch rows being the contraction.  A CTA takes 128-row K tiles in turn and accumulates in
// tensor memory; each thread stages its row transposed into the K-major core-matrix layout
// (A[o][row] = BF16 of dh, B[i][row] = act), so the operands are those of the forward pass
// with the rows as K.  B gets a row of ones (the valid rows) after its IN activation rows, so
// column IN of the product is the bias gradient sum dh[row][o]; 15 zero rows pad N to a
// multiple of 16.  At the end every CTA adds its 128 x (IN + 1) partial sums to the FP32
// gradient.  Shared memory is padded so that at most two CTAs share an SM: two 256-column
// tensor-memory allocations never wait.
template <int IN>
struct WgLayout {
    static constexpr int NB = IN + 16;                               // B rows
    static constexpr uint32_t A = 0, B = TC_ROWS * HID * 2, BAR = B + NB * TC_ROWS * 2, END = BAR + 16;
    static constexpr size_t SMEM = 100 * 1024 + 1024;                // two CTAs per SM at most
    static_assert(END + 1024 <= SMEM, "tiles fit");
    // kind::f16, FP32 accumulator, BF16 A and B, K-major, N = NB, M = 128
    static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NB >> 3) << 17) |
                                      ((uint32_t)(TC_ROWS >> 4) << 24);
};
constexpr uint32_t WG_TMEM_COLS = 256;

template <int IN>
__global__ void __launch_bounds__(128, 1) weight_grad_tc_kernel(long n, const float *__restrict__ dh,
                                                                const __nv_bfloat16 *__restrict__ act,
                                                                float *__restrict__ gw, float *__restrict__ gb,
                                                                unsigned *err) {
    using L = WgLayout<IN>;
    extern __shared__ __align__(16) unsigned char wg_smem_raw[];
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(wg_smem_raw);
    const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
    unsigned char *sm = wg_smem_raw + pad;
    const uint32_t sbase = raw + pad;
    const uint32_t bar = sbase + L::BAR;
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(sm + L::BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long tiles = (n + TC_ROWS - 1) / TC_ROWS;
    if ((long)blockIdx.x >= tiles)
        return;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + L::BAR + 8),
                     "r"(WG_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // B rows IN + 1 .. NB - 1 stay zero
    for (int i = tid; i < (L::NB - IN - 1) * (TC_ROWS / 8); i += blockDim.x) {
        const int r = IN + 1 + i / (TC_ROWS / 8), k8 = i % (TC_ROWS / 8);
        *reinterpret_cast<uint4 *>(sm + L::B + core_off(r, k8, TC_ROWS)) = make_uint4(0u, 0u, 0u, 0u);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    // this thread's place along K in every tile: K-chunk tid / 8, element tid % 8
    const uint32_t kofs = (uint32_t)(tid >> 3) * 128u + (uint32_t)(tid & 7) * 2u;
    uint32_t phase = 0, mma_parity = 0;
    bool failed = false, mma_pending = false, first = true;
    for (long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const long r = tile * TC_ROWS + tid;
        const bool in = r < n;
        // A[o][k] = dh[r][o]
#pragma unroll 1
        for (int o8 = 0; o8 < HID / 8; ++o8) {
            float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
            if (in) {
                v0 = *reinterpret_cast<const float4 *>(dh + r * HID + o8 * 8);
                v1 = *reinterpret_cast<const float4 *>(dh + r * HID + o8 * 8 + 4);
            }
            const float v[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
            unsigned char *dst = sm + L::A + (uint32_t)o8 * (HID / 8) * 128u + kofs;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                *reinterpret_cast<__nv_bfloat16 *>(dst + j * 16) = __float2bfloat16_rn(v[j]);
        }
        // B[i][k] = act[r][i], and the row of ones
#pragma unroll 1
        for (int i8 = 0; i8 < IN / 8; ++i8) {
            uint4 a = make_uint4(0u, 0u, 0u, 0u);
            if (in)
                a = *reinterpret_cast<const uint4 *>(act + r * IN + i8 * 8);
            const uint32_t w[4] = {a.x, a.y, a.z, a.w};
            unsigned char *dst = sm + L::B + (uint32_t)i8 * (TC_ROWS / 8) * 128u + kofs;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                *reinterpret_cast<uint16_t *>(dst + (2 * j) * 16) = (uint16_t)(w[j] & 0xFFFFu);
                *reinterpret_cast<uint16_t *>(dst + (2 * j + 1) * 16) = (uint16_t)(w[j] >> 16);
            }
        }
        *reinterpret_cast<__nv_bfloat16 *>(sm + L::B + (uint32_t)(IN / 8) * (TC_ROWS / 8) * 128u + kofs) =
            __float2bfloat16_rn(in ? 1.f : 0.f);
        tc_fence_before();
        async_proxy_fence();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < TC_ROWS / 16; ++ks) {
                const uint64_t ad = tc_desc(sbase + L::A + ks * 256, 128, (TC_ROWS / 8) * 128);
                const uint64_t bd = tc_desc(sbase + L::B + ks * 256, 128, (TC_ROWS / 8) * 128);
                const uint32_t acc = (!first || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(L::IDESC), "r"(acc));
            }
            tc_commit(bar);
        }
        first = false;
        mma_parity = phase;
        const bool ok = tc_wait(bar, phase);
        phase ^= 1u;
        mma_pending = !ok;
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
    }
    if (!failed) {
        tc_fence_after();
        // row o = this thread's tensor-memory lane: add the partial sums
        const int o = 32 * warp + lane;
        const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
#pragma unroll 1
        for (int c = 0; c < (L::NB + 31) / 32; ++c) {
            float f[32];
            tc_ld32(tmem + lane_base + 32 * c, f);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int i = 32 * c + j;
                if (i < IN)
                    atomicAdd(gw + o * IN + i, f[j]);
                else if (i == IN)
                    atomicAdd(gb + o, f[j]);
            }
        }
    } else {
        if (tid == 0)
            atomicExch(err, 1u);
        if (mma_pending)
            (void)tc_wait(bar, mma_parity);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(WG_TMEM_COLS)
                     : "memory");
    }
}

// Backward of the binary cross-entropy on the logits: dy, dH2 = dy w3 [H2 > 0]
// and dH1 = (dH2 W2) [H1 > 0] (tensor cores; w2t is W2 transposed, [in][out]).
__global__ void mlp_backward_kernel(long n, const float *__restrict__ logit, const float *__restrict__ label,
                                    const __nv_bfloat16 *__restrict__ h1, const __nv_bfloat16 *__restrict__ h2,
                                    const __nv_bfloat16 *__restrict__ w3, const __nv_bfloat16 *__restrict__ w2t,
                                    float *__restrict__ dy, float *__restrict__ dh2, float *__restrict__ dh1,
                                    float *__restrict__ loss_sum) {
    const int lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
    const long tiles = (n + 15) / 16;
    const float inv_n = 1.f / (float)n;
    for (long tile = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile < tiles;
         tile += (long)gridDim.x * (blockDim.x >> 5)) {
        const long r0 = tile * 16;
        const long ra = r0 + g, rb = r0 + g + 8;
        float dya = 0.f, dyb = 0.f;
        if (ra < n) {
            const float z = logit[ra], t = label[ra];
            dya = (1.f / (1.f + __expf(-z)) - t) * inv_n;
        }
        if (rb < n) {
            const float z = logit[rb], t = label[rb];
            dyb = (1.f / (1.f + __expf(-z)) - t) * inv_n;
        }
        if (tg == 0) {
            // loss (sum of BCE terms), one lane per row pair
            float l = 0.f;
            if (ra < n) {
                const float z = logit[ra], t = label[ra];
                l += fmaxf(z, 0.f) - z * t + log1pf(__expf(-fabsf(z)));
            }
            if (rb < n) {
                const float z = logit[rb], t = label[rb];
                l += fmaxf(z, 0.f) - z * t + log1pf(__expf(-fabsf(z)));
            }
            atomicAdd(loss_sum, l);
        }
        if (tg == 0) {
            if (ra < n)
                dy[ra] = dya;
            if (rb < n)
                dy[rb] = dyb;
        }
        // dH2 in the A-fragment layout (k = layer-2 outputs)
        uint32_t a2[8][4];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int c = 8 * j + 2 * tg;
            const float w30 = __bfloat162float(w3[c]), w31 = __bfloat162float(w3[c + 1]);
            const uint32_t ha = ld2(h2, n, ra, HID, c), hb = ld2(h2, n, rb, HID, c);
            const float g0 = bf_lo(ha) > 0.f ? dya * w30 : 0.f, g1 = bf_hi(ha) > 0.f ? dya * w31 : 0.f;
            const float g2 = bf_lo(hb) > 0.f ? dyb * w30 : 0.f, g3 = bf_hi(hb) > 0.f ? dyb * w31 : 0.f;
            if (ra < n) {
                dh2[ra * HID + c] = g0;
                dh2[ra * HID + c + 1] = g1;
            }
            if (rb < n) {
                dh2[rb * HID + c] = g2;
                dh2[rb * HID + c + 1] = g3;
            }
            const int t = j >> 1;
            if (j & 1) {
                a2[t][2] = pack_bf16(g0, g1);
                a2[t][3] = pack_bf16(g2, g3);
            } else {
                a2[t][0] = pack_bf16(g0, g1);
                a2[t][1] = pack_bf16(g2, g3);
            }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const uint32_t b0 = ld2(w2t, HID, 8 * j + g, HID, 16 * t + 2 * tg);
                const uint32_t b1 = ld2(w2t, HID, 8 * j + g, HID, 16 * t + 8 + 2 * tg);
                mma_bf16(acc, a2[t], b0, b1);
            }
            const int c = 8 * j + 2 * tg;
            const uint32_t ha = ld2(h1, n, ra, HID, c), hb = ld2(h1, n, rb, HID, c);
            if (ra < n) {
                dh1[ra * HID + c] = bf_lo(ha) > 0.f ? acc[0] : 0.f;
                dh1[ra * HID + c + 1] = bf_hi(ha) > 0.f ? acc[1] : 0.f;
            }
            if (rb < n) {
                dh1[rb * HID + c] = bf_lo(hb) > 0.f ? acc[2] : 0.f;
                dh1[rb * HID + c + 1] = bf_hi(hb) > 0.f ? acc[3] : 0.f;
            }
        }
    }
}

// grad_w[o][i] += sum_rows dh[row][o] * act[row][i] (act BF16), grad_b[o] += sum dh[row][o]:
// a 32 x 32 output tile per block, a slice of the rows per blockIdx.z.
__global__ void weight_grad_kernel(long n, int out_dim, int in_dim, const float *__restrict__ dh,
                                   const __nv_bfloat16 *__restrict__ act, float *__restrict__ gw,
                                   float *__restrict__ gb) {
    __shared__ float sd[32][33];
    __shared__ float sa[32][33];
    const int o0 = blockIdx.y * 32, i0 = blockIdx.x * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8 threads
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    float accb = 0.f;
    const long per = (n + gridDim.z - 1) / gridDim.z;
    const long lo = (long)blockIdx.z * per, hi = (lo + per < n) ? lo + per : n;
    for (long r = lo; r < hi; r += 32) {
        for (int q = ty; q < 32; q += 8) {
            const long row = r + q;
            sd[q][tx] = (row < hi && o0 + tx < out_dim) ? dh[row * out_dim + o0 + tx] : 0.f;
            sa[q][tx] = (row < hi && i0 + tx < in_dim) ? __bfloat162float(act[row * in_dim + i0 + tx]) : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int q = 0; q < 32; ++q) {
            const float av = sa[q][tx];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                acc[u] += sd[q][ty + 8 * u] * av;
            if (blockIdx.x == 0 && ty == 0)
                accb += sd[q][tx];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int o = o0 + ty + 8 * u, i = i0 + tx;
        if (o < out_dim && i < in_dim)
            atomicAdd(&gw[o * in_dim + i], acc[u]);
    }
    if (blockIdx.x == 0 && ty == 0 && o0 + tx < out_dim)
        atomicAdd(&gb[o0 + tx], accb);
}

// output layer: grad_w3[i] += sum dy*h2[row][i], grad_b3 += sum dy
__global__ void out_grad_kernel(long n, const float *__restrict__ dy, const __nv_bfloat16 *__restrict__ h2,
                                float *__restrict__ gw3, float *__restrict__ gb3) {
    const int i = threadIdx.x;   // 128 threads
    float acc = 0.f, accb = 0.f;
    for (long r = blockIdx.x; r < n; r += gridDim.x) {
        const float d = dy[r];
        acc += d * __bfloat162float(h2[r * HID + i]);
        if (i == 0)
            accb += d;
    }
    atomicAdd(&gw3[i], acc);
    if (i == 0)
        atomicAdd(gb3, accb);
}

// Adam over the flat FP32 parameter vector; refreshes the BF16 copies (and W2^T).
__global__ void adam_kernel(int count, float *__restrict__ p, const float *__restrict__ grad, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                            __nv_bfloat16 *__restrict__ w1, __nv_bfloat16 *__restrict__ w2,
                            __nv_bfloat16 *__restrict__ w2t, __nv_bfloat16 *__restrict__ w3) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count)
        return;
    const float gk = grad[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    const float pk = p[k] - lr * (mk / c1) / (sqrtf(vk / c2) + eps);
    p[k] = pk;
    // layout of the flat vector: w1 | b1 | w2 | b2 | w3 | b3
    const int W1 = HID * IN, B1 = W1 + HID, W2 = B1 + HID * HID, B2 = W2 + HID, W3 = B2 + HID;
    if (k < W1) {
        w1[k] = __float2bfloat16_rn(pk);
    } else if (k >= B1 && k < W2) {
        const int q = k - B1;
        w2[q] = __float2bfloat16_rn(pk);
        w2t[(q % HID) * HID + q / HID] = __float2bfloat16_rn(pk);
    } else if (k >= B2 && k < W3) {
        w3[k - B2] = __float2bfloat16_rn(pk);
    }
}

// ---- features and labels -----------------------------------------------------

// 64 features of every row of a normalised incidence matrix as the first row:
// [0,16) histogram of |R_x & R_y| over the other rows; [16,32) histogram over the
// other rows y of the number of rows z meeting R_x & R_y; [32,48) histogram of the
// column weights of the columns of R_x; [48,64) row index one-hot, fill depth
// n/16, shape b/64, |R_x|/b.  Scaled to [0, 1].
__global__ void features_kernel(uint32_t n_items, uint32_t v, uint32_t b, uint32_t nrows, uint32_t flags,
                                const uint64_t *__restrict__ rows, __nv_bfloat16 *__restrict__ feat) {
    const uint32_t it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n_items)
        return;
    uint64_t R[VMAX];
    for (uint32_t r = 0; r < VMAX; ++r)
        R[r] = (r < nrows) ? rows[(size_t)it * v + r] : 0ull;
    (void)flags;
    unsigned colw[64];
    for (uint32_t c = 0; c < b; ++c) {
        unsigned w = 0;
        for (uint32_t r = 0; r < nrows; ++r)
            w += (unsigned)((R[r] >> c) & 1u);
        colw[c] = w;
    }
    for (uint32_t x = 0; x < nrows; ++x) {
        float f[64];
        for (int q = 0; q < 64; ++q)
            f[q] = 0.f;
        const float inv = 1.f / (float)(nrows > 1 ? nrows - 1 : 1);
        for (uint32_t y = 0; y < nrows; ++y) {
            if (y == x)
                continue;
            const uint64_t xy = R[x] & R[y];
            f[min(__popcll(xy), 15)] += inv;
            unsigned meet = 0;
            for (uint32_t z = 0; z < nrows; ++z)
                if (z != x && z != y && (xy & R[z]))
                    ++meet;
            f[16 + min(meet, 15u)] += inv;
        }
        const float invc = 1.f / (float)(__popcll(R[x]) ? __popcll(R[x]) : 1);
        for (uint32_t c = 0; c < b; ++c)
            if ((R[x] >> c) & 1u)
                f[32 + min(colw[c], 15u)] += invc;
        f[48 + (x & 15u)] = 1.f;
        __nv_bfloat16 *dst = feat + ((size_t)it * v + x) * 64;
        for (int q = 0; q < 48; ++q)
            dst[q] = __float2bfloat16_rn(f[q]);
        for (int q = 48; q < 64; ++q)
            dst[q] = __float2bfloat16_rn(f[q]);
        dst[63] = __float2bfloat16_rn((float)nrows / 16.f);
        dst[62] = __float2bfloat16_rn((float)b / 64.f);
        dst[61] = __float2bfloat16_rn((float)__popcll(R[x]) / (float)b);
    }
}

// rows of every matrix sorted by decreasing score (ties: lower row first), nibble-packed
__global__ void order_kernel(uint32_t n, uint32_t v, const float *__restrict__ scores, uint64_t *__restrict__ orders) {
    const uint32_t it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n)
        return;
    const float *sc = scores + (size_t)it * v;
    uint64_t ord = 0xFEDCBA9876543210ull;
    for (uint32_t x = 0; x < v; ++x) {
        unsigned rank = 0;
        for (uint32_t y = 0; y < v; ++y)
            rank += (sc[y] > sc[x]) || (sc[y] == sc[x] && y < x);
        ord = (ord & ~(15ull << (4 * rank))) | ((uint64_t)x << (4 * rank));
    }
    orders[it] = ord;
}

}  // namespace

cudaError_t launch_order_by_score(uint32_t n, uint32_t v, const float *d_scores, uint64_t *d_orders, cudaStream_t s) {
    if (!n)
        return cudaSuccess;
    order_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, v, d_scores, d_orders);
    return cudaGetLastError();
}

namespace mlp {

cudaError_t forward(long n, const void *x, const void *w1, const float *b1, const void *w2, const float *b2,
                    const void *w3, const float *b3, float *y, void *h1, void *h2, int num_sms, cudaStream_t s) {
    MlpDev w{(const __nv_bfloat16 *)w1, b1, (const __nv_bfloat16 *)w2, b2, (const __nv_bfloat16 *)w3, b3};
    const long tiles = (n + 15) / 16;
    // a persistent grid (the staged weights are loaded once per block): 4 blocks per SM
    long grid = (tiles + 3) / 4;
    if (grid > 4L * num_sms)
        grid = 4L * num_sms;
    if (grid < 1)
        grid = 1;
    // above 48 KB of dynamic shared memory a kernel must opt in (per device: set on every launch)
    const cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)FWD_SMEM);
    if (e != cudaSuccess)
        return e;
    mlp_forward_kernel<<<(int)grid, 128, FWD_SMEM, s>>>(n, (const __nv_bfloat16 *)x, w, y, (__nv_bfloat16 *)h1,
                                                         (__nv_bfloat16 *)h2);
    return cudaGetLastError();
}

cudaError_t forward_tc(long n, const void *x, const void *w1, const float *b1, const void *w2, const float *b2,
                       const void *w3, const float *b3, float *y, void *h1, void *h2, unsigned *err, int num_sms,
                       cudaStream_t s) {
    if (n <= 0)
        return cudaSuccess;
    MlpDev w{(const __nv_bfloat16 *)w1, b1, (const __nv_bfloat16 *)w2, b2, (const __nv_bfloat16 *)w3, b3};
    const long tiles = (n + TC_ROWS - 1) / TC_ROWS;
    // a persistent grid, two CTAs per SM (shared memory allows two; their 2 x 256 tensor-memory
    // columns are the SM's 512, so an allocation never waits)
    long grid = 2L * (num_sms > 0 ? num_sms : 1);
    if (grid > tiles)
        grid = tiles;
    // X as a 2-D tensor (64 BF16 columns, n rows of 128 bytes) read in boxes of 8 x 128
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess)
            return e;
        if (q != cudaDriverEntryPointSuccess || !fn)
            return cudaErrorSymbolNotFound;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    CUtensorMap xmap;
    const cuuint64_t dims[2] = {(cuuint64_t)IN, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)IN * 2};
    const cuuint32_t box[2] = {8, (cuuint32_t)TC_ROWS};
    const cuuint32_t estr[2] = {1, 1};
    if (encode(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(x), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    const cudaError_t e =
        cudaFuncSetAttribute(mlp_forward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
    if (e != cudaSuccess)
        return e;
    mlp_forward_tc_kernel<<<(int)grid, 128, TC_SMEM, s>>>(n, xmap, w, y, (__nv_bfloat16 *)h1, (__nv_bfloat16 *)h2,
                                                          err);
    return cudaGetLastError();
}

cudaError_t backward_tc(long n, const float *logit, const float *label, const void *h1, const void *h2,
                        const void *w3, const void *w2t, float *dy, float *dh2, float *dh1, float *loss,
                        unsigned *err, int num_sms, cudaStream_t s) {
    if (n <= 0)
        return cudaSuccess;
    const long tiles = (n + TC_ROWS - 1) / TC_ROWS;
    // three CTAs fit an SM by shared memory (66 KB each); 3 x 128 tensor-memory columns
    long grid = 3L * (num_sms > 0 ? num_sms : 1);
    if (grid > tiles)
        grid = tiles;
    const cudaError_t e =
        cudaFuncSetAttribute(mlp_backward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TB_SMEM);
    if (e != cudaSuccess)
        return e;
    mlp_backward_tc_kernel<<<(int)grid, 128, TB_SMEM, s>>>(n, logit, label, (const __nv_bfloat16 *)h1,
                                                           (const __nv_bfloat16 *)h2, (const __nv_bfloat16 *)w3,
                                                           (const __nv_bfloat16 *)w2t, dy, dh2, dh1, loss, err);
    return cudaGetLastError();
}

cudaError_t backward(long n, const float *logit, const float *label, const void *h1, const void *h2, const void *w3,
                     const void *w2t, float *dy, float *dh2, float *dh1, float *loss, int num_sms, cudaStream_t s) {
    const long tiles = (n + 15) / 16;
    long grid = (tiles + 3) / 4;
    if (grid > 32L * num_sms)
        grid = 32L * num_sms;
    if (grid < 1)
        grid = 1;
    mlp_backward_kernel<<<(int)grid, 128, 0, s>>>(n, logit, label, (const __nv_bfloat16 *)h1,
                                                   (const __nv_bfloat16 *)h2, (const __nv_bfloat16 *)w3,
                                                   (const __nv_bfloat16 *)w2t, dy, dh2, dh1, loss);
    return cudaGetLastError();
}

cudaError_t weight_grads(long n, const float *dh1, const float *dh2, const float *dy, const void *x, const void *h1,
                         const void *h2, float *grad, int num_sms, cudaStream_t s) {
    const int W1 = HID * IN, B1 = W1 + HID, W2 = B1 + HID * HID, B2 = W2 + HID, W3 = B2 + HID, B3 = W3 + HID;
    int zs = (int)((n + 2047) / 2048);
    if (zs > 4 * num_sms)
        zs = 4 * num_sms;
    if (zs < 1)
        zs = 1;
    weight_grad_kernel<<<dim3(IN / 32, HID / 32, zs), 256, 0, s>>>(n, HID, IN, dh1, (const __nv_bfloat16 *)x,
                                                                   grad, grad + W1);
    weight_grad_kernel<<<dim3(HID / 32, HID / 32, zs), 256, 0, s>>>(n, HID, HID, dh2, (const __nv_bfloat16 *)h1,
                                                                    grad + B1, grad + W2);
    int og = (int)((n + 255) / 256);
    if (og > 8 * num_sms)
        og = 8 * num_sms;
    if (og < 1)
        og = 1;
    out_grad_kernel<<<og, HID, 0, s>>>(n, dy, (const __nv_bfloat16 *)h2, grad + B2, grad + W3);
    (void)B3;
    return cudaGetLastError();
}

cudaError_t weight_grads_tc(long n, const float *dh1, const float *dh2, const float *dy, const void *x, const void *h1,
                            const void *h2, float *grad, unsigned *err, int num_sms, cudaStream_t s) {
    const int W1 = HID * IN, B1 = W1 + HID, W2 = B1 + HID * HID, B2 = W2 + HID, W3 = B2 + HID;
    if (n <= 0)
        return cudaSuccess;
    const long tiles = (n + TC_ROWS - 1) / TC_ROWS;
    long grid = 2L * (num_sms > 0 ? num_sms : 1);
    if (grid > tiles)
        grid = tiles;
    cudaError_t e = cudaFuncSetAttribute(weight_grad_tc_kernel<IN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)WgLayout<IN>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(weight_grad_tc_kernel<HID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)WgLayout<HID>::SMEM);
    if (e != cudaSuccess)
        return e;
    weight_grad_tc_kernel<IN><<<(int)grid, 128, WgLayout<IN>::SMEM, s>>>(n, dh1, (const __nv_bfloat16 *)x, grad,
                                                                         grad + W1, err);
    weight_grad_tc_kernel<HID><<<(int)grid, 128, WgLayout<HID>::SMEM, s>>>(n, dh2, (const __nv_bfloat16 *)h1,
                                                                           grad + B1, grad + W2, err);
    int og = (int)((n + 255) / 256);
    if (og > 8 * num_sms)
        og = 8 * num_sms;
    if (og < 1)
        og = 1;
    out_grad_kernel<<<og, HID, 0, s>>>(n, dy, (const __nv_bfloat16 *)h2, grad + B2, grad + W3);
    return cudaGetLastError();
}

cudaError_t adam(int count, float *p, const float *grad, float *m, float *v, float lr, int step, void *w1, void *w2,
                 void *w2t, void *w3, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.f, c2 = 1.f;
    for (int i = 0; i < step; ++i) {
        c1 *= b1;
        c2 *= b2;
    }
    adam_kernel<<<(count + 255) / 256, 256, 0, s>>>(count, p, grad, m, v, lr, b1, b2, 1e-8f, 1.f - c1, 1.f - c2,
                                                    (__nv_bfloat16 *)w1, (__nv_bfloat16 *)w2, (__nv_bfloat16 *)w2t,
                                                    (__nv_bfloat16 *)w3);
    return cudaGetLastError();
}

cudaError_t features(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *rows, void *feat,
                     cudaStream_t s) {
    features_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, v, b, v, flags, rows, (__nv_bfloat16 *)feat);
    return cudaGetLastError();
}

}  // namespace mlp

}  // namespace canon
