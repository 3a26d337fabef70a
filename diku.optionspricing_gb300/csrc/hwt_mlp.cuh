// Fused surrogate network: the whole 8 -> 256 -> 256 -> 256 -> 256 -> 2 SiLU MLP
// of a 128-row tile in one persistent kernel, activations on chip.
//
//   layer 0 (8 -> 256):   fp32 on the CUDA cores, one thread per row, from fp32
//                         features (the first layer resolves strike-sized features,
//                         which bf16 inputs or weights would move by ~1e-2 strike)
//   layers 1-3 (256x256): tcgen05.mma kind::f16, bf16 activations in shared memory
//                         (A operand, K-major core-matrix layout), bf16 weights
//                         streamed from L2 (B operand), fp32 accumulator in 256
//                         TMEM columns (M = 128, N = 256, K = 16 per instruction);
//                         layer 1 runs two passes into one accumulator: its input as
//                         bf16 hi parts, then (layer 0 recomputed) the lo parts
//   layer 4 (256 -> 2):   fp32 dot products of layer 3's fp32 activations with fp32
//                         weights, in the last layer's epilogue: a partial sum per
//                         128 columns (k in order from 0), the two partials added
//
// Each output row is computed exactly as the layer-by-layer training path computes
// it (same roundings, same K order of the tensor-core sums, layer 4 summed in the
// same order), so a network trained there evaluates the same here.
//
// The fp32 constants (layer 0's weights and bias, the biases of layers 1-3, layer 4's
// weights and bias; 14 KB) are copied to shared memory once per CTA.
// Weights of the three tensor-core layers are pre-packed (the surrogate's refresh
// kernel) into 24 blocks of [256 output rows x 32 K] in the canonical no-swizzle
// K-major layout, 16 KB each (32 streamed per tile: layer 1's twice), so one thread
// streams a block with a single untiled
// bulk copy (cp.async.bulk, completion counted on an mbarrier) through a ring of
// kStages shared-memory stages; the tensor core frees a stage by committing the
// MMAs that read it to the stage's "empty" mbarrier.  One thread (thread 0) issues
// copies and MMAs; all 256 threads run layer 0 and the epilogues, two per tile row
// (row r = TMEM lane r; warps w and w + 4 read lane quarter w % 4 and take the first
// and the second 128 columns).  Two CTAs share an SM (112 KB of shared memory and
// 256 TMEM columns each), so one CTA's epilogue overlaps the other's MMAs.
//
// Every mbarrier wait is bounded.  A CTA whose wait runs out raises *err, stops
// issuing, waits (bounded) for the copies and MMAs it already issued, frees its
// TMEM and returns; if that drain wait runs out as well the tensor core or the copy
// engine has stopped completing work, and the CTA frees its TMEM and returns anyway
// with *err raised.  test_stall injects a wait that nothing completes: 1 before any
// copy or MMA, 2 after the first weight block's MMAs were committed.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "hwt_umma.cuh"

namespace hwt {
namespace mlp {

constexpr int kRows = 128;      // rows per tile (the MMA's M, one per thread)
constexpr int kHidden = 256;
constexpr int kIn = 8;          // 7 standardised features + a zero pad
constexpr int kOut = 2;         // price residual, log-error estimate
constexpr int kKB = 32;         // K per streamed weight block
constexpr int kBlocksPerLayer = kHidden / kKB;  // 8
constexpr int kTcLayers = 3;
constexpr int kBlocks = kTcLayers * kBlocksPerLayer;  // 24 packed blocks
// MMA passes per tile: layer 1 twice (its input as a bf16 hi / lo pair, the two
// products accumulated), layers 2 and 3 once: 32 weight blocks streamed per tile.
constexpr int kPasses = kTcLayers + 1;
constexpr int kSeqBlocks = kPasses * kBlocksPerLayer;

// Packed weight block of the q-th block streamed in a tile.
__host__ __device__ __forceinline__ int seq_block(int q)
{
    const int pass = q / kBlocksPerLayer;
    return (pass <= 1 ? 0 : pass - 1) * kBlocksPerLayer + q % kBlocksPerLayer;
}
constexpr int kStages = 2;      // weight stages in shared memory
constexpr int kCtasPerSm = 2;   // 112 KB of shared memory per CTA fits twice per SM
constexpr int kThreads = 256;   // two threads per row: each takes half of the 256 columns
constexpr int kHalf = kHidden / 2;
constexpr int kActBytes = kRows * kHidden * 2;       // 64 KB
constexpr int kWBlockElems = kHidden * kKB;           // 8192
constexpr int kWBlockBytes = kWBlockElems * 2;        // 16 KB
// fp32 constants kept in shared memory: W0 [8][256], b0..b3 [4][256], W4 [256][2], b4 [2] (+2 pad)
constexpr int kConstFloats = kIn * kHidden + 4 * kHidden + kHidden * kOut + 4;
constexpr int kConstBytes = kConstFloats * 4;
constexpr int kBarBytes = ((2 * kStages + 2) * 8 + 8 + 127) / 128 * 128;  // mbarriers, TMEM slot, abort word
constexpr int kSmemBytes = kActBytes + kStages * kWBlockBytes + kConstBytes + kBarBytes;
static_assert(kSmemBytes * kCtasPerSm + kCtasPerSm * 1024 <= 228 * 1024, "shared memory of the CTAs of one SM");
constexpr int kTmemCols = 256;

struct MlpArgs {
    const float *X;            // [n][8] standardised features
    int n;
    const float *W0, *b0;      // fp32 [8][256], [256]
    const __nv_bfloat16 *Wp;   // packed blocks of layers 1-3 (see pack_offset)
    const float *b1, *b2, *b3; // [256] biases of layers 1-3
    const float *W4;           // [256][2] fp32 weights of layer 4
    const float *b4;           // [2]
    float *out;                // [n][2]
    int *err;
    int test_stall;
};

// Element offset of (output row nrow, k) inside a packed [256 x 32] weight block:
// 8 x 8 core matrices of 128 contiguous bytes, K-adjacent ones 128 bytes apart,
// row-adjacent ones 512 bytes apart.
__host__ __device__ __forceinline__ int pack_offset(int nrow, int k)
{
    return ((((nrow >> 3) * (kKB / 8)) + (k >> 3)) << 6) + ((nrow & 7) << 3) + (k & 7);
}

// Element offset of (row r, k) in the 128 x 256 activation tile: four 64-wide K
// blocks of the same core-matrix layout (16 KB each), as the GEMM stages use.
__device__ __forceinline__ int act_offset(int r, int k) { return (k >> 6) * (kRows * 64) + umma::core_offset(r, k & 63); }

// Layer 0 of one row for output columns [n0, n0 + 8): z = b0 + x W0 (fp32, k in
// order), shared by the fused kernel (weights in shared memory) and the training
// path (weights in global memory).
__device__ __forceinline__ void layer0_chunk(const float (&x)[kIn], const float *__restrict__ W0,
                                             const float *__restrict__ b0, int n0, float (&z)[8])
{
    const float4 *b4 = reinterpret_cast<const float4 *>(b0 + n0);
    const float4 ba = b4[0], bb = b4[1];
    float2 z2[4] = {make_float2(ba.x, ba.y), make_float2(ba.z, ba.w), make_float2(bb.x, bb.y), make_float2(bb.z, bb.w)};
#pragma unroll
    for (int k = 0; k < kIn; ++k) {
        // fma(x_k, W0[k][n], z[n]) for eight columns, two per paired instruction
        const float4 *w4 = reinterpret_cast<const float4 *>(W0 + k * kHidden + n0);
        const float4 wa = w4[0], wb = w4[1];
        const float2 xk = make_float2(x[k], x[k]);
        z2[0] = __ffma2_rn(xk, make_float2(wa.x, wa.y), z2[0]);
        z2[1] = __ffma2_rn(xk, make_float2(wa.z, wa.w), z2[1]);
        z2[2] = __ffma2_rn(xk, make_float2(wb.x, wb.y), z2[2]);
        z2[3] = __ffma2_rn(xk, make_float2(wb.z, wb.w), z2[3]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        z[2 * j] = z2[j].x;
        z[2 * j + 1] = z2[j].y;
    }
}

__device__ __forceinline__ uint32_t pack_silu2(float a, float b)
{
    const float2 h = umma::silu2_f(make_float2(a, b));
    const __nv_bfloat162 q = __floats2bfloat162_rn(h.x, h.y);
    return *reinterpret_cast<const uint32_t *>(&q);
}

// Layer 0's activations as a bf16 pair: hi = bf16(a), lo = bf16(a - hi); layer 1 takes
// hi and lo as two inputs whose products with its weights accumulate (bf16 rounding
// of these activations moved the payoff kinks the network resolves; the pair carries
// about 16 bits).  `lo_part` selects which half to return.
__device__ __forceinline__ uint32_t pack_silu2_split(float a, float b, bool lo_part)
{
    const float2 h = umma::silu2_f(make_float2(a, b));
    const __nv_bfloat162 hi = __floats2bfloat162_rn(h.x, h.y);
    if (!lo_part) return *reinterpret_cast<const uint32_t *>(&hi);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(h.x - __low2float(hi), h.y - __high2float(hi));
    return *reinterpret_cast<const uint32_t *>(&lo);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__global__ void __launch_bounds__(kThreads, kCtasPerSm) mlp_forward_kernel(MlpArgs p)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __nv_bfloat16 *act = reinterpret_cast<__nv_bfloat16 *>(smem);
    unsigned char *wst = smem + kActBytes;
    float *cst = reinterpret_cast<float *>(smem + kActBytes + kStages * kWBlockBytes);
    float *sW0 = cst, *sB = cst + kIn * kHidden, *sW4 = sB + 4 * kHidden, *sB4 = sW4 + kHidden * kOut;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kActBytes + kStages * kWBlockBytes + kConstBytes);
    // bars: full[3], empty[3], acc, never; then the TMEM address and the abort word
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kStages + 2);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    // row r of the tile is TMEM lane r: warps w and w + 4 share lane quarter w % 4 and
    // split the columns (warps 0-3 the first half, 4-7 the second)
    const int r = tid & (kRows - 1), half = tid >> 7, cbase = half * kHalf;
    const uint32_t full0 = umma::smem_u32(&bars[0]), empty0 = umma::smem_u32(&bars[kStages]);
    const uint32_t acc_bar = umma::smem_u32(&bars[2 * kStages]), never_bar = umma::smem_u32(&bars[2 * kStages + 1]);
    constexpr uint32_t IDESC = umma::make_idesc(kHidden);

    if (tid == 0) {
        for (int s = 0; s < 2 * kStages + 2; ++s) umma::mbar_init(umma::smem_u32(&bars[s]), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) umma::tmem_alloc(umma::smem_u32(tmem_slot), kTmemCols);
    // the fp32 constants into shared memory (read by every thread of every tile)
    for (int i = tid; i < kIn * kHidden; i += kThreads) sW0[i] = p.W0[i];
    for (int i = tid; i < kHidden; i += kThreads) {
        sB[i] = p.b0[i];
        sB[kHidden + i] = p.b1[i];
        sB[2 * kHidden + i] = p.b2[i];
        sB[3 * kHidden + i] = p.b3[i];
    }
    for (int i = tid; i < kHidden * kOut; i += kThreads) sW4[i] = p.W4[i];
    if (tid < kOut) sB4[tid] = p.b4[tid];
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's TMEM lane quarter

    uint32_t ld = 0, mm = 0, acc_uses = 0;  // blocks copied, blocks consumed, accumulator completions (thread 0)
    bool ok = true;                          // thread 0: no wait ran out
    int stall = p.test_stall;
    const int ntiles = (p.n + kRows - 1) / kRows;
    // weight blocks this CTA consumes in all (copies never run past them)
    const uint32_t total_blocks =
        (blockIdx.x < ntiles ? (uint32_t)((ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1) : 0u) * kSeqBlocks;

    // Thread 0: copy weight block `ld` (global block ld % kBlocks) into its stage,
    // once the MMAs that last read that stage have completed.
    auto load_next = [&]() -> bool {
        const uint32_t s = ld % kStages;
        if (ld >= (uint32_t)kStages && !umma::mbar_wait(empty0 + 8 * s, ((ld - kStages) / kStages) & 1)) return false;
        bulk_copy_g2s(umma::smem_u32(wst + s * kWBlockBytes), p.Wp + (size_t)seq_block(ld % kSeqBlocks) * kWBlockElems,
                      kWBlockBytes, full0 + 8 * s);
        ++ld;
        return true;
    };

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int row = tile * kRows + r;
        // ---- layer 0 on the CUDA cores: this thread's row and half -> activation tile,
        // the hi parts of the activations (lo_part = false) or their lo parts
        auto layer0 = [&](bool lo_part) {
            float x[kIn];
            if (row < p.n) {
                const float4 *xr = reinterpret_cast<const float4 *>(p.X + (size_t)row * kIn);
                const float4 xa = __ldg(xr), xb = __ldg(xr + 1);
                x[0] = xa.x; x[1] = xa.y; x[2] = xa.z; x[3] = xa.w;
                x[4] = xb.x; x[5] = xb.y; x[6] = xb.z; x[7] = xb.w;
            } else {
#pragma unroll
                for (int k = 0; k < kIn; ++k) x[k] = 0.f;
            }
#pragma unroll 1
            for (int n0 = cbase; n0 < cbase + kHalf; n0 += 8) {
                float z[8];
                layer0_chunk(x, sW0, sB, n0, z);
                uint4 v;
                v.x = pack_silu2_split(z[0], z[1], lo_part);
                v.y = pack_silu2_split(z[2], z[3], lo_part);
                v.z = pack_silu2_split(z[4], z[5], lo_part);
                v.w = pack_silu2_split(z[6], z[7], lo_part);
                *reinterpret_cast<uint4 *>(act + act_offset(r, n0)) = v;
            }
        };
        layer0(false);
        float o0 = 0.f, o1 = 0.f;
#pragma unroll 1
        for (int pass = 0; pass < kPasses; ++pass) {
            const int l = pass == 0 ? 0 : pass - 1;  // the tensor-core layer this pass accumulates
            if (tid == 0 && !ok) *abort_flag = 1;  // a prefetch wait ran out
            umma::fence_proxy_async();  // activation writes -> visible to the tensor core
            umma::fence_before_sync();
            __syncthreads();
            umma::fence_after_sync();
            if (*abort_flag) break;
            if (tid == 0) {
                // blocks of this layer: mm .. mm + 7; at most kStages copies ahead
                const uint32_t end = mm + kBlocksPerLayer;
                while (ok && ld < end && ld < mm + kStages) ok = load_next();
                for (int kb = 0; ok && kb < kBlocksPerLayer; ++kb) {
                    const uint32_t s = mm % kStages;
                    if (stall == 1) {  // injected: a phase nothing completes, before any MMA
                        ok = umma::mbar_wait(never_bar, 0);
                        stall = 0;
                        if (!ok) break;
                    }
                    if (!umma::mbar_wait(full0 + 8 * s, (mm / kStages) & 1)) { ok = false; break; }
                    umma::fence_after_sync();
                    const uint32_t a0 = umma::smem_u32(act), b0 = umma::smem_u32(wst + s * kWBlockBytes);
#pragma unroll
                    for (int kk = 0; kk < kKB / 16; ++kk) {
                        const int ks = kb * (kKB / 16) + kk;  // 16-wide K step in the layer
                        const uint64_t ad = umma::make_desc(a0 + (ks >> 2) * (kRows * 64 * 2) + (ks & 3) * 256, 128, 1024);
                        const uint64_t bd = umma::make_desc(b0 + kk * 256, 128, (kKB / 8) * 128);
                        umma::mma_bf16(tmem, ad, bd, IDESC, (pass == 1 || kb > 0 || kk > 0) ? 1u : 0u);
                    }
                    umma::mma_commit(empty0 + 8 * s);
                    ++mm;
                    if (stall == 2) {  // injected: after this block's MMAs were committed
                        ok = umma::mbar_wait(never_bar, 0);
                        stall = 0;
                        if (!ok) break;
                    }
                    // refill the stage block mm - 2 used (its MMAs are one block behind)
                    if (ld < end && ld < mm + kStages - 1) ok = load_next();
                }
                if (ok) umma::mma_commit(acc_bar);
                else *abort_flag = 1;
            }
            __syncthreads();
            if (*abort_flag) break;
            // every MMA of the layer has completed once acc_bar's phase does
            if (!umma::mbar_wait(acc_bar, acc_uses & 1)) {
                *abort_flag = 1;
                ok = false;
            }
            ++acc_uses;
            umma::fence_after_sync();
            if (__syncthreads_or(*abort_flag)) break;
            // the stages are free: prefetch the next pass's (or the next tile's) first blocks
            if (tid == 0) {
                while (ok && ld < total_blocks && ld < mm + kStages) ok = load_next();  // a failure is seen at the next barrier
            }
            if (pass == 0) {
                layer0(true);  // layer 1's second input: the lo parts, over the hi parts just read
                continue;
            }
            // ---- epilogue: accumulator + bias -> SiLU -> bf16 (next layer's A) or layer 4
            const float *bias = sB + (l + 1) * kHidden;
#pragma unroll 1
            for (int c2 = cbase; c2 < cbase + kHalf; c2 += 32) {
                // two 16-column TMEM loads in flight, the biases fetched meanwhile
                uint32_t ra[16], rb[16];
                umma::tmem_ld16_async(trow + (uint32_t)c2, ra);
                umma::tmem_ld16_async(trow + (uint32_t)(c2 + 16), rb);
                float4 bv[8];
                const float4 *b4 = reinterpret_cast<const float4 *>(bias + c2);
#pragma unroll
                for (int q = 0; q < 8; ++q) bv[q] = b4[q];
                umma::tmem_wait_ld();
#pragma unroll
              for (int half = 0; half < 2; ++half) {
                const int c = c2 + 16 * half;
                float v[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(half ? rb[i] : ra[i]);
#pragma unroll
                for (int q = 0; q < 4; ++q) {  // + bias, two lanes per paired add
                    const float4 b = bv[4 * half + q];
                    const float2 s0 = __fadd2_rn(make_float2(v[4 * q], v[4 * q + 1]), make_float2(b.x, b.y));
                    const float2 s1 = __fadd2_rn(make_float2(v[4 * q + 2], v[4 * q + 3]), make_float2(b.z, b.w));
                    v[4 * q] = s0.x; v[4 * q + 1] = s0.y; v[4 * q + 2] = s1.x; v[4 * q + 3] = s1.y;
                }
                if (l + 1 < kTcLayers) {
                    uint4 lo, hi;
                    lo.x = pack_silu2(v[0], v[1]);
                    lo.y = pack_silu2(v[2], v[3]);
                    lo.z = pack_silu2(v[4], v[5]);
                    lo.w = pack_silu2(v[6], v[7]);
                    hi.x = pack_silu2(v[8], v[9]);
                    hi.y = pack_silu2(v[10], v[11]);
                    hi.z = pack_silu2(v[12], v[13]);
                    hi.w = pack_silu2(v[14], v[15]);
                    *reinterpret_cast<uint4 *>(act + act_offset(r, c)) = lo;
                    *reinterpret_cast<uint4 *>(act + act_offset(r, c + 8)) = hi;
                } else {
                    const float4 *w4 = reinterpret_cast<const float4 *>(sW4 + 2 * c);
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float4 w = w4[q];  // rows c + 2q, c + 2q + 1, two outputs each
                        const float2 h = umma::silu2_f(make_float2(v[2 * q], v[2 * q + 1]));
                        // (o0, o1) += h_k (W4[k][0], W4[k][1]), the two outputs in one paired FMA
                        float2 o = __ffma2_rn(make_float2(h.x, h.x), make_float2(w.x, w.y), make_float2(o0, o1));
                        o = __ffma2_rn(make_float2(h.y, h.y), make_float2(w.z, w.w), o);
                        o0 = o.x;
                        o1 = o.y;
                    }
                }
              }
            }
        }
        // layer 4: the second half's partial sums through the (now free) activation tile
        float2 *part = reinterpret_cast<float2 *>(act);
        if (half == 1) part[r] = make_float2(o0, o1);
        if (__syncthreads_or((tid == 0 && !ok) || *abort_flag)) {
            if (tid == 0) *abort_flag = 1;
            break;
        }
        if (half == 0 && row < p.n) {
            const float2 q = part[r];
            float2 res;
            res.x = (o0 + q.x) + sB4[0];
            res.y = (o1 + q.y) + sB4[1];
            *reinterpret_cast<float2 *>(p.out + (size_t)row * kOut) = res;
        }
        __syncthreads();  // the partial sums are read before the next tile's layer 0 overwrites them
    }

    __syncthreads();
    if (tid == 0) {
        if (*abort_flag || !ok) {
            // drain: copies in flight land, committed MMAs complete (bounded)
            bool drained = true;
            for (uint32_t b = mm; b < ld; ++b) drained = umma::mbar_wait(full0 + 8 * (b % kStages), (b / kStages) & 1) && drained;
            if (mm > 0) drained = umma::mbar_wait(empty0 + 8 * ((mm - 1) % kStages), ((mm - 1) / kStages) & 1) && drained;
            (void)drained;
            if (p.err) atomicExch(p.err, 1);
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after_sync();
        umma::tmem_dealloc(tmem, kTmemCols);
    }
}

}  // namespace mlp
}  // namespace hwt
