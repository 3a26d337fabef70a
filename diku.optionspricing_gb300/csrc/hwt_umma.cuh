// BF16 GEMM on the 5th-generation tensor cores (tcgen05) for the surrogate MLP:
// forward, backward-data and backward-weight products, fp32 accumulation in
// tensor memory (TMEM), fused epilogues.
//
//   C[M][N] = op(A)[M][K] * op(B)[K][N]
//   A: row-major [M][K] (TA = false) or stored [K][M] (TA = true)
//   B: stored [N][K], K contiguous (TB = false) or [K][N] (TB = true)
//
// One CTA of 128 threads computes a 128 x BN tile (BN = 16..256, a multiple of
// 16) with one tcgen05.mma.cta_group::1.kind::f16 per 16-wide K step (M = 128,
// N = BN), accumulating in BN columns of TMEM.  K advances in blocks of 64 through
// STAGES shared-memory stages filled by cp.async (16-byte chunks, zero fill past
// the edges), STAGES - 1 blocks ahead of the tensor core.  One thread issues a
// block's four MMAs and commits them to the stage's mbarrier; a stage is refilled
// once the MMAs that read it have completed.  Operands sit in shared memory in the
// canonical layouts without swizzle, made of 8 x 8 "core matrices" of 128
// contiguous bytes: K-major for operands stored with K contiguous, MN-major for
// operands stored transposed (the weight-gradient product), so that every copy
// moves 16 contiguous bytes.  In both layouts the descriptors' leading byte offset
// is the K-direction core-matrix stride and the stride byte offset the
// MN-direction one (each reading checked on GB300 against the swapped one).  The epilogue reads the accumulator
// with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = tile rows), 16 columns at
// a time, and applies the surrogate's fused operations (bias + SiLU, bias,
// dY * SiLU'(Z), split-K partials per slice or atomics) with 16-byte loads and stores.
//
// Every wait on an mbarrier is bounded: past the limit the CTA raises *err, stops
// issuing work, waits (bounded) for the MMAs it already committed, frees its TMEM
// and returns.  test_stall injects a wait that nothing completes: 1 before any MMA,
// 2 after the first K block's MMAs were committed.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace hwt {
namespace umma {

constexpr int BM = 128;           // rows per tile (the MMA's M)
constexpr int BK = 64;            // K per stage (four 16-wide MMAs)
constexpr int THREADS = 128;
constexpr int STAGES = 3;
constexpr uint64_t kWaitNs = 250000000ull;  // an mbarrier wait gives up after 0.25 s

enum Epilogue : int {
    EPI_BIAS_SILU = 0,   // Z = acc + bias -> store Z (fp32) and silu(Z) (bf16)
    EPI_BIAS = 1,        // Y = acc + bias -> store fp32 (and bf16 if given)
    EPI_DSILU = 2,       // dZ = acc * silu'(Z) -> store bf16 (and fp32 if given)
    EPI_ATOMIC = 3,      // C += acc (fp32 atomics, split-K)
    EPI_SLICE = 4,       // C[z] = acc: split-K slice z's partial (fp32), summed in order afterwards
};

struct GemmArgs {
    const __nv_bfloat16 *A, *B;
    int M, N, K;
    int lda, ldb;        // leading dimensions of the stored arrays
    int k_chunk;         // K range per gridDim.z slice (a multiple of BK)
    const float *bias;   // [N]
    const float *Zin;    // [M][ldc] pre-activations (EPI_DSILU)
    float *Cf;           // [M][ldc] fp32 out
    __nv_bfloat16 *Cb;   // [M][ldcb] bf16 out
    int ldc, ldcb;
    int epi;
    int *err;            // set to 1 by a CTA whose mbarrier wait ran out
    int test_stall;      // fault injection: 1 = before any MMA, 2 = after block 0's MMAs, a wait
                         // on a phase nothing completes
};

// Dynamic shared memory of one CTA for tile width bn.
__host__ __device__ constexpr int smem_bytes(int bn) { return STAGES * (BM + bn) * BK * 2 + 64; }

// TMEM columns to allocate for bn accumulator columns (a power of two >= 32).
__host__ __device__ constexpr int tmem_cols(int bn) { return bn <= 32 ? 32 : (bn <= 64 ? 64 : (bn <= 128 ? 128 : 256)); }

// Hardware tanh approximation (one MUFU operation, PTX tanh.approx.f32).
__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// SiLU z * sigmoid(z) with sigmoid(z) = (1 + tanh(z / 2)) / 2: with h = z / 2,
// silu = h + h tanh(h), one MUFU operation per activation (the exp-and-reciprocal
// form takes two, and the activations of the fused network are MUFU-bound).  Its
// error (~5e-4 |z| at most) is below the bf16 rounding the activations then take.
__device__ __forceinline__ float silu_f(float z)
{
    const float h = 0.5f * z;
    return fmaf(h, tanh_approx(h), h);
}

// silu_f on a pair with the paired FP32 instructions (each lane rounds as the scalar
// code: the same bits, half the FP32 instruction issues).
__device__ __forceinline__ float2 silu2_f(float2 z)
{
    const float2 h = __fmul2_rn(make_float2(0.5f, 0.5f), z);
    return __ffma2_rn(h, make_float2(tanh_approx(h.x), tanh_approx(h.y)), h);
}

// d silu / dz = s (1 + z (1 - s)) with the same sigmoid s.
__device__ __forceinline__ float dsilu_f(float z)
{
    const float s = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
    return s * fmaf(z, 1.0f - s, 1.0f);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading / stride byte offsets
// (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // version
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor, kind::f16: D fp32, A and B bf16, both K-major, M = 128, N = bn.
__host__ __device__ constexpr uint32_t make_idesc(int bn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the mbarrier phase with the given parity; false once kWaitNs have
// passed (global timer) without it.  mbarrier.try_wait suspends the thread in
// hardware until the phase completes or a 20 us hint elapses, so a completed phase
// wakes the waiter at once (a polling loop with sleeps overshoots).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    uint64_t t0 = 0;
    for (unsigned i = 0;; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity), "r"(20000u)
            : "memory");
        if (done) return true;
        if (i == 0) t0 = global_ns();
        else if (global_ns() - t0 > kWaitNs) return false;
    }
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Makes this thread's generic-proxy shared-memory writes visible to the tensor core.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// Arrives once on the mbarrier when every tcgen05 operation this thread issued has completed.
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive fp32 accumulator columns of this thread's TMEM lane, without
// waiting: the registers are valid after tmem_wait_ld().
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16 consecutive fp32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Element offset of (row r, k) in a K-major no-swizzle tile with BK columns.
__device__ __forceinline__ int core_offset(int r, int k) { return (((r >> 3) * (BK / 8) + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7); }

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Element offset of (row r, k) in an MN-major no-swizzle tile of ROWS rows: a core
// matrix holds 8 K-rows of 8 consecutive rows (16 bytes each); MN-adjacent core
// matrices are 128 bytes apart, K-adjacent ones (ROWS / 8) * 128 bytes.
template <int ROWS>
__device__ __forceinline__ int mn_offset(int r, int k) { return (((k >> 3) * (ROWS / 8) + (r >> 3)) << 6) + ((k & 7) << 3) + (r & 7); }

// Stages rows [row0, row0+ROWS) x K [k0, k0+BK) of an operand into sh; elements
// past the edges are zero.
//  * TRANS = false (element (r, k) at r * ld + k): K-major tile;
//  * TRANS = true (element (r, k) at k * ld + r): MN-major tile,
// so that both read 16 contiguous bytes per copy.  With `vec` (ld % 8 == 0 and a
// 16-byte aligned base) every 16-byte chunk is one cp.async whose byte count
// zero-fills what lies past the edge, and a warp writes whole core matrices;
// otherwise element copies.
template <int ROWS, bool TRANS>
__device__ __forceinline__ void stage(__nv_bfloat16 *sh, const __nv_bfloat16 *g, int row0, int k0, int rows, int kend,
                                      int ld, bool vec)
{
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    if (vec) {
        for (int idx = threadIdx.x; idx < ROWS * (BK / 8); idx += THREADS) {
            int n = 0;  // valid elements of the chunk (0..8)
            const __nv_bfloat16 *src = g;
            __nv_bfloat16 *dst;
            if (!TRANS) {
                // lane -> (row, 8-wide K chunk): one core-matrix row each
                const int r = idx / (BK / 8), k = (idx % (BK / 8)) * 8;
                const int gr = row0 + r, gk = k0 + k;
                n = gr < rows ? max(0, min(8, kend - gk)) : 0;
                if (n) src = g + (size_t)gr * ld + gk;
                dst = sh + core_offset(r, k);
            } else {
                // lane -> (k & 7, 8-row chunk, k / 8): 8 lanes fill one core matrix
                const int kl = idx & 7, rest = idx >> 3;
                const int rc = rest % (ROWS / 8), kh = rest / (ROWS / 8);
                const int r = rc * 8, k = kh * 8 + kl;
                const int gr = row0 + r, gk = k0 + k;
                n = gk < kend ? max(0, min(8, rows - gr)) : 0;
                if (n) src = g + (size_t)gk * ld + gr;
                dst = sh + mn_offset<ROWS>(r, k);
            }
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(2 * n)
                         : "memory");
        }
    } else if (!TRANS) {
        for (int idx = threadIdx.x; idx < ROWS * BK; idx += THREADS) {
            const int r = idx / BK, k = idx % BK;
            const int gr = row0 + r, gk = k0 + k;
            sh[core_offset(r, k)] = (gr < rows && gk < kend) ? g[(size_t)gr * ld + gk] : zero;
        }
    } else {
        for (int idx = threadIdx.x; idx < ROWS * BK; idx += THREADS) {
            const int k = idx / ROWS, r = idx % ROWS;  // consecutive threads read consecutive rows
            const int gr = row0 + r, gk = k0 + k;
            sh[mn_offset<ROWS>(r, k)] = (gr < rows && gk < kend) ? g[(size_t)gk * ld + gr] : zero;
        }
    }
}

// Descriptor of the 16-wide K step kk of a staged tile of ROWS rows.
template <int ROWS, bool TRANS>
__device__ __forceinline__ uint64_t step_desc(uint32_t base, int kk)
{
    if (!TRANS) return make_desc(base + kk * 256, 128, (BK / 8) * 128);
    return make_desc(base + kk * 2 * (ROWS / 8) * 128, (ROWS / 8) * 128, 128);
}

template <bool TA, bool TB, int BN>
__global__ void __launch_bounds__(THREADS) umma_gemm_kernel(GemmArgs p)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __nv_bfloat16 *sA[STAGES], *sB[STAGES];
#pragma unroll
    for (int s = 0; s < STAGES; ++s) {
        sA[s] = reinterpret_cast<__nv_bfloat16 *>(smem) + s * (BM + BN) * BK;
        sB[s] = sA[s] + BM * BK;
    }
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + STAGES * (BM + BN) * BK * 2);  // STAGES + "never"
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + STAGES + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kbeg = blockIdx.z * p.k_chunk;
    const int kend = min(kbeg + p.k_chunk, p.K);
    constexpr int NCOLS = tmem_cols(BN);
    constexpr uint32_t IDESC = make_idesc(BN) | ((TA ? 1u : 0u) << 15) | ((TB ? 1u : 0u) << 16);  // MN-major bits

    if (threadIdx.x == 0) {
        for (int s = 0; s <= STAGES; ++s) mbar_init(smem_u32(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(tmem_slot), NCOLS);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    // 16-byte chunks start at multiples of 8 elements: along K for K-major operands
    // (kbeg % 8 == 0), along the rows for MN-major ones (tile origins are multiples of 16)
    const bool vecA = (p.lda % 8 == 0) && ((reinterpret_cast<uintptr_t>(p.A) & 15) == 0) && (TA || kbeg % 8 == 0);
    const bool vecB = (p.ldb % 8 == 0) && ((reinterpret_cast<uintptr_t>(p.B) & 15) == 0) && (TB || kbeg % 8 == 0);
    int nkb = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;
    int issued = 0;  // K blocks whose MMAs were committed
    bool ok = true;
    if (p.test_stall == 1) {
        // a fresh mbarrier's phase 0 never completes without arrivals: the bounded
        // wait runs out, and the CTA skips its work and reports it
        ok = mbar_wait(smem_u32(&bars[0]), 0u);
        if (!ok) nkb = 0;
    }
    auto load = [&](int kb) {
        const int s = kb % STAGES, k0 = kbeg + kb * BK;
        stage<BM, TA>(sA[s], p.A, m0, k0, p.M, kend, p.lda, vecA);
        stage<BN, TB>(sB[s], p.B, n0, k0, p.N, kend, p.ldb, vecB);
    };
    // prologue: the first STAGES - 1 blocks in flight (one cp.async group each)
#pragma unroll
    for (int kb = 0; kb < STAGES - 1; ++kb) {
        if (kb < nkb) load(kb);
        cp_async_commit();
    }
    for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % STAGES;
        cp_async_wait<STAGES - 2>();  // this thread's copies of block kb have landed
        fence_proxy_async();          // ... and are visible to the tensor core
        __syncthreads();
        if (threadIdx.x == 0) {
            fence_after_sync();
            const uint32_t a0 = smem_u32(sA[s]), b0 = smem_u32(sB[s]);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk)
                mma_bf16(tmem, step_desc<BM, TA>(a0, kk), step_desc<BN, TB>(b0, kk), IDESC, (kb > 0 || kk > 0) ? 1u : 0u);
            mma_commit(smem_u32(&bars[s]));
        }
        issued = kb + 1;
        if (p.test_stall == 2 && kb == 0) {
            // injected: a phase nothing completes, with block 0's MMAs in flight
            ok = mbar_wait(smem_u32(&bars[STAGES]), 0u);
            __syncthreads_and(ok ? 1 : 0);
            ok = false;
            break;
        }
        // refill the stage block kb - 1 used, once its MMAs are done
        const int nb = kb + STAGES - 1;
        if (nb < nkb) {
            if (kb >= 1) {
                const int pb = kb - 1;
                ok = mbar_wait(smem_u32(&bars[pb % STAGES]), (uint32_t)((pb / STAGES) & 1));
            }
            if (__syncthreads_and(ok ? 1 : 0) == 0) {
                ok = false;
                break;
            }
            load(nb);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    // The last commit covers every MMA this CTA issued: wait for it (bounded) before
    // the epilogue reads TMEM or, after a wait that ran out, before TMEM is freed.
    // If this wait runs out too, the tensor core is not completing work; the CTA
    // then frees TMEM and returns with *err raised all the same.
    bool done = true;
    if (issued > 0) {
        const int last = issued - 1;
        done = mbar_wait(smem_u32(&bars[last % STAGES]), (uint32_t)((last / STAGES) & 1));
    }
    if (!ok || !done) {
        if (p.err) atomicExch(p.err, 1);
    }
    fence_after_sync();
    // (a split-K slice with no K block has nothing to add)
    const bool good = __syncthreads_and((ok && done && issued == nkb && nkb > 0) ? 1 : 0) != 0;

    if (good) {
        const int m = m0 + warp * 32 + lane;  // this thread's tile row = TMEM lane
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        auto al16 = [](const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
        const bool vf = (p.ldc % 4 == 0) && al16(p.Cf) && al16(p.Zin) && al16(p.bias) && (p.bias == nullptr || n0 % 4 == 0);
        const bool vb = (p.ldcb % 8 == 0) && al16(p.Cb);
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
            float v[16];
            tmem_ld16(trow + (uint32_t)c, v);
            const int n = n0 + c;
            if (m >= p.M || n >= p.N) continue;
            const bool full = n + 16 <= p.N;
            if (full && vf && (p.epi == EPI_ATOMIC || p.epi == EPI_SLICE || vb || !p.Cb)) {
                float4 *cf = p.Cf ? reinterpret_cast<float4 *>(p.Cf + (size_t)m * p.ldc + n) : nullptr;
                if (p.epi == EPI_SLICE) {
                    float4 *cz = reinterpret_cast<float4 *>(p.Cf + ((size_t)blockIdx.z * p.M + m) * p.ldc + n);
#pragma unroll
                    for (int q = 0; q < 4; ++q) cz[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    continue;
                }
                if (p.epi == EPI_ATOMIC) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) atomicAdd(cf + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
                    continue;
                }
                if (p.epi == EPI_DSILU) {
                    const float4 *zin = reinterpret_cast<const float4 *>(p.Zin + (size_t)m * p.ldc + n);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float4 z = zin[q];
                        v[4 * q] *= dsilu_f(z.x); v[4 * q + 1] *= dsilu_f(z.y);
                        v[4 * q + 2] *= dsilu_f(z.z); v[4 * q + 3] *= dsilu_f(z.w);
                    }
                } else if (p.bias) {
                    const float4 *b4 = reinterpret_cast<const float4 *>(p.bias + n);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float4 b = b4[q];
                        v[4 * q] += b.x; v[4 * q + 1] += b.y; v[4 * q + 2] += b.z; v[4 * q + 3] += b.w;
                    }
                }
                if (cf) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) cf[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
                if (p.Cb) {
                    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16(p.epi == EPI_BIAS_SILU ? silu_f(v[i]) : v[i]);
                    uint4 *cb = reinterpret_cast<uint4 *>(p.Cb + (size_t)m * p.ldcb + n);
                    cb[0] = reinterpret_cast<const uint4 *>(h)[0];
                    cb[1] = reinterpret_cast<const uint4 *>(h)[1];
                }
                continue;
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int nn = n + i;
                if (nn >= p.N) break;
                const float a = v[i];
                switch (p.epi) {
                    case EPI_BIAS_SILU: {
                        const float z = a + p.bias[nn];
                        if (p.Cf) p.Cf[(size_t)m * p.ldc + nn] = z;
                        p.Cb[(size_t)m * p.ldcb + nn] = __float2bfloat16(silu_f(z));
                        break;
                    }
                    case EPI_BIAS: {
                        const float y = a + (p.bias ? p.bias[nn] : 0.f);
                        if (p.Cf) p.Cf[(size_t)m * p.ldc + nn] = y;
                        if (p.Cb) p.Cb[(size_t)m * p.ldcb + nn] = __float2bfloat16(y);
                        break;
                    }
                    case EPI_DSILU: {
                        const float d = a * dsilu_f(p.Zin[(size_t)m * p.ldc + nn]);
                        if (p.Cf) p.Cf[(size_t)m * p.ldc + nn] = d;
                        p.Cb[(size_t)m * p.ldcb + nn] = __float2bfloat16(d);
                        break;
                    }
                    case EPI_SLICE:
                        p.Cf[((size_t)blockIdx.z * p.M + m) * p.ldc + nn] = a;
                        break;
                    default:
                        if (a != 0.f) atomicAdd(p.Cf + (size_t)m * p.ldc + nn, a);
                        break;
                }
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        tmem_dealloc(tmem, NCOLS);
    }
}

}  // namespace umma
}  // namespace hwt
