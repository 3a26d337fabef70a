// BF16 tensor-core GEMM for the surrogate MLP (forward, backward-data and
// backward-weight products), fp32 accumulation, fused epilogues.
//
//   C[M][N] = op(A)[M][K] * op(B)[K][N]
//   A: row-major [M][K] (TA = false) or stored [K][M] (TA = true)
//   B: stored [N][K], K contiguous (TB = false) or [K][N] (TB = true)
// Tiles of 128 x 128 x 32 per 256-thread block (8 warps as 2 x 4, warp tile
// 64 x 32), operands staged in shared memory in a K-contiguous layout and fed
// to mma.sync.m16n8k16 through ldmatrix.  Split-K over gridDim.z accumulates
// with atomics (weight gradients).  Every global access is bounds-checked; out
// of range operands are zero.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace hwt {
namespace mlp {

constexpr int BM = 128, BN = 128, BK = 32, LDS = BK + 8;  // +8 bf16 keeps ldmatrix rows conflict-free
constexpr int GEMM_THREADS = 256;

enum Epilogue : int {
    EPI_BIAS_SILU = 0,   // Z = acc + bias -> store Z (fp32) and silu(Z) (bf16)
    EPI_BIAS = 1,        // Y = acc + bias -> store fp32 (and bf16 if given)
    EPI_DSILU = 2,       // dZ = acc * silu'(Z) -> store bf16 (and fp32 if given)
    EPI_ATOMIC = 3,      // C += acc (fp32 atomics, split-K)
};

struct GemmArgs {
    const __nv_bfloat16 *A, *B;
    int M, N, K;
    int lda, ldb;        // leading dimensions of the stored arrays
    int k_chunk;         // K range per gridDim.z slice
    // epilogue
    const float *bias;   // [N]
    const float *Zin;    // [M][ldc] pre-activations (EPI_DSILU)
    float *Cf;           // [M][ldc] fp32 out
    __nv_bfloat16 *Cb;   // [M][ldcb] bf16 out
    int ldc, ldcb;
    int epi;
};

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + __expf(-z)); }

__device__ __forceinline__ float dsilu_f(float z)
{
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ void ldsm_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Stages a ROWS x BK tile of a K-contiguous operand (row r, col k) into sh[ROWS][LDS].
// trans: the array is stored [K][ROWS] (element (r, k) at k * ld + r).
template <int ROWS>
__device__ __forceinline__ void stage_tile(__nv_bfloat16 *sh, const __nv_bfloat16 *g, int row0, int k0, int rows,
                                           int kend, int ld, bool trans)
{
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    if (!trans) {
        // 8-element (16 B) chunks along K when aligned, else scalar
        const bool vec = (ld % 8 == 0) && ((reinterpret_cast<uintptr_t>(g) & 15) == 0);
        for (int idx = threadIdx.x; idx < ROWS * (BK / 8); idx += GEMM_THREADS) {
            const int r = idx / (BK / 8), c8 = (idx % (BK / 8)) * 8;
            const int gr = row0 + r, gk = k0 + c8;
            __nv_bfloat16 *dst = sh + r * LDS + c8;
            if (vec && gr < rows && gk + 8 <= kend) {
                *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(g + (size_t)gr * ld + gk);
            } else {
                for (int q = 0; q < 8; ++q)
                    dst[q] = (gr < rows && gk + q < kend) ? g[(size_t)gr * ld + gk + q] : zero;
            }
        }
    } else {
        for (int idx = threadIdx.x; idx < ROWS * BK; idx += GEMM_THREADS) {
            const int k = idx / ROWS, r = idx % ROWS;  // consecutive threads read consecutive rows
            const int gr = row0 + r, gk = k0 + k;
            sh[r * LDS + k] = (gr < rows && gk < kend) ? g[(size_t)gk * ld + gr] : zero;
        }
    }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(GEMM_THREADS) gemm_kernel(GemmArgs p)
{
    __shared__ __align__(16) __nv_bfloat16 sA[BM * LDS];
    __shared__ __align__(16) __nv_bfloat16 sB[BN * LDS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 2) * 64, wn = (warp & 3) * 32;  // warp tile origin in the block tile
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kbeg = blockIdx.z * p.k_chunk;
    int kend = kbeg + p.k_chunk;
    if (kend > p.K) kend = p.K;

    float acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        stage_tile<BM>(sA, p.A, m0, k0, p.M, kend, p.lda, TA);
        stage_tile<BN>(sB, p.B, n0, k0, p.N, kend, p.ldb, TB);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t a[4][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = wm + i * 16 + (lane & 15), c = kk + (lane >> 4) * 8;
                ldsm_x4(a[i][0], a[i][1], a[i][2], a[i][3], sA + r * LDS + c);
            }
#pragma unroll
            for (int j = 0; j < 4; j += 2) {
                const int r = wn + j * 8 + (lane & 7) + ((lane >> 4) << 3), c = kk + ((lane >> 3) & 1) * 8;
                ldsm_x4(b[j][0], b[j][1], b[j + 1][0], b[j + 1][1], sB + r * LDS + c);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j][0], b[j][1]);
        }
        __syncthreads();
    }

    // epilogue: fragment (i, j, q) is row wm + 16 i + g (+8 for q >= 2), col wn + 8 j + 2 t (+1 for odd q)
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int m = m0 + wm + i * 16 + g + ((q >> 1) << 3);
                const int n = n0 + wn + j * 8 + 2 * t + (q & 1);
                if (m >= p.M || n >= p.N) continue;
                float v = acc[i][j][q];
                switch (p.epi) {
                    case EPI_BIAS_SILU: {
                        const float z = v + p.bias[n];
                        if (p.Cf) p.Cf[(size_t)m * p.ldc + n] = z;
                        p.Cb[(size_t)m * p.ldcb + n] = __float2bfloat16(silu_f(z));
                        break;
                    }
                    case EPI_BIAS: {
                        const float y = v + (p.bias ? p.bias[n] : 0.f);
                        if (p.Cf) p.Cf[(size_t)m * p.ldc + n] = y;
                        if (p.Cb) p.Cb[(size_t)m * p.ldcb + n] = __float2bfloat16(y);
                        break;
                    }
                    case EPI_DSILU: {
                        const float d = v * dsilu_f(p.Zin[(size_t)m * p.ldc + n]);
                        if (p.Cf) p.Cf[(size_t)m * p.ldc + n] = d;
                        p.Cb[(size_t)m * p.ldcb + n] = __float2bfloat16(d);
                        break;
                    }
                    default:
                        atomicAdd(p.Cf + (size_t)m * p.ldc + n, v);
                        break;
                }
            }
        }
    }
}

}  // namespace mlp
}  // namespace hwt
