// Plain FP64 GPU tree: one block per option, following the reference pricer's
// step structure (seq/Seq.hpp:24-179) literally.  Forward induction of the
// Arrow-Debreu prices with the alpha of every step fitted to the curve (the sum
// over the new row, log against the discount factor, Domain.hpp:98-104), then
// backward induction of the bond with the payoff at the maturity step and the
// reference's infinity clamps (Domain.hpp:147-169).  The scatter of the
// reference is written as a gather so every node is owned by one thread.
//
// Per-node exp(-(alpha_i + j dr) dt) is split into exp(-alpha_i dt) (one exp per
// step) times exp(-(j dr) dt) (one per column), so a node costs a handful of
// FP64 multiply-adds.  Rows, branching tables and the per-step discounts live in
// shared memory.
#include <float.h>

#include "hwt_internal.h"
#include "hwt_model.cuh"

namespace hwt {
namespace {

constexpr int kPlainThreads = 128;

__device__ __forceinline__ double block_sum(double v, double *red)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(kPlainThreads) plain_kernel(EngineParams p, int max_width, int max_height)
{
    extern __shared__ double sm[];
    __shared__ double red[kPlainThreads / 32];
    const int Wcap = max_width;
    double *up = sm, *stay = up + Wcap, *down = stay + Wcap, *G = down + Wcap;
    double *A = G + Wcap, *B = A + Wcap, *E = B + Wcap;  // E: max_height + 1
    const int tid = threadIdx.x;

    for (int opt = blockIdx.x; opt < p.opt.n; opt += gridDim.x) {
        if (p.s.keys[opt] < 0) continue;  // rejected by validation
        const Tree t = p.s.trees[opt];
        const int W = t.width, jc = t.jc, jmax = t.jmax, n = t.n;
        if (n <= 0) {
            if (tid == 0) p.out[t.idx] = 100.0;
            continue;
        }
        double jump_b = 0.0, jump_t = 0.0;
        for (int k = tid; k < W; k += blockDim.x) {
            const int j = k - jc;
            const Branch b = branch(j, jmax, t.M);
            up[k] = b.up; stay[k] = b.stay; down[k] = b.down;
            G[k] = column_discount(j, t.dr, t.dt);
            A[k] = (k == jc) ? 1.0 : 0.0;
            B[k] = 0.0;
        }
        if (t.edges) { jump_b = pu_b(-jmax, t.M); jump_t = pd_c(jmax, t.M); }
        if (tid == 0) {
            const double r0 = yield_at_year<double>(t.dt, t.term_unit, p.yc.rate, p.yc.day, p.yc.n);
            E[0] = exp(-r0 * t.dt);  // exp(-(alpha_0 + 0 dr) dt), Seq.hpp:58,70
        }
        __syncthreads();

        double *Q = A, *Qn = B;
        for (int i = 0; i < n; ++i) {
            const int jh = i < jmax ? i : jmax;          // source nodes |j| <= jh
            const int jh1 = (i + 1) < jmax ? i + 1 : jmax; // target nodes |j| <= jh1
            const double Ei = E[i];
            for (int k = jc - jh + tid; k <= jc + jh; k += blockDim.x) Q[k] *= Ei * G[k];
            __syncthreads();
            double part = 0.0;
            for (int k = jc - jh1 + tid; k <= jc + jh1; k += blockDim.x) {
                double v = stay[k] * Q[k];
                if (k >= 1) v += up[k - 1] * Q[k - 1];
                if (k + 1 < W) v += down[k + 1] * Q[k + 1];
                if (t.edges) {
                    if (k == 2) v += jump_b * Q[0];
                    if (k == W - 3) v += jump_t * Q[W - 1];
                }
                Qn[k] = v;
                part += v * G[k];
            }
            const double sum = block_sum(part, red);
            if (tid == 0) {
                const double ti = (i + 2) * t.dt;
                const double R = yield_at_year<double>(ti, t.term_unit, p.yc.rate, p.yc.day, p.yc.n);
                const double P = exp(-R * ti);
                const double alpha = log(sum / P) / t.dt;
                E[i + 1] = exp(-alpha * t.dt);
            }
            double *tmp = Q; Q = Qn; Qn = tmp;
            __syncthreads();
        }

        // Backward induction from the bond's face value.
        for (int k = tid; k < W; k += blockDim.x) { Q[k] = 100.0; Qn[k] = 0.0; }
        __syncthreads();
        double *C = Q, *Cn = Qn;
        for (int i = n - 1; i >= 0; --i) {
            const int jh = i < jmax ? i : jmax;
            const double Ei = E[i];
            const bool maturity = (i == t.m);
            for (int k = jc - jh + tid; k <= jc + jh; k += blockDim.x) {
                double v = stay[k] * C[k];
                if (k + 1 < W) v += up[k] * C[k + 1];
                if (k >= 1) v += down[k] * C[k - 1];
                if (t.edges) {
                    if (k == 0) v += jump_b * C[2];
                    if (k == W - 1) v += jump_t * C[W - 3];
                }
                double res = v * (Ei * G[k]);
                if (maturity) {
                    const double a = (t.type == 1) ? (t.X - res) : (res - t.X);
                    res = a < 0.0 ? 0.0 : a;
                }
                if (res == INFINITY) res = DBL_MAX;
                else if (res == -INFINITY) res = DBL_MIN;
                Cn[k] = res;
            }
            double *tmp = C; C = Cn; Cn = tmp;
            __syncthreads();
        }
        if (tid == 0) p.out[t.idx] = C[jc];
        __syncthreads();
    }
}

}  // namespace

size_t plain_smem_bytes(int max_width, int max_height)
{
    return sizeof(double) * ((size_t)6 * max_width + (size_t)max_height + 1);
}

cudaError_t launch_plain(const EngineParams &p, int max_width, int max_height, cudaStream_t stream)
{
    const size_t smem = plain_smem_bytes(max_width, max_height);
    cudaError_t e = cudaFuncSetAttribute(plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, plain_kernel, kPlainThreads, smem);
    if (per < 1) return cudaErrorInvalidConfiguration;
    int grid = sms * per;
    if (grid > p.opt.n) grid = p.opt.n;
    if (grid < 1) return cudaSuccess;
    plain_kernel<<<grid, kPlainThreads, smem, stream>>>(p, max_width, max_height);
    return cudaGetLastError();
}

}  // namespace hwt
