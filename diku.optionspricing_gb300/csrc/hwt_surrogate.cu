// Learned surrogate: a 7 -> 256 -> 256 -> 256 -> 256 -> 1 SiLU MLP that maps
// standardised option parameters to price / forward bond price.  Weights are
// kept as fp32 masters with bf16 copies for the tcgen05 tensor-core GEMMs
// (hwt_umma.cuh); activations between layers are bf16, accumulation fp32 in
// tensor memory.
// Training: Adam with cosine decay on labels priced by the batched FP64 tree.
// Inference: options inside the training box go through the network, the rest
// to the tree; a random sample of the in-box options is re-priced by the tree
// as the judge of every batch.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/hwtree.h"
#include "hwt_internal.h"
#include "hwt_umma.cuh"
#include "hwt_model.cuh"

using namespace hwt;
using namespace hwt::umma;

namespace {

constexpr int kLayers = 5;
constexpr int kIn = 7, kInPad = 8, kHidden = 256;
const int kFanIn[kLayers] = {kInPad, kHidden, kHidden, kHidden, kHidden};
const int kFanOut[kLayers] = {kHidden, kHidden, kHidden, kHidden, 1};
constexpr int kChunk = 65536;  // samples per inference pass

struct FeatureNorm {
    float mean[kIn], inv_std[kIn];
};

// ---------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------

// Hull-White closed-form price of a European option on a zero-coupon bond
// (Jamshidian 1989) with face 100: the control variate of the residual network.
__device__ double hw_closed_form(double t, double T, double X, double a, double sigma, double Pt, double PT, int type)
{
    const double B = -expm1(-a * (T - t)) / a;
    const double sp = sigma * B * sqrt(-expm1(-2.0 * a * t) / (2.0 * a));
    const double bond = 100.0 * PT, strike = X * Pt;
    if (!(sp > 1e-12)) return type == 1 ? fmax(strike - bond, 0.0) : fmax(bond - strike, 0.0);
    const double h = log(bond / strike) / sp + 0.5 * sp;
    return type == 1 ? strike * normcdf(-h + sp) - bond * normcdf(-h) : bond * normcdf(h) - strike * normcdf(h - sp);
}

// Features, forward bond price, control-variate price and in-box flag of each option.
__global__ void features_kernel(DevOptions o, DevYield yc, hwt_box box, FeatureNorm fn, __nv_bfloat16 *X,
                                double *F, double *base, uint8_t *inbox)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= o.n) return;
    const double t = o.option_maturity[i], T = o.bond_maturity[i];
    const int tu = o.term_unit[i];
    const double Pt = exp(-yield_at_year<double>(t, tu, yc.rate, yc.day, yc.n) * t);
    const double PT = exp(-yield_at_year<double>(T, tu, yc.rate, yc.day, yc.n) * T);
    const double fwd = 100.0 * PT / Pt;
    const double mny = o.strike[i] / fwd;
    const double a = o.a[i], sg = o.sigma[i];
    const int steps = o.term_steps[i];
    const double v[kIn] = {t, T, mny, a, sg, (double)steps, (double)o.type[i]};
#pragma unroll
    for (int q = 0; q < kIn; ++q) X[(size_t)i * kInPad + q] = __float2bfloat16(((float)v[q] - fn.mean[q]) * fn.inv_std[q]);
    X[(size_t)i * kInPad + kIn] = __float2bfloat16(0.f);
    F[i] = fwd;
    base[i] = box.residual ? hw_closed_form(t, T, o.strike[i], a, sg, Pt, PT, o.type[i]) : 0.0;
    const double span = T - t;
    const bool in = t >= box.t_min && t <= box.t_max && span >= box.span_min && span <= box.span_max &&
                    mny >= box.moneyness_min && mny <= box.moneyness_max && a >= box.a_min && a <= box.a_max &&
                    sg >= box.sigma_min && sg <= box.sigma_max && steps >= box.steps_min && steps <= box.steps_max &&
                    tu == box.term_unit && (o.type[i] == 0 || o.type[i] == 1) && isfinite(mny);
    inbox[i] = in ? 1 : 0;
}

// r = out - y; dZ = r / n (bf16 operand of the backward GEMMs); loss += 0.5 r^2 / n
__global__ void loss_kernel(const float *out, const float *y, int n, __nv_bfloat16 *dZ, float *dZf, double *loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (i < n) {
        const float r = out[i] - y[i];
        const float d = r / (float)n;
        dZ[i] = __float2bfloat16(d);
        dZf[i] = d;
        l = 0.5 * (double)r * (double)r / n;
    }
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l);
}

// db[c] += sum over rows of d[r][c]  (d fp32 [n][ld])
__global__ void colsum_kernel(const float *d, int n, int cols, int ld, float *db)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    const int rows_per = (n + gridDim.y - 1) / gridDim.y;
    const int r0 = blockIdx.y * rows_per, r1 = min(n, r0 + rows_per);
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;  // four independent chains of loads
    int r = r0;
    for (; r + 4 <= r1; r += 4) {
        s0 += d[(size_t)r * ld + c];
        s1 += d[(size_t)(r + 1) * ld + c];
        s2 += d[(size_t)(r + 2) * ld + c];
        s3 += d[(size_t)(r + 3) * ld + c];
    }
    for (; r < r1; ++r) s0 += d[(size_t)r * ld + c];
    atomicAdd(db + c, (s0 + s1) + (s2 + s3));
}

struct AdamArgs {
    float *w, *m, *v;
    const float *g;
    int n;
    float lr, b1, b2, eps, c1, c2;
};

// Per-step training state kept on the device, so that one captured CUDA graph
// serves every step: the Adam step count t, the step index in the learning-rate
// schedule, the batch index within the epoch, and the step's lr and bias corrections.
struct StepState {
    long long t;     // Adam steps taken
    long long step;  // schedule position within this training call
    int k;           // next batch of the epoch
    int cur;         // batch this step trains on
    float lr, c1, c2;
};

__global__ void step_begin_kernel(StepState *st, double lr0, double lr_min, long long total)
{
    const long long t = st->t + 1;
    st->t = t;
    const double step = (double)st->step;
    st->step = st->step + 1;
    st->lr = (float)(lr_min + 0.5 * (lr0 - lr_min) * (1.0 + cos(3.14159265358979323846 * step / (double)total)));
    st->c1 = 1.f - powf(0.9f, (float)t);
    st->c2 = 1.f - powf(0.999f, (float)t);
    st->cur = st->k;
    st->k = st->k + 1;
}

// Batch `cur` of the shuffled samples into the fixed input and target buffers.
__global__ void batch_copy_kernel(const __nv_bfloat16 *Xs, const float *ys, const StepState *st, int batch,
                                  __nv_bfloat16 *X, float *y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch) return;
    const size_t row = (size_t)st->cur * batch + i;
    *reinterpret_cast<uint4 *>(X + (size_t)i * kInPad) = *reinterpret_cast<const uint4 *>(Xs + row * kInPad);
    y[i] = ys[row];
}

// Adam with lr and bias corrections from the args, or from the step state if given.
__global__ void adam_kernel(AdamArgs a, const StepState *st)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if (st) {
        a.lr = st->lr;
        a.c1 = st->c1;
        a.c2 = st->c2;
    }
    const float g = a.g[i];
    const float m = a.b1 * a.m[i] + (1.f - a.b1) * g;
    const float v = a.b2 * a.v[i] + (1.f - a.b2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    a.w[i] -= a.lr * (m / a.c1) / (sqrtf(v / a.c2) + a.eps);
}

// bf16 copies of W[in][out]: Wt[out][in_pad] (forward operand) and Wb[in_pad][out]
__global__ void refresh_kernel(const float *W, int in, int in_pad, int out, __nv_bfloat16 *Wt, __nv_bfloat16 *Wb)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= in_pad * out) return;
    const int k = idx / out, n = idx % out;
    const __nv_bfloat16 v = __float2bfloat16(k < in ? W[(size_t)k * out + n] : 0.f);
    Wt[(size_t)n * in_pad + k] = v;
    Wb[(size_t)k * out + n] = v;
}

__global__ void gather_rows_kernel(const __nv_bfloat16 *X, const float *y, const int32_t *perm, int n,
                                   __nv_bfloat16 *Xo, float *yo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = perm[i];
    *reinterpret_cast<uint4 *>(Xo + (size_t)i * kInPad) = *reinterpret_cast<const uint4 *>(X + (size_t)s * kInPad);
    yo[i] = y[s];
}

__global__ void targets_kernel(const double *price, const double *F, const double *base, int n, double ymean,
                               double yinv, float *y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)(((price[i] - base[i]) / F[i] - ymean) * yinv);
}

// Price from the network output for in-box options.
__global__ void decode_kernel(const float *out, const double *F, const double *base, const uint8_t *inbox, int n,
                              double ymean, double ystd, double *price)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && inbox[i]) price[i] = base[i] + F[i] * ((double)out[i] * ystd + ymean);
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Tree work list: out-of-box options, and in-box options drawn for the judge.
// kind: 1 = routed, 2 = judged.
__global__ void route_kernel(const uint8_t *inbox, int n, unsigned long long seed, unsigned long long thresh,
                             int32_t *list, uint8_t *kind, int32_t *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint8_t k = 0;
    if (!inbox[i]) k = 1;
    else if (mix64(seed ^ (unsigned long long)i) < thresh) k = 2;
    kind[i] = k;
    if (k) list[atomicAdd(count, 1)] = i;
}

__global__ void gather_options_kernel(DevOptions src, const int32_t *list, const int32_t *count, DevOptions dst_mut,
                                      double *strike, double *bm, double *om, uint16_t *tu, uint16_t *ts, double *a,
                                      double *sg, int8_t *ty)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *count) return;
    const int i = list[j];
    strike[j] = src.strike[i]; bm[j] = src.bond_maturity[i]; om[j] = src.option_maturity[i];
    tu[j] = src.term_unit[i]; ts[j] = src.term_steps[i]; a[j] = src.a[i]; sg[j] = src.sigma[i]; ty[j] = src.type[i];
    (void)dst_mut;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct hwt_surrogate {
    hwt_ctx *ctx = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    hwt_box box;
    FeatureNorm fn;
    double ymean = 0.0, ystd = 1.0;
    int trained = 0;
    std::string err;
    // parameters (fp32 masters) and Adam state, one flat buffer each
    size_t n_params = 0;
    float *d_w = nullptr, *d_m = nullptr, *d_v = nullptr, *d_g = nullptr;
    size_t w_off[kLayers], b_off[kLayers];
    __nv_bfloat16 *d_wt[kLayers] = {}, *d_wb[kLayers] = {};
    long adam_t = 0;
    // activations for one batch / chunk
    int act_cap = 0;
    __nv_bfloat16 *d_h[kLayers + 1] = {};  // h[0] = X, h[l+1] = silu(z_l) for l < 4
    float *d_z[kLayers] = {};              // pre-activations (z[4] = output)
    __nv_bfloat16 *d_dz = nullptr, *d_dz2 = nullptr;
    float *d_dzf = nullptr;
    double *d_loss = nullptr;
    float *d_y = nullptr;
    int *d_gemm_err = nullptr;  // raised by a GEMM whose mbarrier wait ran out
    int stall = 0;              // fault injection for tests (hwt_surrogate_inject_stall)
};

namespace {

int sfail(hwt_surrogate *s, int code, const std::string &m)
{
    s->err = m;
    return code;
}

#define SCUDA(s, call, what)                                                                      \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            cudaGetLastError();                                                                   \
            return sfail((s), e_ == cudaErrorMemoryAllocation ? HWT_ENOMEM : HWT_ECUDA,           \
                         std::string(what) + ": " + cudaGetErrorString(e_));                      \
        }                                                                                         \
    } while (0)

int ensure_act(hwt_surrogate *s, int rows)
{
    if (rows <= s->act_cap) return HWT_OK;
    for (int l = 0; l <= kLayers; ++l) { cudaFree(s->d_h[l]); s->d_h[l] = nullptr; }
    for (int l = 0; l < kLayers; ++l) { cudaFree(s->d_z[l]); s->d_z[l] = nullptr; }
    cudaFree(s->d_dz); cudaFree(s->d_dz2); cudaFree(s->d_dzf); cudaFree(s->d_y);
    SCUDA(s, cudaMalloc(&s->d_h[0], sizeof(__nv_bfloat16) * (size_t)rows * kInPad), "alloc X");
    for (int l = 1; l < kLayers; ++l) SCUDA(s, cudaMalloc(&s->d_h[l], sizeof(__nv_bfloat16) * (size_t)rows * kHidden), "alloc H");
    for (int l = 0; l < kLayers; ++l) SCUDA(s, cudaMalloc(&s->d_z[l], sizeof(float) * (size_t)rows * kFanOut[l]), "alloc Z");
    SCUDA(s, cudaMalloc(&s->d_dz, sizeof(__nv_bfloat16) * (size_t)rows * kHidden), "alloc dZ");
    SCUDA(s, cudaMalloc(&s->d_dz2, sizeof(__nv_bfloat16) * (size_t)rows * kHidden), "alloc dZ");
    SCUDA(s, cudaMalloc(&s->d_dzf, sizeof(float) * (size_t)rows * kHidden), "alloc dZf");
    SCUDA(s, cudaMalloc(&s->d_y, sizeof(float) * (size_t)rows), "alloc y");
    s->act_cap = rows;
    return HWT_OK;
}

template <bool TA, bool TB, int BN>
cudaError_t gemm_bn(const GemmArgs &a, int splits, cudaStream_t st)
{
    auto kern = umma_gemm_kernel<TA, TB, BN>;
    dim3 grid((a.N + BN - 1) / BN, (a.M + BM - 1) / BM, splits);
    kern<<<grid, THREADS, smem_bytes(BN), st>>>(a);
    return cudaGetLastError();
}

// Dynamic shared memory above 48 KB for every GEMM instantiation, once at set-up
// (outside any stream capture).
cudaError_t gemm_attributes()
{
    cudaError_t e = cudaSuccess;
    auto set = [&](auto kern, int bn) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(bn));
    };
    set(umma_gemm_kernel<false, false, 16>, 16);
    set(umma_gemm_kernel<false, false, 64>, 64);
    set(umma_gemm_kernel<false, false, 128>, 128);
    set(umma_gemm_kernel<true, true, 16>, 16);
    set(umma_gemm_kernel<true, true, 64>, 64);
    set(umma_gemm_kernel<true, true, 128>, 128);
    return e;
}

// Tile width: the output width rounded up to 16 (one tile for the 1-wide output
// layer), at most 128 so that a 256-wide layer spreads over two column tiles.
template <bool TA, bool TB>
cudaError_t gemm(const GemmArgs &a, int splits, cudaStream_t st)
{
    if (a.N <= 16) return gemm_bn<TA, TB, 16>(a, splits, st);
    if (a.N <= 64) return gemm_bn<TA, TB, 64>(a, splits, st);
    return gemm_bn<TA, TB, 128>(a, splits, st);
}

GemmArgs gargs(const hwt_surrogate *s, const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K, int lda,
               int ldb, int epi)
{
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.A = A; g.B = B; g.M = M; g.N = N; g.K = K; g.lda = lda; g.ldb = ldb; g.epi = epi;
    g.k_chunk = (K + BK - 1) / BK * BK;
    g.err = s->d_gemm_err;
    g.test_stall = s->stall;
    return g;
}

// HWT_ETIMEOUT (and the flag cleared) if a GEMM gave up waiting since the last check.
int gemm_status(hwt_surrogate *s)
{
    int flag = 0;
    SCUDA(s, cudaMemcpy(&flag, s->d_gemm_err, sizeof(int), cudaMemcpyDeviceToHost), "GEMM status");
    if (flag == 0) return HWT_OK;
    SCUDA(s, cudaMemset(s->d_gemm_err, 0, sizeof(int)), "GEMM status");
    return sfail(s, HWT_ETIMEOUT, "tensor-core GEMM: an mbarrier wait ran out");
}

// Forward through all layers for `rows` samples already in d_h[0].  Output
// (normalised) in d_z[4].
int forward(hwt_surrogate *s, int rows)
{
    for (int l = 0; l < kLayers; ++l) {
        const bool last = l == kLayers - 1;
        GemmArgs g = gargs(s, s->d_h[l], s->d_wt[l], rows, kFanOut[l], kFanIn[l], kFanIn[l], kFanIn[l],
                           last ? EPI_BIAS : EPI_BIAS_SILU);
        g.bias = s->d_w + s->b_off[l];
        g.Cf = s->d_z[l];
        g.ldc = kFanOut[l];
        g.Cb = last ? nullptr : s->d_h[l + 1];
        g.ldcb = kFanOut[l];
        SCUDA(s, (gemm<false, false>(g, 1, s->stream)), "forward gemm");
    }
    return HWT_OK;
}

// Loss and gradients (into d_g) for `rows` samples in d_h[0] with targets d_y.
int backward(hwt_surrogate *s, int rows, bool zero_loss)
{
    SCUDA(s, cudaMemsetAsync(s->d_g, 0, sizeof(float) * s->n_params, s->stream), "zero grads");
    if (zero_loss) SCUDA(s, cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream), "zero loss");
    loss_kernel<<<(rows + 255) / 256, 256, 0, s->stream>>>(s->d_z[kLayers - 1], s->d_y, rows, s->d_dz, s->d_dzf, s->d_loss);
    SCUDA(s, cudaGetLastError(), "loss kernel");
    __nv_bfloat16 *dz = s->d_dz, *dz_next = s->d_dz2;
    const int splits = std::max(1, std::min(64, rows / 512));
    int kc = (rows + splits - 1) / splits;
    kc = (kc + BK - 1) / BK * BK;
    for (int l = kLayers - 1; l >= 0; --l) {
        const int in = kFanIn[l], out = kFanOut[l];
        // dW_l[in][out] = H_l^T dZ_l   (split-K over the batch)
        GemmArgs gw = gargs(s, s->d_h[l], dz, in, out, rows, in, out, EPI_ATOMIC);
        gw.Cf = s->d_g + s->w_off[l];
        gw.ldc = out;
        gw.k_chunk = kc;
        SCUDA(s, (gemm<true, true>(gw, (rows + kc - 1) / kc, s->stream)), "dW gemm");
        // db_l = column sums of dZ_l (fp32 copy in d_dzf)
        dim3 cg((out + 255) / 256, std::max(1, std::min(256, rows / 32)));
        colsum_kernel<<<cg, 256, 0, s->stream>>>(s->d_dzf, rows, out, out, s->d_g + s->b_off[l]);
        SCUDA(s, cudaGetLastError(), "db kernel");
        if (l == 0) break;
        // dZ_{l-1} = (dZ_l W_l^T) * silu'(Z_{l-1})
        GemmArgs gd = gargs(s, dz, s->d_wb[l], rows, in, out, out, out, EPI_DSILU);
        gd.Zin = s->d_z[l - 1];
        gd.Cf = s->d_dzf;
        gd.ldc = in;
        gd.Cb = dz_next;
        gd.ldcb = in;
        SCUDA(s, (gemm<false, false>(gd, 1, s->stream)), "dX gemm");
        std::swap(dz, dz_next);
    }
    return HWT_OK;
}

int refresh(hwt_surrogate *s)
{
    for (int l = 0; l < kLayers; ++l) {
        const int in = l == 0 ? kIn : kFanIn[l];
        const int tot = kFanIn[l] * kFanOut[l];
        refresh_kernel<<<(tot + 255) / 256, 256, 0, s->stream>>>(s->d_w + s->w_off[l], in, kFanIn[l], kFanOut[l],
                                                               s->d_wt[l], s->d_wb[l]);
        SCUDA(s, cudaGetLastError(), "refresh kernel");
    }
    return HWT_OK;
}

// One training step on the batch the step state names, everything from device
// state: the body of the captured training graph.
int train_step(hwt_surrogate *s, const __nv_bfloat16 *Xs, const float *ys, StepState *st, int batch, double lr0,
               double lr_min, long long total)
{
    step_begin_kernel<<<1, 1, 0, s->stream>>>(st, lr0, lr_min, total);
    SCUDA(s, cudaGetLastError(), "step kernel");
    batch_copy_kernel<<<(batch + 255) / 256, 256, 0, s->stream>>>(Xs, ys, st, batch, s->d_h[0], s->d_y);
    SCUDA(s, cudaGetLastError(), "batch kernel");
    int r = forward(s, batch);
    if (!r) r = backward(s, batch, false);
    if (r) return r;
    AdamArgs a;
    a.w = s->d_w; a.m = s->d_m; a.v = s->d_v; a.g = s->d_g; a.n = (int)s->n_params;
    a.lr = 0.f; a.b1 = 0.9f; a.b2 = 0.999f; a.eps = 1e-8f; a.c1 = 1.f; a.c2 = 1.f;
    adam_kernel<<<((int)s->n_params + 255) / 256, 256, 0, s->stream>>>(a, st);
    SCUDA(s, cudaGetLastError(), "adam kernel");
    return refresh(s);
}

void box_norm(const hwt_box &b, FeatureNorm &fn)
{
    const double lo[kIn] = {b.t_min, b.t_min + b.span_min, b.moneyness_min, b.a_min, b.sigma_min, (double)b.steps_min, 0.0};
    const double hi[kIn] = {b.t_max, b.t_max + b.span_max, b.moneyness_max, b.a_max, b.sigma_max, (double)b.steps_max, 1.0};
    for (int q = 0; q < kIn; ++q) {
        const double w = std::max(hi[q] - lo[q], 1e-12);
        fn.mean[q] = (float)(0.5 * (lo[q] + hi[q]));
        fn.inv_std[q] = (float)(1.0 / (w / sqrt(12.0)));
    }
}

}  // namespace

extern "C" {

hwt_surrogate *hwt_surrogate_create(hwt_ctx *ctx, const hwt_box *box, uint64_t seed)
{
    if (!ctx || !box) return nullptr;
    hwt_surrogate *s = new hwt_surrogate();
    s->ctx = ctx;
    s->box = *box;
    box_norm(*box, s->fn);
    cudaGetDevice(&s->device);
    bool ok = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess;
    size_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
        s->w_off[l] = off; off += (size_t)kFanIn[l] * kFanOut[l];
        s->b_off[l] = off; off += kFanOut[l];
    }
    s->n_params = off;
    ok = ok && cudaMalloc(&s->d_w, 4 * off) == cudaSuccess && cudaMalloc(&s->d_m, 4 * off) == cudaSuccess &&
         cudaMalloc(&s->d_v, 4 * off) == cudaSuccess && cudaMalloc(&s->d_g, 4 * off) == cudaSuccess &&
         cudaMalloc(&s->d_loss, sizeof(double)) == cudaSuccess &&
         cudaMalloc(&s->d_gemm_err, sizeof(int)) == cudaSuccess && cudaMemset(s->d_gemm_err, 0, sizeof(int)) == cudaSuccess;
    for (int l = 0; l < kLayers && ok; ++l) {
        ok = cudaMalloc(&s->d_wt[l], 2 * (size_t)kFanIn[l] * kFanOut[l]) == cudaSuccess &&
             cudaMalloc(&s->d_wb[l], 2 * (size_t)kFanIn[l] * kFanOut[l]) == cudaSuccess;
    }
    if (ok) {
        // He initialisation from a seeded host generator (splitmix64 + Box-Muller)
        std::vector<float> w(off, 0.f);
        unsigned long long st = seed ? seed : 0x1234567ull;
        auto next = [&]() {
            st += 0x9e3779b97f4a7c15ull;
            unsigned long long z = st;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
            return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
        };
        for (int l = 0; l < kLayers; ++l) {
            const int in = l == 0 ? kIn : kFanIn[l];
            const double sd = sqrt(2.0 / in) * (l == kLayers - 1 ? 0.1 : 1.0);
            for (int k = 0; k < in; ++k)
                for (int n = 0; n < kFanOut[l]; ++n) {
                    const double u1 = std::max(next(), 1e-300), u2 = next();
                    w[s->w_off[l] + (size_t)k * kFanOut[l] + n] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
                }
        }
        ok = cudaMemcpy(s->d_w, w.data(), 4 * off, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemset(s->d_m, 0, 4 * off) == cudaSuccess && cudaMemset(s->d_v, 0, 4 * off) == cudaSuccess;
        ok = ok && gemm_attributes() == cudaSuccess;
        ok = ok && refresh(s) == HWT_OK && cudaStreamSynchronize(s->stream) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        hwt_surrogate_destroy(s);
        return nullptr;
    }
    return s;
}

void hwt_surrogate_destroy(hwt_surrogate *s)
{
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->d_w); cudaFree(s->d_m); cudaFree(s->d_v); cudaFree(s->d_g); cudaFree(s->d_loss); cudaFree(s->d_gemm_err);
    for (int l = 0; l < kLayers; ++l) { cudaFree(s->d_wt[l]); cudaFree(s->d_wb[l]); cudaFree(s->d_z[l]); }
    for (int l = 0; l <= kLayers; ++l) cudaFree(s->d_h[l]);
    cudaFree(s->d_dz); cudaFree(s->d_dz2); cudaFree(s->d_dzf); cudaFree(s->d_y);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

const char *hwt_surrogate_last_error(const hwt_surrogate *s) { return s ? s->err.c_str() : "no surrogate"; }

int hwt_surrogate_inject_stall(hwt_surrogate *s, int on)
{
    if (!s) return HWT_EINVAL;
    s->stall = on ? 1 : 0;
    return HWT_OK;
}

int64_t hwt_surrogate_param_count(const hwt_surrogate *s) { return s ? (int64_t)s->n_params : 0; }

int hwt_surrogate_params(hwt_surrogate *s, float *buf, int64_t n, int set)
{
    if (!s || !buf || n != (int64_t)s->n_params) return HWT_EINVAL;
    if (set) {
        SCUDA(s, cudaMemcpy(s->d_w, buf, 4 * n, cudaMemcpyHostToDevice), "set params");
        int r = refresh(s);
        if (r) return r;
        SCUDA(s, cudaStreamSynchronize(s->stream), "refresh");
    } else {
        SCUDA(s, cudaMemcpy(buf, s->d_w, 4 * n, cudaMemcpyDeviceToHost), "get params");
    }
    return HWT_OK;
}

int hwt_surrogate_forward(hwt_surrogate *s, const float *x, int n, float *out)
{
    if (!s || !x || !out || n <= 0) return HWT_EINVAL;
    int r = ensure_act(s, n);
    if (r) return r;
    std::vector<__nv_bfloat16> xb((size_t)n * kInPad);
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < kInPad; ++q) xb[(size_t)i * kInPad + q] = __float2bfloat16(q < kIn ? x[(size_t)i * kIn + q] : 0.f);
    SCUDA(s, cudaMemcpy(s->d_h[0], xb.data(), 2 * xb.size(), cudaMemcpyHostToDevice), "x H2D");
    if ((r = forward(s, n))) return r;
    SCUDA(s, cudaMemcpyAsync(out, s->d_z[kLayers - 1], 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "out D2H");
    SCUDA(s, cudaStreamSynchronize(s->stream), "forward");
    return gemm_status(s);
}

int hwt_surrogate_loss_grads(hwt_surrogate *s, const float *x, const float *y, int n, double *loss, float *grads)
{
    if (!s || !x || !y || n <= 0) return HWT_EINVAL;
    int r = ensure_act(s, n);
    if (r) return r;
    std::vector<__nv_bfloat16> xb((size_t)n * kInPad);
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < kInPad; ++q) xb[(size_t)i * kInPad + q] = __float2bfloat16(q < kIn ? x[(size_t)i * kIn + q] : 0.f);
    SCUDA(s, cudaMemcpy(s->d_h[0], xb.data(), 2 * xb.size(), cudaMemcpyHostToDevice), "x H2D");
    SCUDA(s, cudaMemcpy(s->d_y, y, 4 * (size_t)n, cudaMemcpyHostToDevice), "y H2D");
    if ((r = forward(s, n))) return r;
    if ((r = backward(s, n, true))) return r;
    if (grads) SCUDA(s, cudaMemcpyAsync(grads, s->d_g, 4 * s->n_params, cudaMemcpyDeviceToHost, s->stream), "grads D2H");
    double l = 0;
    SCUDA(s, cudaMemcpyAsync(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s->stream), "loss D2H");
    SCUDA(s, cudaStreamSynchronize(s->stream), "grads");
    if (loss) *loss = l;
    return gemm_status(s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// training, pricing, checkpoints
// ---------------------------------------------------------------------------
namespace {

struct DevBatch {  // device copy of host option records
    double *strike = nullptr, *bm = nullptr, *om = nullptr, *a = nullptr, *sg = nullptr;
    uint16_t *tu = nullptr, *ts = nullptr;
    int8_t *ty = nullptr;
    int64_t cap = 0;
};

void free_batch(DevBatch &b)
{
    cudaFree(b.strike); cudaFree(b.bm); cudaFree(b.om); cudaFree(b.a); cudaFree(b.sg);
    cudaFree(b.tu); cudaFree(b.ts); cudaFree(b.ty);
    b = DevBatch();
}

bool alloc_batch(DevBatch &b, int64_t n)
{
    free_batch(b);
    bool ok = cudaMalloc(&b.strike, 8 * n) == cudaSuccess && cudaMalloc(&b.bm, 8 * n) == cudaSuccess &&
              cudaMalloc(&b.om, 8 * n) == cudaSuccess && cudaMalloc(&b.a, 8 * n) == cudaSuccess &&
              cudaMalloc(&b.sg, 8 * n) == cudaSuccess && cudaMalloc(&b.tu, 2 * n) == cudaSuccess &&
              cudaMalloc(&b.ts, 2 * n) == cudaSuccess && cudaMalloc(&b.ty, n) == cudaSuccess;
    b.cap = ok ? n : 0;
    return ok;
}

DevOptions dev_view(const DevBatch &b, int n)
{
    DevOptions o;
    o.n = n; o.strike = b.strike; o.bond_maturity = b.bm; o.option_maturity = b.om; o.term_unit = b.tu;
    o.term_steps = b.ts; o.a = b.a; o.sigma = b.sg; o.type = b.ty;
    return o;
}

hwt_options abi_view(const DevBatch &b, int n)
{
    hwt_options o;
    o.n = n; o.strike = b.strike; o.bond_maturity = b.bm; o.option_maturity = b.om; o.term_unit = b.tu;
    o.term_steps = b.ts; o.a = b.a; o.sigma = b.sg; o.type = b.ty;
    return o;
}

cudaError_t upload_batch(DevBatch &b, const hwt_options *o, cudaStream_t st)
{
    const size_t n = o->n;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b.strike, o->strike, 8 * n, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b.bm, o->bond_maturity, 8 * n, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b.om, o->option_maturity, 8 * n, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b.a, o->a, 8 * n, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b.sg, o->sigma, 8 * n, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b.tu, o->term_unit, 2 * n, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b.ts, o->term_steps, 2 * n, cudaMemcpyHostToDevice, st))) return e;
    return cudaMemcpyAsync(b.ty, o->type, n, cudaMemcpyHostToDevice, st);
}

// Device copy of a host yield curve (double rates, float rates, days).
struct DevCurve {
    double *rate = nullptr;
    float *rate_f = nullptr;
    int32_t *day = nullptr;
    int n = 0;
};

int upload_curve(hwt_surrogate *s, DevCurve &c, const hwt_yield *y)
{
    if (!y || y->n <= 0 || !y->rate || !y->day) return sfail(s, HWT_EINVAL, "yield curve is empty or NULL");
    std::vector<float> rf(y->n);
    for (int i = 0; i < y->n; ++i) rf[i] = (float)y->rate[i];
    SCUDA(s, cudaMalloc(&c.rate, 8 * y->n), "curve alloc");
    SCUDA(s, cudaMalloc(&c.rate_f, 4 * y->n), "curve alloc");
    SCUDA(s, cudaMalloc(&c.day, 4 * y->n), "curve alloc");
    SCUDA(s, cudaMemcpy(c.rate, y->rate, 8 * y->n, cudaMemcpyHostToDevice), "curve H2D");
    SCUDA(s, cudaMemcpy(c.rate_f, rf.data(), 4 * y->n, cudaMemcpyHostToDevice), "curve H2D");
    SCUDA(s, cudaMemcpy(c.day, y->day, 4 * y->n, cudaMemcpyHostToDevice), "curve H2D");
    c.n = y->n;
    return HWT_OK;
}

void free_curve(DevCurve &c)
{
    cudaFree(c.rate); cudaFree(c.rate_f); cudaFree(c.day);
    c = DevCurve();
}

// Forward pass of `rows` samples whose bf16 features start at X (row stride kInPad).
int forward_from(hwt_surrogate *s, const __nv_bfloat16 *X, int rows)
{
    __nv_bfloat16 *keep = s->d_h[0];
    s->d_h[0] = const_cast<__nv_bfloat16 *>(X);
    const int r = forward(s, rows);
    s->d_h[0] = keep;
    return r;
}

struct Scoped {
    std::vector<void *> ptrs;
    ~Scoped()
    {
        for (void *p : ptrs) cudaFree(p);
    }
};

}  // namespace

extern "C" {

int hwt_surrogate_train(hwt_surrogate *s, const hwt_options *samples, const hwt_yield *y,
                        const hwt_train_config *cfg, hwt_train_stats *stats)
{
    if (!s || !samples || !y || !cfg) return HWT_EINVAL;
    const int n = samples->n;
    const int batch = cfg->batch > 0 ? cfg->batch : 8192;
    const int epochs = cfg->epochs > 0 ? cfg->epochs : 1;
    if (n < batch) return sfail(s, HWT_EINVAL, "fewer samples than one batch");
    if (stats) memset(stats, 0, sizeof(*stats));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);

    // 1. labels from the FP64 batched tree
    std::vector<double> price(n);
    hwt_config tc;
    memset(&tc, 0, sizeof(tc));
    tc.mode = HWT_BATCHED_FP64;
    tc.use_graph = 1;
    hwt_stats ts;
    int r = hwt_price_ex(s->ctx, samples, y, &tc, price.data(), &ts);
    if (r) return sfail(s, r, std::string("labelling with the tree failed: ") + hwt_last_error(s->ctx));

    // 2. features and targets on the device
    DevBatch b;
    if (!alloc_batch(b, n)) {
        free_batch(b);
        return sfail(s, HWT_ENOMEM, "sample buffers");
    }
    DevCurve cv;
    Scoped guard;
    if ((r = upload_curve(s, cv, y))) { free_batch(b); return r; }
    __nv_bfloat16 *X = nullptr, *Xs = nullptr;
    double *F = nullptr, *dprice = nullptr, *base = nullptr;
    uint8_t *inbox = nullptr;
    float *yv = nullptr, *ys = nullptr;
    int32_t *perm = nullptr;
    bool ok = cudaMalloc(&X, 2ull * n * kInPad) == cudaSuccess && cudaMalloc(&Xs, 2ull * n * kInPad) == cudaSuccess &&
              cudaMalloc(&F, 8ull * n) == cudaSuccess && cudaMalloc(&dprice, 8ull * n) == cudaSuccess &&
              cudaMalloc(&base, 8ull * n) == cudaSuccess &&
              cudaMalloc(&inbox, n) == cudaSuccess && cudaMalloc(&yv, 4ull * n) == cudaSuccess &&
              cudaMalloc(&ys, 4ull * n) == cudaSuccess && cudaMalloc(&perm, 4ull * n) == cudaSuccess;
    guard.ptrs = {X, Xs, F, dprice, base, inbox, yv, ys, perm};
    if (!ok) { free_batch(b); free_curve(cv); return sfail(s, HWT_ENOMEM, "training buffers"); }
    if (upload_batch(b, samples, s->stream) != cudaSuccess) { free_batch(b); free_curve(cv); return sfail(s, HWT_ECUDA, "samples H2D"); }
    DevYield yc;
    yc.n = cv.n; yc.rate = cv.rate; yc.rate_f = cv.rate_f; yc.day = cv.day;
    features_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(dev_view(b, n), yc, s->box, s->fn, X, F, base, inbox);
    std::vector<double> Fh(n), bh(n);
    std::vector<uint8_t> ib(n);
    cudaMemcpyAsync(Fh.data(), F, 8ull * n, cudaMemcpyDeviceToHost, s->stream);
    cudaMemcpyAsync(bh.data(), base, 8ull * n, cudaMemcpyDeviceToHost, s->stream);
    cudaMemcpyAsync(ib.data(), inbox, n, cudaMemcpyDeviceToHost, s->stream);
    cudaError_t ce = cudaStreamSynchronize(s->stream);
    free_batch(b);
    free_curve(cv);
    if (ce != cudaSuccess) return sfail(s, HWT_ECUDA, std::string("features: ") + cudaGetErrorString(ce));
    double sum = 0, sum2 = 0;
    int64_t nin = 0;
    for (int i = 0; i < n; ++i) {
        if (!ib[i]) continue;
        const double v = (price[i] - bh[i]) / Fh[i];
        sum += v; sum2 += v * v; ++nin;
    }
    if (nin < batch) return sfail(s, HWT_EINVAL, "fewer in-box samples than one batch");
    s->ymean = sum / nin;
    s->ystd = std::max(sqrt(std::max(sum2 / nin - s->ymean * s->ymean, 0.0)), 1e-12);
    SCUDA(s, cudaMemcpyAsync(dprice, price.data(), 8ull * n, cudaMemcpyHostToDevice, s->stream), "prices H2D");
    targets_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(dprice, F, base, n, s->ymean, 1.0 / s->ystd, yv);
    SCUDA(s, cudaGetLastError(), "targets");
    if ((r = ensure_act(s, batch))) return r;

    // 3. Adam with cosine decay over the in-box samples, reshuffled every epoch
    std::vector<int32_t> idx;
    idx.reserve(nin);
    for (int i = 0; i < n; ++i)
        if (ib[i]) idx.push_back(i);
    unsigned long long rs = cfg->seed ? cfg->seed : 7ull;
    auto rnd = [&]() {
        rs += 0x9e3779b97f4a7c15ull;
        unsigned long long z = rs;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    };
    const int steps_per_epoch = (int)(nin / batch);
    const long total = (long)steps_per_epoch * epochs;
    const double lr0 = cfg->lr > 0 ? cfg->lr : 1e-3, lr_min = cfg->lr_min;
    long step = 0;
    double last_epoch_loss = 0;
    // one training step captured as a CUDA graph (about 30 kernels), replayed per step
    StepState *dstate = nullptr;
    SCUDA(s, cudaMalloc(&dstate, sizeof(StepState)), "step state");
    guard.ptrs.push_back(dstate);
    {
        StepState h;
        memset(&h, 0, sizeof(h));
        h.t = s->adam_t;
        SCUDA(s, cudaMemcpy(dstate, &h, sizeof(h), cudaMemcpyHostToDevice), "step state H2D");
    }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    struct GraphGuard {
        cudaGraph_t *g;
        cudaGraphExec_t *x;
        ~GraphGuard()
        {
            if (*x) cudaGraphExecDestroy(*x);
            if (*g) cudaGraphDestroy(*g);
        }
    } gguard{&graph, &gexec};
    SCUDA(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    r = train_step(s, Xs, ys, dstate, batch, lr0, lr_min, (long long)total);
    {
        const cudaError_t ce2 = cudaStreamEndCapture(s->stream, &graph);
        if (r) return r;
        SCUDA(s, ce2, "end capture");
    }
    SCUDA(s, cudaGraphInstantiate(&gexec, graph, 0), "instantiate training graph");
    cudaEventRecord(e0, s->stream);
    for (int ep = 0; ep < epochs; ++ep) {
        for (int64_t i = nin - 1; i > 0; --i) std::swap(idx[i], idx[rnd() % (unsigned long long)(i + 1)]);
        SCUDA(s, cudaMemcpyAsync(perm, idx.data(), 4ull * nin, cudaMemcpyHostToDevice, s->stream), "perm H2D");
        gather_rows_kernel<<<(int)((nin + 255) / 256), 256, 0, s->stream>>>(X, yv, perm, (int)nin, Xs, ys);
        SCUDA(s, cudaStreamSynchronize(s->stream), "shuffle");  // perm host buffer is rewritten next epoch
        SCUDA(s, cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream), "zero loss");
        SCUDA(s, cudaMemsetAsync(&dstate->k, 0, sizeof(int), s->stream), "epoch start");
        for (int k = 0; k < steps_per_epoch; ++k, ++step)
            SCUDA(s, cudaGraphLaunch(gexec, s->stream), "training step");
        double l = 0;
        SCUDA(s, cudaMemcpyAsync(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s->stream), "loss D2H");
        SCUDA(s, cudaStreamSynchronize(s->stream), "epoch");
        last_epoch_loss = l / steps_per_epoch;
    }
    cudaEventRecord(e1, s->stream);
    cudaEventSynchronize(e1);
    {
        StepState h;
        SCUDA(s, cudaMemcpy(&h, dstate, sizeof(h), cudaMemcpyDeviceToHost), "step state D2H");
        s->adam_t = (long)h.t;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->trained = 1;
    if (stats) {
        stats->final_loss = last_epoch_loss;
        stats->train_ms = ms;
        stats->label_ms = ts.total_ms;
        stats->steps = step;
        stats->samples = nin;
        stats->samples_per_s = (double)step * batch / (ms * 1e-3);
        stats->y_mean = s->ymean;
        stats->y_std = s->ystd;
    }
    return gemm_status(s);
}

int hwt_surrogate_price(hwt_surrogate *s, const hwt_options *o, const hwt_yield *y, double judge_fraction,
                        uint64_t seed, int tree_mode, double judge_tolerance, double *out, hwt_surrogate_stats *stats)
{
    if (!s || !o || !y || (o->n > 0 && !out)) return HWT_EINVAL;
    if (!s->trained) return sfail(s, HWT_EINVAL, "the surrogate has not been trained or loaded");
    if (tree_mode < HWT_BATCHED_FP64 || tree_mode > HWT_BATCHED_MIXED) return sfail(s, HWT_EINVAL, "tree mode must be batched");
    const int n = o->n;
    if (stats) memset(stats, 0, sizeof(*stats));
    if (n == 0) return HWT_OK;
    cudaEvent_t ev[4];
    for (auto &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], s->stream);
    DevBatch b, sub;
    DevCurve cv;
    Scoped guard;
    int r;
    if (!alloc_batch(b, n)) { free_batch(b); return sfail(s, HWT_ENOMEM, "option buffers"); }
    if ((r = upload_curve(s, cv, y))) { free_batch(b); return r; }
    __nv_bfloat16 *X = nullptr;
    double *F = nullptr, *dout = nullptr, *tree_out = nullptr, *base = nullptr;
    uint8_t *inbox = nullptr, *kind = nullptr;
    int32_t *list = nullptr, *count = nullptr;
    bool ok = cudaMalloc(&X, 2ull * n * kInPad) == cudaSuccess && cudaMalloc(&F, 8ull * n) == cudaSuccess &&
              cudaMalloc(&base, 8ull * n) == cudaSuccess &&
              cudaMalloc(&dout, 8ull * n) == cudaSuccess && cudaMalloc(&tree_out, 8ull * n) == cudaSuccess &&
              cudaMalloc(&inbox, n) == cudaSuccess && cudaMalloc(&kind, n) == cudaSuccess &&
              cudaMalloc(&list, 4ull * n) == cudaSuccess && cudaMalloc(&count, 4) == cudaSuccess;
    guard.ptrs = {X, F, dout, tree_out, base, inbox, kind, list, count};
    if (!ok) { free_batch(b); free_curve(cv); return sfail(s, HWT_ENOMEM, "pricing buffers"); }
    if (upload_batch(b, o, s->stream) != cudaSuccess) { free_batch(b); free_curve(cv); return sfail(s, HWT_ECUDA, "options H2D"); }
    DevYield yc;
    yc.n = cv.n; yc.rate = cv.rate; yc.rate_f = cv.rate_f; yc.day = cv.day;
    features_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(dev_view(b, n), yc, s->box, s->fn, X, F, base, inbox);
    // network on every option (out-of-box rows are overwritten by the tree)
    if ((r = ensure_act(s, std::min(n, kChunk)))) { free_batch(b); free_curve(cv); return r; }
    for (int c0 = 0; c0 < n; c0 += kChunk) {
        const int rows = std::min(kChunk, n - c0);
        if ((r = forward_from(s, X + (size_t)c0 * kInPad, rows))) { free_batch(b); free_curve(cv); return r; }
        decode_kernel<<<(rows + 255) / 256, 256, 0, s->stream>>>(s->d_z[kLayers - 1], F + c0, base + c0, inbox + c0, rows,
                                                               s->ymean, s->ystd, dout + c0);
    }
    cudaEventRecord(ev[1], s->stream);
    // route out-of-box options and the judge's sample to the tree
    SCUDA(s, cudaMemsetAsync(count, 0, 4, s->stream), "count");
    const double jf = std::min(std::max(judge_fraction, 0.0), 1.0);
    const unsigned long long thresh = jf >= 1.0 ? ~0ull : (unsigned long long)(jf * 18446744073709551616.0);
    route_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(inbox, n, seed, thresh, list, kind, count);
    int m = 0;
    SCUDA(s, cudaMemcpyAsync(&m, count, 4, cudaMemcpyDeviceToHost, s->stream), "count D2H");
    SCUDA(s, cudaStreamSynchronize(s->stream), "route");
    std::vector<int32_t> hl(m);
    std::vector<double> tree_px(m);
    double tree_ms = 0;
    if (m > 0) {
        if (!alloc_batch(sub, m)) { free_batch(b); free_batch(sub); free_curve(cv); return sfail(s, HWT_ENOMEM, "routed buffers"); }
        gather_options_kernel<<<(m + 255) / 256, 256, 0, s->stream>>>(dev_view(b, n), list, count, dev_view(sub, m),
                                                                    sub.strike, sub.bm, sub.om, sub.tu, sub.ts, sub.a,
                                                                    sub.sg, sub.ty);
        SCUDA(s, cudaStreamSynchronize(s->stream), "gather");
        hwt_options so = abi_view(sub, m);
        hwt_config tc;
        memset(&tc, 0, sizeof(tc));
        tc.mode = tree_mode;
        tc.use_graph = 1;
        hwt_stats ts;
        r = hwt_price_device(s->ctx, &so, y, &tc, tree_out, &ts);
        free_batch(sub);
        if (r && r != HWT_EINVAL) { free_batch(b); free_curve(cv); return sfail(s, r, hwt_last_error(s->ctx)); }
        tree_ms = ts.total_ms;
        cudaMemcpy(hl.data(), list, 4ull * m, cudaMemcpyDeviceToHost);
        cudaMemcpy(tree_px.data(), tree_out, 8ull * m, cudaMemcpyDeviceToHost);
    }
    cudaEventRecord(ev[2], s->stream);
    SCUDA(s, cudaMemcpyAsync(out, dout, 8ull * n, cudaMemcpyDeviceToHost, s->stream), "prices D2H");
    std::vector<uint8_t> kh(n);
    SCUDA(s, cudaMemcpyAsync(kh.data(), kind, n, cudaMemcpyDeviceToHost, s->stream), "kind D2H");
    cudaEventRecord(ev[3], s->stream);
    SCUDA(s, cudaStreamSynchronize(s->stream), "price");
    free_batch(b);
    free_curve(cv);
    // judge: |network - tree| on the sample; every tree-priced option returns the tree price
    std::vector<double> errs;
    errs.reserve(m);
    int64_t routed = 0;
    double worst = 0.0;
    for (int j = 0; j < m; ++j) {
        const int i = hl[j];
        if (kh[i] == 2) {
            const double e = fabs(out[i] - tree_px[j]);
            errs.push_back(e);
            worst = std::max(worst, e != e ? INFINITY : e);
        } else {
            ++routed;
        }
        out[i] = tree_px[j];
    }
    int fell_back = 0;
    double fallback_ms = 0;
    if (judge_tolerance > 0 && worst > judge_tolerance) {
        // the network failed its judge on this batch: the tree prices all of it
        hwt_config tc;
        memset(&tc, 0, sizeof(tc));
        tc.mode = tree_mode;
        tc.use_graph = 1;
        hwt_stats ts;
        r = hwt_price_ex(s->ctx, o, y, &tc, out, &ts);
        if (r) return sfail(s, r, hwt_last_error(s->ctx));
        fell_back = 1;
        fallback_ms = ts.total_ms;
    }
    if (stats) {
        float t0 = 0, t1 = 0, t2 = 0;
        cudaEventElapsedTime(&t0, ev[0], ev[1]);
        cudaEventElapsedTime(&t1, ev[0], ev[3]);
        cudaEventElapsedTime(&t2, ev[1], ev[2]);
        stats->n_in_box = n - routed;
        stats->n_routed = routed;
        stats->n_judged = (int64_t)errs.size();
        if (!errs.empty()) {
            std::vector<double> e = errs;
            std::sort(e.begin(), e.end());
            double sm = 0;
            for (double v : e) sm += v;
            stats->judge_max_abs = e.back();
            stats->judge_p99_abs = e[std::min(e.size() - 1, (size_t)floor(0.99 * (e.size() - 1)))];
            stats->judge_mean_abs = sm / e.size();
        }
        stats->fell_back = fell_back;
        stats->network_ms = t0;
        stats->tree_ms = tree_ms + fallback_ms;
        stats->route_ms = t2;
        stats->total_ms = t1 + fallback_ms;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return gemm_status(s);
}

int hwt_surrogate_save(const hwt_surrogate *s, const char *path)
{
    if (!s || !path) return HWT_EINVAL;
    std::vector<float> w(s->n_params), m(s->n_params), v(s->n_params);
    if (cudaMemcpy(w.data(), s->d_w, 4 * s->n_params, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(m.data(), s->d_m, 4 * s->n_params, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(v.data(), s->d_v, 4 * s->n_params, cudaMemcpyDeviceToHost) != cudaSuccess)
        return HWT_ECUDA;
    FILE *f = fopen(path, "wb");
    if (!f) return HWT_EINVAL;
    const uint32_t magic = 0x48575453u, version = 1;
    const uint64_t np = s->n_params;
    const int64_t t = s->adam_t;
    bool ok = fwrite(&magic, 4, 1, f) == 1 && fwrite(&version, 4, 1, f) == 1 && fwrite(&s->box, sizeof(hwt_box), 1, f) == 1 &&
              fwrite(&s->ymean, 8, 1, f) == 1 && fwrite(&s->ystd, 8, 1, f) == 1 && fwrite(&t, 8, 1, f) == 1 &&
              fwrite(&np, 8, 1, f) == 1 && fwrite(w.data(), 4, np, f) == np && fwrite(m.data(), 4, np, f) == np &&
              fwrite(v.data(), 4, np, f) == np;
    fclose(f);
    return ok ? HWT_OK : HWT_EINVAL;
}

int hwt_surrogate_load(hwt_surrogate *s, const char *path)
{
    if (!s || !path) return HWT_EINVAL;
    FILE *f = fopen(path, "rb");
    if (!f) return sfail(s, HWT_EINVAL, "cannot open checkpoint");
    uint32_t magic = 0, version = 0;
    uint64_t np = 0;
    int64_t t = 0;
    hwt_box box;
    double ym = 0, ysd = 1;
    bool ok = fread(&magic, 4, 1, f) == 1 && fread(&version, 4, 1, f) == 1 && magic == 0x48575453u && version == 1 &&
              fread(&box, sizeof(hwt_box), 1, f) == 1 && fread(&ym, 8, 1, f) == 1 && fread(&ysd, 8, 1, f) == 1 &&
              fread(&t, 8, 1, f) == 1 && fread(&np, 8, 1, f) == 1 && np == s->n_params;
    std::vector<float> w(s->n_params), m(s->n_params), v(s->n_params);
    ok = ok && fread(w.data(), 4, np, f) == np && fread(m.data(), 4, np, f) == np && fread(v.data(), 4, np, f) == np;
    fclose(f);
    if (!ok) return sfail(s, HWT_EINVAL, "checkpoint is not a surrogate of this shape");
    s->box = box;
    box_norm(box, s->fn);
    s->ymean = ym;
    s->ystd = ysd;
    s->adam_t = t;
    SCUDA(s, cudaMemcpy(s->d_w, w.data(), 4 * np, cudaMemcpyHostToDevice), "load");
    SCUDA(s, cudaMemcpy(s->d_m, m.data(), 4 * np, cudaMemcpyHostToDevice), "load");
    SCUDA(s, cudaMemcpy(s->d_v, v.data(), 4 * np, cudaMemcpyHostToDevice), "load");
    int r = refresh(s);
    if (r) return r;
    SCUDA(s, cudaStreamSynchronize(s->stream), "load");
    s->trained = 1;
    return HWT_OK;
}

}  // extern "C"
