// Learned surrogate: an 8 -> 256 -> 256 -> 256 -> 256 -> 2 SiLU MLP that maps
// standardised option parameters (7 features and a zero pad) to
//   output 0: (price - Hull-White closed-form price) / forward bond price,
//             standardised (or price / forward bond price with residual = 0), and
//   output 1: an estimate of log |output-0 error| (the error head), which routes
//             the options it does not trust to the tree.
// Layers 0 and 4 run in fp32 on the CUDA cores (layer 0 from fp32 features, layer
// 4 from the fp32 activations of layer 3); layers 1-3 keep fp32 master weights with
// bf16 copies for the tcgen05 tensor cores, bf16 activations and fp32 accumulation.
// Training: Adam with cosine decay on labels priced by the batched FP64 tree, the
// layer-by-layer tensor-core GEMMs of hwt_umma.cuh, one CUDA graph per step; a
// held-out slice of the samples calibrates the error head's routing threshold.
// Inference: the fused network kernel of hwt_mlp.cuh; options outside the training
// box and options the error head flags go to the tree, and a random sample of the
// network's answers is re-priced by the tree as the judge of every batch.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/hwtree.h"
#include "hwt_internal.h"
#include "hwt_mlp.cuh"
#include "hwt_model.cuh"
#include "hwt_umma.cuh"

using namespace hwt;
using namespace hwt::umma;

namespace {

constexpr int kLayers = 5;
constexpr int kIn = 7, kInPad = mlp::kIn, kHidden = mlp::kHidden, kOut = mlp::kOut;
const int kFanIn[kLayers] = {kInPad, kHidden, kHidden, kHidden, kHidden};
const int kFanOut[kLayers] = {kHidden, kHidden, kHidden, kHidden, kOut};
constexpr float kErrEps = 1e-3f;  // floor of the error head's target log(|r| + eps), standardised units
constexpr int kMaxCurve = 4096;

// Tolerances the routing is calibrated at (kCalTol, after the training loop); a call
// with a judge tolerance routes with the largest of them not above kJudgeMargin times
// it, so that answers just under the judge's tolerance on the held-out samples go to
// the tree too and the judge's sample rarely meets one above it.
constexpr int kCalTols = 12;
constexpr double kJudgeMargin = 0.9;

struct FeatureNorm {
    double mean[kIn], inv_std[kIn];
};

// ---------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------

// Hull-White closed-form price of a European option on a zero-coupon bond
// (Jamshidian 1989) with face 100: the control variate of the residual network.
// In terms of the forward bond price fwd = 100 P(T) / P(t) and the moneyness
// mny = X / fwd: bond = fwd P(t), strike = X P(t), log(bond / strike) = -log(mny)
// (no divisions beyond 1 / a: the FP64 pipe is this kernel's bound).
__device__ double hw_closed_form(double t, double T, double X, double a, double sigma, double Pt, double fwd,
                                 double mny, int type)
{
    const double ia = 1.0 / a;
    const double B = -expm1(-a * (T - t)) * ia;
    const double sp = sigma * B * sqrt(-expm1(-2.0 * a * t) * (0.5 * ia));
    if (!(sp > 1e-12)) return Pt * (type == 1 ? fmax(X - fwd, 0.0) : fmax(fwd - X, 0.0));
    const double h = -log(mny) / sp + 0.5 * sp;
    return Pt * (type == 1 ? X * normcdf(-h + sp) - fwd * normcdf(-h) : fwd * normcdf(h) - X * normcdf(h - sp));
}

// fp32 features, forward bond price, control-variate price and in-box flag of each option.
__global__ void features_kernel(DevOptions o, DevYield yc, hwt_box box, FeatureNorm fn, float *X, double *F,
                                double *base, uint8_t *inbox)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= o.n) return;
    const double t = o.option_maturity[i], T = o.bond_maturity[i];
    const int tu = o.term_unit[i];
    const double rtt = yield_at_year<double>(t, tu, yc.rate, yc.day, yc.n) * t;
    const double rTT = yield_at_year<double>(T, tu, yc.rate, yc.day, yc.n) * T;
    const double Pt = exp(-rtt);
    const double fwd = 100.0 * exp(rtt - rTT);  // 100 P(T) / P(t)
    const double mny = o.strike[i] / fwd;
    const double a = o.a[i], sg = o.sigma[i];
    const int steps = o.term_steps[i];
    // moneyness standardised in double (the price moves with it at about the forward
    // price per unit); the other features are exact or smooth, standardised in float
    const float v[kIn] = {(float)t, (float)T, 0.f, (float)a, (float)sg, (float)steps, (float)o.type[i]};
    float x[kInPad];
#pragma unroll
    for (int q = 0; q < kIn; ++q) x[q] = (v[q] - (float)fn.mean[q]) * (float)fn.inv_std[q];
    x[2] = (float)((mny - fn.mean[2]) * fn.inv_std[2]);
    x[kIn] = 0.f;
    float4 *xr = reinterpret_cast<float4 *>(X + (size_t)i * kInPad);
    xr[0] = make_float4(x[0], x[1], x[2], x[3]);
    xr[1] = make_float4(x[4], x[5], x[6], x[7]);
    F[i] = fwd;
    const double span = T - t;
    const bool in = t >= box.t_min && t <= box.t_max && span >= box.span_min && span <= box.span_max &&
                    mny >= box.moneyness_min && mny <= box.moneyness_max && a >= box.a_min && a <= box.a_max &&
                    sg >= box.sigma_min && sg <= box.sigma_max && steps >= box.steps_min && steps <= box.steps_max &&
                    tu == box.term_unit && (o.type[i] == 0 || o.type[i] == 1) && isfinite(mny);
    inbox[i] = in ? 1 : 0;
    // the control variate only where the network answers (the FP64 closed form is
    // most of this kernel's time)
    base[i] = (box.residual && in) ? hw_closed_form(t, T, o.strike[i], a, sg, Pt, fwd, mny, o.type[i]) : 0.0;
}

// Layer 0 of the training path: Z0 = X W0 + b0 (fp32) and layer 1's input H1 =
// [bf16 hi | bf16 lo] of silu(Z0) ([n][512]: hi = bf16(a), lo = bf16(a - hi)), one warp
// per row (eight columns per lane), with the fused kernel's arithmetic.
__global__ void layer0_kernel(const float *X, const float *W0, const float *b0, int n, float *Z0, __nv_bfloat16 *H1)
{
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = gt >> 5, n0 = (gt & 31) * 8;
    if (row >= n) return;
    const float4 *xr = reinterpret_cast<const float4 *>(X + (size_t)row * kInPad);
    const float4 xa = xr[0], xb = xr[1];
    const float x[kInPad] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
    float z[8];
    mlp::layer0_chunk(x, W0, b0, n0, z);
    float4 *zr = reinterpret_cast<float4 *>(Z0 + (size_t)row * kHidden + n0);
    zr[0] = make_float4(z[0], z[1], z[2], z[3]);
    zr[1] = make_float4(z[4], z[5], z[6], z[7]);
    for (int part = 0; part < 2; ++part) {
        uint4 h;
        h.x = mlp::pack_silu2_split(z[0], z[1], part == 1);
        h.y = mlp::pack_silu2_split(z[2], z[3], part == 1);
        h.z = mlp::pack_silu2_split(z[4], z[5], part == 1);
        h.w = mlp::pack_silu2_split(z[6], z[7], part == 1);
        *reinterpret_cast<uint4 *>(H1 + (size_t)row * 2 * kHidden + part * kHidden + n0) = h;
    }
}

// Partial dW0[k][c] = sum over a slice of rows of X[r][k] dZ0[r][c] (fp32), one
// slice of rows per block, into part[block][k][c] (summed in block order afterwards).
__global__ void dw0_kernel(const float *X, const float *dZ, int n, float *part)
{
    const int c = threadIdx.x;  // kHidden threads
    const int per = (n + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    float acc[kInPad] = {};
    for (int r = r0; r < r1; ++r) {
        const float d = dZ[(size_t)r * kHidden + c];
        const float4 *xr = reinterpret_cast<const float4 *>(X + (size_t)r * kInPad);
        const float4 xa = __ldg(xr), xb = __ldg(xr + 1);
        acc[0] = fmaf(xa.x, d, acc[0]); acc[1] = fmaf(xa.y, d, acc[1]);
        acc[2] = fmaf(xa.z, d, acc[2]); acc[3] = fmaf(xa.w, d, acc[3]);
        acc[4] = fmaf(xb.x, d, acc[4]); acc[5] = fmaf(xb.y, d, acc[5]);
        acc[6] = fmaf(xb.z, d, acc[6]); acc[7] = fmaf(xb.w, d, acc[7]);
    }
    for (int k = 0; k < kInPad; ++k) part[((size_t)blockIdx.x * kInPad + k) * kHidden + c] = acc[k];
}

// Layer 4 of the training path in fp32: out[r][c] = b4[c] + sum_k silu(Z3[r][k]) W4[k][c],
// summed as the fused kernel's last epilogue does: one partial per 128 columns (k in
// order), the second added to the first, then the bias.
__global__ void layer4_kernel(const float *Z3, const float *W4, const float *b4, int n, float *out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float *z = Z3 + (size_t)r * kHidden;
    float p0[2] = {0.f, 0.f}, p1[2] = {0.f, 0.f};
    for (int h = 0; h < 2; ++h)
        for (int k = h * mlp::kHalf; k < (h + 1) * mlp::kHalf; ++k) {
            const float a = silu_f(z[k]);
            p0[h] = fmaf(a, __ldg(W4 + 2 * k), p0[h]);
            p1[h] = fmaf(a, __ldg(W4 + 2 * k + 1), p1[h]);
        }
    out[2 * r] = (p0[0] + p0[1]) + __ldg(b4);
    out[2 * r + 1] = (p1[0] + p1[1]) + __ldg(b4 + 1);
}

// Backward through layer 4 (fp32): dZ3[r][k] = (dZ4[r] . W4[k]) silu'(Z3[r][k]), as
// bf16 (operand of the next GEMMs) and fp32 (column sums); one warp per row.
__global__ void layer4_back_kernel(const float *Z3, const float *dZ4, const float *W4, int n, __nv_bfloat16 *dZb,
                                   float *dZf)
{
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = gt >> 5, lane = gt & 31;
    if (r >= n) return;
    const float d0 = dZ4[2 * r], d1 = dZ4[2 * r + 1];
    for (int k = lane; k < kHidden; k += 32) {
        const float g = fmaf(d0, __ldg(W4 + 2 * k), d1 * __ldg(W4 + 2 * k + 1)) * dsilu_f(Z3[(size_t)r * kHidden + k]);
        dZb[(size_t)r * kHidden + k] = __float2bfloat16(g);
        dZf[(size_t)r * kHidden + k] = g;
    }
}

// Partial dW4[k][c] = sum over a slice of rows of silu(Z3[r][k]) dZ4[r][c] (fp32), one
// slice of rows per block, into part[block][k][c].
__global__ void dw4_kernel(const float *Z3, const float *dZ4, int n, float *part)
{
    const int k = threadIdx.x;  // kHidden threads
    const int per = (n + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    float a0 = 0.f, a1 = 0.f;
    for (int r = r0; r < r1; ++r) {
        const float h = silu_f(Z3[(size_t)r * kHidden + k]);
        a0 = fmaf(h, __ldg(dZ4 + 2 * r), a0);
        a1 = fmaf(h, __ldg(dZ4 + 2 * r + 1), a1);
    }
    part[(size_t)blockIdx.x * kHidden * 2 + 2 * k] = a0;
    part[(size_t)blockIdx.x * kHidden * 2 + 2 * k + 1] = a1;
}

// Outputs [n][2] against targets y: r = o0 - y; error-head target g = log(|r| + eps)
// (held constant); loss += 0.5 r^2 / n + 0.5 lam (o1 - g)^2 / n; dZ = its gradient.
__global__ void loss_kernel(const float *out, const float *y, int n, float lam, __nv_bfloat16 *dZ, float *dZf,
                            double *loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (i < n) {
        const float r = out[2 * i] - y[i];
        const float g = logf(fabsf(r) + kErrEps);
        const float r1 = out[2 * i + 1] - g;
        const float d0 = r / (float)n, d1 = lam * r1 / (float)n;
        dZ[2 * i] = __float2bfloat16(d0);
        dZ[2 * i + 1] = __float2bfloat16(d1);
        dZf[2 * i] = d0;
        dZf[2 * i + 1] = d1;
        l = (0.5 * (double)r * r + 0.5 * (double)lam * (double)r1 * r1) / n;
    }
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l);
}

// Partial column sums of d (fp32 [n][ld]) over a slice of rows per block row:
// part[blockIdx.y][c].
__global__ void colsum_kernel(const float *d, int n, int cols, int ld, float *part)
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
    part[(size_t)blockIdx.y * cols + c] = (s0 + s1) + (s2 + s3);
}

// out[e] = sum over slices s of part[s][e], in slice order: the partial sums of the
// gradient kernels above and of the split-K GEMM, added the same way every step
// (the training is reproducible bit for bit).
__global__ void reduce_slices_kernel(const float *part, int slices, int len, float *out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= len) return;
    float acc = 0.f;
    for (int z = 0; z < slices; ++z) acc += part[(size_t)z * len + e];
    out[e] = acc;
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
__global__ void batch_copy_kernel(const float *Xs, const float *ys, const StepState *st, int batch, float *X, float *y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch) return;
    const size_t row = (size_t)st->cur * batch + i;
    const float4 *src = reinterpret_cast<const float4 *>(Xs + row * kInPad);
    float4 *dst = reinterpret_cast<float4 *>(X + (size_t)i * kInPad);
    dst[0] = src[0];
    dst[1] = src[1];
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

// bf16 copies of W[in][out] (layers 1-3): Wt[out][in] (forward operand; with dup,
// [out][2 in] holding it twice, for the hi / lo input pair of layer 1), Wb[in][out]
// (backward-data operand) and the fused kernel's packed blocks.
__global__ void refresh_kernel(const float *W, int in, int out, __nv_bfloat16 *Wt, int dup, __nv_bfloat16 *Wb,
                               __nv_bfloat16 *Wp, float *Wr)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= in * out) return;
    const int k = idx / out, n = idx % out;
    const __nv_bfloat16 v = __float2bfloat16(W[(size_t)k * out + n]);
    const int ldt = dup ? 2 * in : in;
    Wt[(size_t)n * ldt + k] = v;
    if (dup) Wt[(size_t)n * ldt + in + k] = v;
    Wb[(size_t)k * out + n] = v;
    if (Wp) Wp[(size_t)(k / mlp::kKB) * mlp::kWBlockElems + mlp::pack_offset(n, k % mlp::kKB)] = v;
    if (Wr) Wr[(size_t)k * out + n] = __bfloat162float(v);
}

__global__ void gather_rows_kernel(const float *X, const float *y, const int32_t *perm, int n, float *Xo, float *yo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = perm[i];
    const float4 *src = reinterpret_cast<const float4 *>(X + (size_t)s * kInPad);
    float4 *dst = reinterpret_cast<float4 *>(Xo + (size_t)i * kInPad);
    dst[0] = src[0];
    dst[1] = src[1];
    if (y) yo[i] = y[s];
}

__global__ void targets_kernel(const double *price, const double *F, const double *base, int n, double ymean,
                               double yinv, float *y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)(((price[i] - base[i]) / F[i] - ymean) * yinv);
}

// Error of the network's price head against the target, in price units up to the
// constant y_std: |o - y| F (hard-sample mining ranks the training samples by it).
__global__ void sample_err_kernel(const float *out, const float *y, const double *F, int n, float *err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float e = fabsf(out[2 * i] - y[i]) * (float)F[i];
        err[i] = e == e ? e : INFINITY;
    }
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Kinds of an option in a priced batch.
enum Kind : uint8_t {
    KIND_NETWORK = 0,  // answered by the network
    KIND_OUTSIDE = 1,  // outside the training box: tree
    KIND_JUDGED = 2,   // answered by the network and re-priced by the tree (the judge's sample)
    KIND_FLAGGED = 3,  // inside the box, but the error head does not trust the network: tree
};

// Decodes the network's answers and builds the tree's work list: out-of-box and
// flagged options (the tree answers them), and the judge's draw among the network's
// answers.  counts[k] = options of kind k (k = 1..3).
__global__ void decode_route_kernel(const float *out, const double *F, const double *base, const uint8_t *inbox,
                                    const double *strike, int n, double ymean, double ystd, float log_tau_over_ystd,
                                    const double *points, const double *deltas, int n_points, unsigned long long seed,
                                    unsigned long long thresh, double *price, uint8_t *kind, int32_t *list,
                                    int32_t *counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;  // no early return: the whole warp takes part in the append below
    uint8_t k = KIND_NETWORK;
    if (!valid) {
    } else if (!inbox[i]) {
        k = KIND_OUTSIDE;
    } else {
        const float2 o = reinterpret_cast<const float2 *>(out)[i];
        price[i] = base[i] + F[i] * ((double)o.x * ystd + ymean);
        // predicted |price error| = exp(o1) ystd F > tau  <=>  o1 > log(tau / ystd) - log(F)
        bool flag = o.y > log_tau_over_ystd - logf((float)F[i]);
        // a strike within its own distance (moneyness) of a routing point of a
        // single-tree box (a payoff kink of the box's tree or a box edge)
        if (n_points > 0) {
            const double x = strike[i] / F[i];
            for (int j = 0; j < n_points; ++j) flag = flag || fabs(x - points[j]) <= deltas[j];
        }
        if (flag) k = KIND_FLAGGED;
        else if (mix64(seed ^ (unsigned long long)i) < thresh) k = KIND_JUDGED;
    }
    if (valid) kind[i] = k;
    // warp-aggregated append to the tree's list: one atomic per warp, and one per
    // kind present (a batch that routes most options would otherwise serialise on
    // the two counters)
    const bool app = valid && k != KIND_NETWORK;
    const unsigned m = __ballot_sync(0xffffffffu, app);
    if (m != 0u) {
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        int at = 0;
        if (lane == leader) at = atomicAdd(counts, __popc(m));
        at = __shfl_sync(0xffffffffu, at, leader);
        if (app) list[at + __popc(m & ((1u << lane) - 1u))] = i;
        for (int kk = KIND_OUTSIDE; kk <= KIND_FLAGGED; ++kk) {
            const unsigned mk = __ballot_sync(0xffffffffu, app && k == kk);
            if (mk != 0u && lane == __ffs(mk) - 1) atomicAdd(counts + kk, __popc(mk));
        }
    }
}

// Network answers of kind KIND_NETWORK into the list (the whole-batch fallback).
__global__ void network_list_kernel(const uint8_t *kind, int n, int32_t *list, int32_t *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && kind[i] == KIND_NETWORK) list[atomicAdd(count, 1)] = i;
}

__global__ void gather_options_kernel(DevOptions src, const int32_t *list, int m, double *strike, double *bm,
                                      double *om, uint16_t *tu, uint16_t *ts, double *a, double *sg, int8_t *ty)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int i = list[j];
    strike[j] = src.strike[i]; bm[j] = src.bond_maturity[i]; om[j] = src.option_maturity[i];
    tu[j] = src.term_unit[i]; ts[j] = src.term_steps[i]; a[j] = src.a[i]; sg[j] = src.sigma[i]; ty[j] = src.type[i];
}

// Tree prices back into the batch; the judge's |network - tree| (else -1) per entry.
__global__ void scatter_tree_kernel(const int32_t *list, int m, const double *tree, const uint8_t *kind, double *price,
                                    double *err)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int i = list[j];
    const double t = tree[j];
    err[j] = kind[i] == KIND_JUDGED ? fabs(price[i] - t) : -1.0;
    price[i] = t;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

struct DevBatch {  // device copy of option records
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

// Grows (never shrinks) the batch to n options.
bool grow_batch(DevBatch &b, int64_t n)
{
    if (n <= b.cap) return true;
    free_batch(b);
    bool ok = cudaMalloc(&b.strike, 8 * n) == cudaSuccess && cudaMalloc(&b.bm, 8 * n) == cudaSuccess &&
              cudaMalloc(&b.om, 8 * n) == cudaSuccess && cudaMalloc(&b.a, 8 * n) == cudaSuccess &&
              cudaMalloc(&b.sg, 8 * n) == cudaSuccess && cudaMalloc(&b.tu, 2 * n) == cudaSuccess &&
              cudaMalloc(&b.ts, 2 * n) == cudaSuccess && cudaMalloc(&b.ty, n) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_batch(b);
        return false;
    }
    b.cap = n;
    return true;
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

// Grow-only device buffer.
template <typename T>
struct Buf {
    T *p = nullptr;
    size_t cap = 0;
    bool grow(size_t n)
    {
        if (n <= cap) return true;
        cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, sizeof(T) * n) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cap = n;
        return true;
    }
    void release()
    {
        cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

}  // namespace

struct hwt_surrogate {
    hwt_ctx *ctx = nullptr;
    int device = 0, sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[5] = {};
    hwt_box box;
    FeatureNorm fn;
    double ymean = 0.0, ystd = 1.0;
    double route_tau = INFINITY;  // price error the error head's routing keeps network answers under
    // Single-tree boxes: the payoff kinks of the box's tree in moneyness (from the
    // training labels) and the distance from them inside which options go to the tree
    std::vector<double> kinks;
    // per routing point (the kinks, then the box's two moneyness edges): options
    // within this distance of it go to the tree (< 0: none); kink_delta is the largest
    std::vector<double> route_delta;
    double kink_delta = -1.0;     // < 0: no kink routing
    // The same routing calibrated at a ladder of tolerances (kCalTol)
    double cal_tau[kCalTols], cal_delta[kCalTols], cal_answered[kCalTols];
    std::vector<double> cal_deltas[kCalTols];
    int cal_valid = 0;
    Buf<double> dkinks;
    int trained = 0;
    std::string err;
    // parameters (fp32 masters) and Adam state, one flat buffer each
    size_t n_params = 0;
    float *d_w = nullptr, *d_m = nullptr, *d_v = nullptr, *d_g = nullptr;
    size_t w_off[kLayers], b_off[kLayers];
    __nv_bfloat16 *d_wt[kLayers] = {}, *d_wb[kLayers] = {};  // layers 1-4
    __nv_bfloat16 *d_wp = nullptr;                           // packed blocks of layers 1-3
    long adam_t = 0;
    // training activations for one batch
    int act_cap = 0;
    float *d_x = nullptr;                  // [rows][8] fp32 features
    __nv_bfloat16 *d_h[kLayers] = {};      // d_h[l] = bf16 input of layer l (l >= 1)
    float *d_z[kLayers] = {};              // pre-activations (z[4] = outputs [rows][2])
    __nv_bfloat16 *d_dz = nullptr, *d_dz2 = nullptr;
    float *d_dzf = nullptr;
    float *d_part = nullptr;               // per-slice partial gradients, summed in order
    float *d_dz4 = nullptr;                // [rows][2] fp32 output gradients
    double *d_loss = nullptr;
    float *d_y = nullptr;
    int *d_gemm_err = nullptr;  // raised by a kernel whose mbarrier wait ran out
    int stall = 0;              // fault injection for tests (hwt_surrogate_inject_stall)
    // pricing buffers (grow-only)
    DevBatch opts, sub;
    Buf<float> xf, out2;
    Buf<double> F, base, price, tree, errs;
    Buf<uint8_t> inbox, kind;
    Buf<int32_t> list, counts;
    Buf<double> crate;
    Buf<float> crate_f;
    Buf<int32_t> cday;
    std::vector<double> curve_rate;  // the curve now on the device
    std::vector<int32_t> curve_day;
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

// Split-K slices of the weight-gradient GEMMs for a batch of `rows` samples.
int grad_splits(int rows) { return std::max(1, std::min(64, rows / 512)); }

int ensure_act(hwt_surrogate *s, int rows)
{
    if (rows <= s->act_cap) return HWT_OK;
    cudaFree(s->d_x); s->d_x = nullptr;
    for (int l = 0; l < kLayers; ++l) {
        cudaFree(s->d_h[l]); s->d_h[l] = nullptr;
        cudaFree(s->d_z[l]); s->d_z[l] = nullptr;
    }
    cudaFree(s->d_dz); cudaFree(s->d_dz2); cudaFree(s->d_dzf); cudaFree(s->d_y); cudaFree(s->d_dz4);
    cudaFree(s->d_part);
    s->d_dz = s->d_dz2 = nullptr; s->d_dzf = nullptr; s->d_y = nullptr; s->d_dz4 = nullptr; s->d_part = nullptr;
    s->act_cap = 0;
    SCUDA(s, cudaMalloc(&s->d_x, sizeof(float) * (size_t)rows * kInPad), "alloc X");
    for (int l = 1; l < kLayers; ++l)  // H1 holds layer 1's hi / lo input pair
        SCUDA(s, cudaMalloc(&s->d_h[l], sizeof(__nv_bfloat16) * (size_t)rows * kHidden * (l == 1 ? 2 : 1)), "alloc H");
    for (int l = 0; l < kLayers; ++l) SCUDA(s, cudaMalloc(&s->d_z[l], sizeof(float) * (size_t)rows * kFanOut[l]), "alloc Z");
    SCUDA(s, cudaMalloc(&s->d_dz, sizeof(__nv_bfloat16) * (size_t)rows * kHidden), "alloc dZ");
    SCUDA(s, cudaMalloc(&s->d_dz2, sizeof(__nv_bfloat16) * (size_t)rows * kHidden), "alloc dZ");
    SCUDA(s, cudaMalloc(&s->d_dzf, sizeof(float) * (size_t)rows * kHidden), "alloc dZf");
    SCUDA(s, cudaMalloc(&s->d_y, sizeof(float) * (size_t)rows), "alloc y");
    SCUDA(s, cudaMalloc(&s->d_dz4, sizeof(float) * (size_t)rows * kOut), "alloc dZ4");
    // partials: the weight-gradient GEMM's split-K slices (at most 64 of [256][256]) or
    // 256 row slices of the fp32 kernels (at most [8][256] each)
    const size_t part = std::max((size_t)grad_splits(rows) * kHidden * kHidden, (size_t)256 * kInPad * kHidden);
    SCUDA(s, cudaMalloc(&s->d_part, sizeof(float) * part), "alloc partials");
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

// Dynamic shared memory above 48 KB for every kernel that needs it, once at set-up
// (outside any stream capture).
cudaError_t kernel_attributes()
{
    cudaError_t e = cudaSuccess;
    auto set = [&](auto kern, int bytes) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    };
    set(umma_gemm_kernel<false, false, 16>, smem_bytes(16));
    set(umma_gemm_kernel<false, false, 64>, smem_bytes(64));
    set(umma_gemm_kernel<false, false, 128>, smem_bytes(128));
    set(umma_gemm_kernel<true, true, 16>, smem_bytes(16));
    set(umma_gemm_kernel<true, true, 64>, smem_bytes(64));
    set(umma_gemm_kernel<true, true, 128>, smem_bytes(128));
    set(mlp::mlp_forward_kernel, mlp::kSmemBytes);
    return e;
}

// Tile width: the output width rounded up to 16 (one tile for the 2-wide output
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

// HWT_ETIMEOUT (and the flag cleared) if a tensor-core kernel gave up waiting since
// the last check.
int gemm_status(hwt_surrogate *s)
{
    int flag = 0;
    SCUDA(s, cudaMemcpy(&flag, s->d_gemm_err, sizeof(int), cudaMemcpyDeviceToHost), "tensor-core status");
    if (flag == 0) return HWT_OK;
    SCUDA(s, cudaMemset(s->d_gemm_err, 0, sizeof(int)), "tensor-core status");
    return sfail(s, HWT_ETIMEOUT, "tensor-core kernel: an mbarrier wait ran out");
}

// Layer-by-layer forward (the training path) for `rows` samples in d_x; outputs in
// d_z[4] ([rows][2]).
int forward_layers(hwt_surrogate *s, int rows)
{
    layer0_kernel<<<(rows * 32 + 255) / 256, 256, 0, s->stream>>>(s->d_x, s->d_w + s->w_off[0], s->d_w + s->b_off[0],
                                                                  rows, s->d_z[0], s->d_h[1]);
    SCUDA(s, cudaGetLastError(), "layer 0");
    for (int l = 1; l < kLayers - 1; ++l) {
        const bool to_last = l == kLayers - 2;  // layer 4 reads fp32 Z3, not bf16 activations
        // layer 1: K = 512 over [hi | lo] inputs and [W1 | W1], the two products accumulated
        const int K = l == 1 ? 2 * kFanIn[l] : kFanIn[l];
        GemmArgs g = gargs(s, s->d_h[l], s->d_wt[l], rows, kFanOut[l], K, K, K, EPI_BIAS_SILU);
        g.bias = s->d_w + s->b_off[l];
        g.Cf = s->d_z[l];
        g.ldc = kFanOut[l];
        g.Cb = to_last ? nullptr : s->d_h[l + 1];
        g.ldcb = kFanOut[l];
        if (to_last) g.epi = EPI_BIAS;
        SCUDA(s, (gemm<false, false>(g, 1, s->stream)), "forward gemm");
    }
    layer4_kernel<<<(rows + 127) / 128, 128, 0, s->stream>>>(s->d_z[kLayers - 2], s->d_w + s->w_off[kLayers - 1],
                                                             s->d_w + s->b_off[kLayers - 1], rows, s->d_z[kLayers - 1]);
    SCUDA(s, cudaGetLastError(), "layer 4");
    return HWT_OK;
}

// Fused forward of `rows` samples (fp32 features X) into out [rows][2].
int forward_fused(hwt_surrogate *s, const float *X, int rows, float *out)
{
    if (rows <= 0) return HWT_OK;
    mlp::MlpArgs a;
    a.X = X;
    a.n = rows;
    a.W0 = s->d_w + s->w_off[0];
    a.b0 = s->d_w + s->b_off[0];
    a.Wp = s->d_wp;
    a.b1 = s->d_w + s->b_off[1];
    a.b2 = s->d_w + s->b_off[2];
    a.b3 = s->d_w + s->b_off[3];
    a.W4 = s->d_w + s->w_off[kLayers - 1];
    a.b4 = s->d_w + s->b_off[4];
    a.out = out;
    a.err = s->d_gemm_err;
    a.test_stall = s->stall;
    const int tiles = (rows + mlp::kRows - 1) / mlp::kRows;
    const int grid = std::min(tiles, mlp::kCtasPerSm * s->sms);
    mlp::mlp_forward_kernel<<<grid, mlp::kThreads, mlp::kSmemBytes, s->stream>>>(a);
    SCUDA(s, cudaGetLastError(), "fused network kernel");
    return HWT_OK;
}

// Loss and gradients (into d_g) for `rows` samples in d_x with targets d_y.
int backward(hwt_surrogate *s, int rows, float lam, bool zero_loss)
{
    SCUDA(s, cudaMemsetAsync(s->d_g, 0, sizeof(float) * s->n_params, s->stream), "zero grads");
    if (zero_loss) SCUDA(s, cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream), "zero loss");
    loss_kernel<<<(rows + 255) / 256, 256, 0, s->stream>>>(s->d_z[kLayers - 1], s->d_y, rows, lam, s->d_dz, s->d_dz4,
                                                           s->d_loss);
    SCUDA(s, cudaGetLastError(), "loss kernel");
    __nv_bfloat16 *dz = s->d_dz, *dz_next = s->d_dz2;
    const int splits = grad_splits(rows);
    int kc = (rows + splits - 1) / splits;
    kc = (kc + BK - 1) / BK * BK;
    const int nslice = std::max(1, std::min(256, rows / 32));  // row slices of the fp32 kernels
    auto reduce = [&](int slices, int len, float *out) {
        reduce_slices_kernel<<<(len + 255) / 256, 256, 0, s->stream>>>(s->d_part, slices, len, out);
        return cudaGetLastError();
    };
    // layer 4 in fp32: dW4 = silu(Z3)^T dZ4, db4 = column sums of dZ4, dZ3 = (dZ4 W4^T) silu'(Z3)
    {
        const float *dz4 = s->d_dz4;
        dw4_kernel<<<nslice, kHidden, 0, s->stream>>>(s->d_z[kLayers - 2], dz4, rows, s->d_part);
        SCUDA(s, cudaGetLastError(), "dW4 kernel");
        SCUDA(s, reduce(nslice, kHidden * kOut, s->d_g + s->w_off[kLayers - 1]), "dW4 sum");
        dim3 cg(1, nslice);
        colsum_kernel<<<cg, 256, 0, s->stream>>>(dz4, rows, kOut, kOut, s->d_part);
        SCUDA(s, cudaGetLastError(), "db4 kernel");
        SCUDA(s, reduce(nslice, kOut, s->d_g + s->b_off[kLayers - 1]), "db4 sum");
        layer4_back_kernel<<<(rows * 32 + 255) / 256, 256, 0, s->stream>>>(s->d_z[kLayers - 2], dz4,
                                                                           s->d_w + s->w_off[kLayers - 1], rows, dz,
                                                                           s->d_dzf);
        SCUDA(s, cudaGetLastError(), "layer 4 backward");
    }
    for (int l = kLayers - 2; l >= 1; --l) {
        const int in = kFanIn[l], out = kFanOut[l];
        // dW_l[in][out] = H_l^T dZ_l   (split-K over the batch; layer 1 from the hi parts)
        GemmArgs gw = gargs(s, s->d_h[l], dz, in, out, rows, l == 1 ? 2 * in : in, out, EPI_SLICE);
        gw.Cf = s->d_part;
        gw.ldc = out;
        gw.k_chunk = kc;
        const int zs = (rows + kc - 1) / kc;  // every slice holds at least one K block
        SCUDA(s, (gemm<true, true>(gw, zs, s->stream)), "dW gemm");
        SCUDA(s, reduce(zs, in * out, s->d_g + s->w_off[l]), "dW sum");
        // db_l = column sums of dZ_l (fp32 copy in d_dzf)
        dim3 cg((out + 255) / 256, nslice);
        colsum_kernel<<<cg, 256, 0, s->stream>>>(s->d_dzf, rows, out, out, s->d_part);
        SCUDA(s, cudaGetLastError(), "db kernel");
        SCUDA(s, reduce(nslice, out, s->d_g + s->b_off[l]), "db sum");
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
    // layer 0 in fp32: dW0 = X^T dZ0, db0 = column sums of dZ0
    dw0_kernel<<<nslice, kHidden, 0, s->stream>>>(s->d_x, s->d_dzf, rows, s->d_part);
    SCUDA(s, cudaGetLastError(), "dW0 kernel");
    SCUDA(s, reduce(nslice, kInPad * kHidden, s->d_g + s->w_off[0]), "dW0 sum");
    dim3 cg(1, nslice);
    colsum_kernel<<<cg, 256, 0, s->stream>>>(s->d_dzf, rows, kHidden, kHidden, s->d_part);
    SCUDA(s, cudaGetLastError(), "db0 kernel");
    SCUDA(s, reduce(nslice, kHidden, s->d_g + s->b_off[0]), "db0 sum");
    return HWT_OK;
}

int refresh(hwt_surrogate *s)
{
    for (int l = 1; l < kLayers - 1; ++l) {  // layer 4 stays fp32
        const int tot = kFanIn[l] * kFanOut[l];
        __nv_bfloat16 *wp = s->d_wp + (size_t)(l - 1) * mlp::kBlocksPerLayer * mlp::kWBlockElems;
        refresh_kernel<<<(tot + 255) / 256, 256, 0, s->stream>>>(s->d_w + s->w_off[l], kFanIn[l], kFanOut[l], s->d_wt[l],
                                                               l == 1 ? 1 : 0, s->d_wb[l], wp, nullptr);
        SCUDA(s, cudaGetLastError(), "refresh kernel");
    }
    return HWT_OK;
}

// One training step on the batch the step state names, everything from device
// state: the body of the captured training graph.
int train_step(hwt_surrogate *s, const float *Xs, const float *ys, StepState *st, int batch, double lr0,
               double lr_min, long long total, float lam)
{
    step_begin_kernel<<<1, 1, 0, s->stream>>>(st, lr0, lr_min, total);
    SCUDA(s, cudaGetLastError(), "step kernel");
    batch_copy_kernel<<<(batch + 255) / 256, 256, 0, s->stream>>>(Xs, ys, st, batch, s->d_x, s->d_y);
    SCUDA(s, cudaGetLastError(), "batch kernel");
    int r = forward_layers(s, batch);
    if (!r) r = backward(s, batch, lam, false);
    if (r) return r;
    AdamArgs a;
    a.w = s->d_w; a.m = s->d_m; a.v = s->d_v; a.g = s->d_g; a.n = (int)s->n_params;
    a.lr = 0.f; a.b1 = 0.9f; a.b2 = 0.999f; a.eps = 1e-8f; a.c1 = 1.f; a.c2 = 1.f;
    adam_kernel<<<((int)s->n_params + 255) / 256, 256, 0, s->stream>>>(a, st);
    SCUDA(s, cudaGetLastError(), "adam kernel");
    return refresh(s);
}

// Mean and 1 / std of a uniform variable on [lo, hi]; a dimension the box pins to
// one value gets inv_std 0 (its feature is 0 inside the box).
void box_norm(const hwt_box &b, FeatureNorm &fn)
{
    const double lo[kIn] = {b.t_min, b.t_min + b.span_min, b.moneyness_min, b.a_min, b.sigma_min, (double)b.steps_min, 0.0};
    const double hi[kIn] = {b.t_max, b.t_max + b.span_max, b.moneyness_max, b.a_max, b.sigma_max, (double)b.steps_max, 1.0};
    for (int q = 0; q < kIn; ++q) {
        const double w = hi[q] - lo[q];
        fn.mean[q] = 0.5 * (lo[q] + hi[q]);
        fn.inv_std[q] = w > 1e-12 ? sqrt(12.0) / w : 0.0;
    }
}

int upload_curve(hwt_surrogate *s, const hwt_yield *y, DevYield &yc)
{
    if (!y || y->n <= 0 || !y->rate || !y->day) return sfail(s, HWT_EINVAL, "yield curve is empty or NULL");
    if (y->n > kMaxCurve) return sfail(s, HWT_EINVAL, "yield curve has more than 4096 nodes");
    for (int i = 0; i < y->n; ++i)
        if (!std::isfinite(y->rate[i])) return sfail(s, HWT_EINVAL, "yield curve rate is not finite");
    if (!s->crate.grow(kMaxCurve) || !s->crate_f.grow(kMaxCurve) || !s->cday.grow(kMaxCurve))
        return sfail(s, HWT_ENOMEM, "curve buffers");
    const bool same = (int)s->curve_rate.size() == y->n && memcmp(s->curve_rate.data(), y->rate, 8 * y->n) == 0 &&
                      memcmp(s->curve_day.data(), y->day, 4 * y->n) == 0;
    if (!same) {
        std::vector<float> rf(y->n);
        for (int i = 0; i < y->n; ++i) rf[i] = (float)y->rate[i];
        SCUDA(s, cudaStreamSynchronize(s->stream), "curve");  // no kernel may still read the old curve
        SCUDA(s, cudaMemcpy(s->crate.p, y->rate, 8 * y->n, cudaMemcpyHostToDevice), "curve H2D");
        SCUDA(s, cudaMemcpy(s->crate_f.p, rf.data(), 4 * y->n, cudaMemcpyHostToDevice), "curve H2D");
        SCUDA(s, cudaMemcpy(s->cday.p, y->day, 4 * y->n, cudaMemcpyHostToDevice), "curve H2D");
        s->curve_rate.assign(y->rate, y->rate + y->n);
        s->curve_day.assign(y->day, y->day + y->n);
    }
    yc.n = y->n;
    yc.rate = s->crate.p;
    yc.rate_f = s->crate_f.p;
    yc.day = s->cday.p;
    return HWT_OK;
}

// Standardised host features x [n][7] into the training input buffer (fp32, padded).
int upload_features(hwt_surrogate *s, const float *x, int n)
{
    int r = ensure_act(s, n);
    if (r) return r;
    std::vector<float> xp((size_t)n * kInPad, 0.f);
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < kIn; ++q) xp[(size_t)i * kInPad + q] = x[(size_t)i * kIn + q];
    SCUDA(s, cudaMemcpy(s->d_x, xp.data(), 4 * xp.size(), cudaMemcpyHostToDevice), "x H2D");
    return HWT_OK;
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
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    bool ok = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess;
    for (auto &e : s->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    size_t off = 0;
    for (int l = 0; l < kLayers; ++l) {  // every block starts on a 16-byte boundary
        s->w_off[l] = off; off += ((size_t)kFanIn[l] * kFanOut[l] + 3) / 4 * 4;
        s->b_off[l] = off; off += ((size_t)kFanOut[l] + 3) / 4 * 4;
    }
    s->n_params = off;
    ok = ok && cudaMalloc(&s->d_w, 4 * off) == cudaSuccess && cudaMalloc(&s->d_m, 4 * off) == cudaSuccess &&
         cudaMalloc(&s->d_v, 4 * off) == cudaSuccess && cudaMalloc(&s->d_g, 4 * off) == cudaSuccess &&
         cudaMalloc(&s->d_loss, sizeof(double)) == cudaSuccess &&
         cudaMalloc(&s->d_gemm_err, sizeof(int)) == cudaSuccess && cudaMemset(s->d_gemm_err, 0, sizeof(int)) == cudaSuccess &&
         cudaMalloc(&s->d_wp, 2ull * mlp::kBlocks * mlp::kWBlockElems) == cudaSuccess;
    for (int l = 1; l < kLayers - 1 && ok; ++l) {  // layer 1's forward operand twice (hi / lo inputs)
        ok = cudaMalloc(&s->d_wt[l], 2 * (size_t)kFanIn[l] * kFanOut[l] * (l == 1 ? 2 : 1)) == cudaSuccess &&
             cudaMalloc(&s->d_wb[l], 2 * (size_t)kFanIn[l] * kFanOut[l]) == cudaSuccess;
    }
    if (ok) {
        // He initialisation from a seeded host generator (splitmix64 + Box-Muller);
        // the zero pad row of layer 0 and the padding words stay zero
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
        ok = ok && kernel_attributes() == cudaSuccess;
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
    cudaFree(s->d_wp); cudaFree(s->d_x);
    for (int l = 0; l < kLayers; ++l) { cudaFree(s->d_wt[l]); cudaFree(s->d_wb[l]); cudaFree(s->d_z[l]); cudaFree(s->d_h[l]); }
    cudaFree(s->d_part);
    cudaFree(s->d_dz); cudaFree(s->d_dz2); cudaFree(s->d_dzf); cudaFree(s->d_y); cudaFree(s->d_dz4);
    free_batch(s->opts);
    free_batch(s->sub);
    s->xf.release(); s->out2.release(); s->F.release(); s->base.release(); s->price.release(); s->tree.release();
    s->errs.release(); s->inbox.release(); s->kind.release(); s->list.release(); s->counts.release();
    s->crate.release(); s->crate_f.release(); s->cday.release(); s->dkinks.release();
    for (auto &e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

const char *hwt_surrogate_last_error(const hwt_surrogate *s) { return s ? s->err.c_str() : "no surrogate"; }

int hwt_surrogate_inject_stall(hwt_surrogate *s, int mode)
{
    if (!s || mode < 0 || mode > 2) return HWT_EINVAL;
    s->stall = mode;
    return HWT_OK;
}

int64_t hwt_surrogate_param_count(const hwt_surrogate *s)
{
    if (!s) return 0;
    int64_t n = 0;
    for (int l = 0; l < kLayers; ++l) n += (int64_t)kFanIn[l] * kFanOut[l] + kFanOut[l];
    return n;
}

// Parameters in the flat layout [W_0, b_0, ..., W_4, b_4] (no padding words).
int hwt_surrogate_params(hwt_surrogate *s, float *buf, int64_t n, int set)
{
    if (!s || !buf || n != hwt_surrogate_param_count(s)) return HWT_EINVAL;
    std::vector<float> w(s->n_params, 0.f);
    if (!set) SCUDA(s, cudaMemcpy(w.data(), s->d_w, 4 * s->n_params, cudaMemcpyDeviceToHost), "get params");
    size_t q = 0;
    for (int l = 0; l < kLayers; ++l) {
        const size_t nw = (size_t)kFanIn[l] * kFanOut[l], nb = kFanOut[l];
        for (size_t i = 0; i < nw + nb; ++i, ++q) {
            float &dst = w[(i < nw ? s->w_off[l] + i : s->b_off[l] + (i - nw))];
            if (set) dst = buf[q];
            else buf[q] = dst;
        }
    }
    if (set) {
        SCUDA(s, cudaMemcpy(s->d_w, w.data(), 4 * s->n_params, cudaMemcpyHostToDevice), "set params");
        int r = refresh(s);
        if (r) return r;
        SCUDA(s, cudaStreamSynchronize(s->stream), "refresh");
    }
    return HWT_OK;
}

int hwt_surrogate_forward_ex(hwt_surrogate *s, const float *x, int n, float *out, int path)
{
    if (!s || !x || !out || n <= 0 || (path != 0 && path != 1)) return HWT_EINVAL;
    int r = upload_features(s, x, n);
    if (r) return r;
    if (path == 0) {
        if (!s->out2.grow((size_t)n * kOut)) return sfail(s, HWT_ENOMEM, "output buffer");
        if ((r = forward_fused(s, s->d_x, n, s->out2.p))) return r;
        SCUDA(s, cudaMemcpyAsync(out, s->out2.p, 4ull * n * kOut, cudaMemcpyDeviceToHost, s->stream), "out D2H");
    } else {
        if ((r = forward_layers(s, n))) return r;
        SCUDA(s, cudaMemcpyAsync(out, s->d_z[kLayers - 1], 4ull * n * kOut, cudaMemcpyDeviceToHost, s->stream), "out D2H");
    }
    SCUDA(s, cudaStreamSynchronize(s->stream), "forward");
    return gemm_status(s);
}

int hwt_surrogate_forward(hwt_surrogate *s, const float *x, int n, float *out)
{
    return hwt_surrogate_forward_ex(s, x, n, out, 0);
}

int hwt_surrogate_forward_device(hwt_surrogate *s, const float *dev_x, int n, float *dev_out, double *kernel_ms)
{
    if (!s || !dev_x || !dev_out || n <= 0) return HWT_EINVAL;
    if ((reinterpret_cast<uintptr_t>(dev_x) & 15) != 0 || (reinterpret_cast<uintptr_t>(dev_out) & 7) != 0)
        return sfail(s, HWT_EINVAL, "feature rows must start on 16-byte boundaries, outputs on 8");
    SCUDA(s, cudaEventRecord(s->ev[0], s->stream), "event");
    int r = forward_fused(s, dev_x, n, dev_out);
    if (r) return r;
    SCUDA(s, cudaEventRecord(s->ev[1], s->stream), "event");
    SCUDA(s, cudaEventSynchronize(s->ev[1]), "forward");
    if (kernel_ms) {
        float ms = 0;
        cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]);
        *kernel_ms = ms;
    }
    return gemm_status(s);
}

int hwt_surrogate_loss_grads(hwt_surrogate *s, const float *x, const float *y, int n, double err_weight, double *loss,
                             float *grads)
{
    if (!s || !x || !y || n <= 0) return HWT_EINVAL;
    int r = upload_features(s, x, n);
    if (r) return r;
    SCUDA(s, cudaMemcpy(s->d_y, y, 4 * (size_t)n, cudaMemcpyHostToDevice), "y H2D");
    if ((r = forward_layers(s, n))) return r;
    if ((r = backward(s, n, (float)err_weight, true))) return r;
    std::vector<float> g(s->n_params);
    double l = 0;
    SCUDA(s, cudaMemcpyAsync(g.data(), s->d_g, 4 * s->n_params, cudaMemcpyDeviceToHost, s->stream), "grads D2H");
    SCUDA(s, cudaMemcpyAsync(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s->stream), "loss D2H");
    SCUDA(s, cudaStreamSynchronize(s->stream), "grads");
    if (loss) *loss = l;
    if (grads) {
        size_t q = 0;
        for (int lyr = 0; lyr < kLayers; ++lyr) {
            const size_t nw = (size_t)kFanIn[lyr] * kFanOut[lyr], nb = kFanOut[lyr];
            for (size_t i = 0; i < nw; ++i) grads[q++] = g[s->w_off[lyr] + i];
            for (size_t i = 0; i < nb; ++i) grads[q++] = g[s->b_off[lyr] + i];
        }
    }
    return gemm_status(s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// training, pricing, checkpoints
// ---------------------------------------------------------------------------
namespace {

struct Scoped {
    std::vector<void *> ptrs;
    ~Scoped()
    {
        for (void *p : ptrs) cudaFree(p);
    }
};

// Features, forward prices and closed-form bases of the host options into the
// surrogate's pricing buffers (options copied to s->opts).
int features_for(hwt_surrogate *s, const hwt_options *o, const hwt_yield *y, cudaEvent_t after_copy = nullptr)
{
    const int n = o->n;
    DevYield yc;
    int r = upload_curve(s, y, yc);
    if (r) return r;
    if (!grow_batch(s->opts, n) || !s->xf.grow((size_t)n * kInPad) || !s->F.grow(n) || !s->base.grow(n) ||
        !s->inbox.grow(n))
        return sfail(s, HWT_ENOMEM, "pricing buffers");
    SCUDA(s, upload_batch(s->opts, o, s->stream), "options H2D");
    if (after_copy) SCUDA(s, cudaEventRecord(after_copy, s->stream), "event");
    features_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(dev_view(s->opts, n), yc, s->box, s->fn, s->xf.p, s->F.p,
                                                           s->base.p, s->inbox.p);
    SCUDA(s, cudaGetLastError(), "features kernel");
    return HWT_OK;
}

// Router threshold from held-out samples: the largest predicted error tau such that
// every held-out sample the network would answer (predicted <= tau) has a true
// error <= tol.  pred and err in price units.
double calibrate_tau(const std::vector<double> &pred, const std::vector<double> &err, double tol, double *answered,
                     double *max_answered, double *p99_answered)
{
    const size_t n = pred.size();
    std::vector<size_t> idx(n);
    for (size_t i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return pred[a] < pred[b]; });
    size_t k = 0;  // answered: idx[0..k)
    double run = 0.0;
    while (k < n) {
        const double e = err[idx[k]];
        if (!(e <= tol)) break;
        run = std::max(run, e);
        ++k;
    }
    // ties: a threshold equal to the next prediction would also admit it
    while (k > 0 && k < n && pred[idx[k]] == pred[idx[k - 1]]) --k;
    double tau = k == 0 ? -1.0 : pred[idx[k - 1]];
    std::vector<double> ea;
    ea.reserve(k);
    run = 0.0;
    for (size_t i = 0; i < k; ++i) {
        ea.push_back(err[idx[i]]);
        run = std::max(run, err[idx[i]]);
    }
    *answered = n ? (double)k / n : 0.0;
    *max_answered = run;
    if (!ea.empty()) {
        std::sort(ea.begin(), ea.end());
        *p99_answered = ea[std::min(ea.size() - 1, (size_t)floor(0.99 * (ea.size() - 1)))];
    } else {
        *p99_answered = 0.0;
    }
    return tau;
}

constexpr int kMaxKinks = 256;
constexpr double kKinkBand = 0.005;  // moneyness: ~0.44 strike units around a kink of the book's tree
const double kCalTol[kCalTols] = {2.5e-5, 5e-5, 9e-5, 1e-4, 1.8e-4, 2e-4, 4.5e-4, 5e-4, 9e-4, 1e-3, 1.8e-3, 2e-3};

// A box that pins every tree parameter (maturities, a, sigma, steps): all its
// options share one tree, and only strike and type vary.
bool single_tree_box(const hwt_box &b)
{
    return b.t_min == b.t_max && b.span_min == b.span_max && b.a_min == b.a_max && b.sigma_min == b.sigma_max &&
           b.steps_min == b.steps_max;
}

// Payoff kinks of one tree as moneyness values x = strike / F, from labelled
// samples (x, price) of one option type.  The tree's price is piecewise linear in
// the strike: the root value is a fixed linear combination of the maturity row's
// payoffs max(+-(bond value - strike), 0), so its slope changes exactly where the
// strike crosses a maturity-node bond value.  A slope change above `thr` (price per
// unit of moneyness) between consecutive samples at least 1e-8 apart marks one.
void detect_kinks(std::vector<std::pair<double, double>> &pts, double thr, std::vector<double> &out)
{
    std::sort(pts.begin(), pts.end());
    std::vector<std::pair<double, double>> q;
    q.reserve(pts.size());
    for (const auto &pt : pts)
        if (q.empty() || pt.first - q.back().first > 1e-8) q.push_back(pt);
    for (size_t i = 2; i < q.size(); ++i) {
        const double s0 = (q[i - 1].second - q[i - 2].second) / (q[i - 1].first - q[i - 2].first);
        const double s1 = (q[i].second - q[i - 1].second) / (q[i].first - q[i - 1].first);
        if (fabs(s1 - s0) > thr) out.push_back(q[i - 1].first);
    }
}

// Sorted kinks, detections closer than 1e-4 in moneyness merged to their midpoint
// (one kink is detected on both sides of the sample gap it falls in, and once per
// option type; neighbouring kinks of a tree are about B(T - t) dr apart in log
// moneyness, 2e-2 for the book's tree).
std::vector<double> merge_kinks(std::vector<double> k)
{
    std::sort(k.begin(), k.end());
    std::vector<double> m;
    size_t i = 0;
    while (i < k.size()) {
        size_t j = i;
        while (j + 1 < k.size() && k[j + 1] - k[i] <= 1e-4) ++j;
        m.push_back(0.5 * (k[i] + k[j]));
        i = j + 1;
    }
    return m;
}

double kink_distance(const std::vector<double> &kinks, double x)
{
    double d = INFINITY;
    for (double k : kinks) d = std::min(d, fabs(x - k));
    return d;
}

// Index of the point nearest to x (points non-empty).
int nearest_point(const std::vector<double> &pts, double x)
{
    int b = 0;
    for (int k = 1; k < (int)pts.size(); ++k)
        if (fabs(x - pts[k]) < fabs(x - pts[b])) b = k;
    return b;
}

// x within its own routing distance of some point (the decode kernel's test).
bool routed_near(const std::vector<double> &pts, const std::vector<double> &delta, double x)
{
    for (size_t k = 0; k < delta.size() && k < pts.size(); ++k)
        if (fabs(x - pts[k]) <= delta[k]) return true;
    return false;
}

// Distances per routing point: each sample above tol widens the distance of the
// point nearest to it until it is reached (-1: no such sample).
void route_distances(const std::vector<double> &pts, const double *x, const double *err, int64_t n, double tol,
                     std::vector<double> &delta)
{
    delta.assign(pts.size(), -1.0);
    if (pts.empty()) return;
    for (int64_t j = 0; j < n; ++j)
        if (!(err[j] <= tol)) {
            const int k = nearest_point(pts, x[j]);
            delta[k] = std::max(delta[k], fabs(x[j] - pts[k]));
        }
}

// Kinks of one tree from (moneyness, price, type) samples: detect_kinks per type,
// then merge_kinks.
std::vector<double> find_kinks(const double *x, const double *price, const int8_t *type, int64_t n)
{
    std::vector<double> k;
    for (int t = 0; t <= 1; ++t) {
        std::vector<std::pair<double, double>> pts;
        for (int64_t i = 0; i < n; ++i)
            if (type[i] == t) pts.emplace_back(x[i], price[i]);
        detect_kinks(pts, 1e-3, k);
    }
    return merge_kinks(k);
}

double max_of(const std::vector<double> &v)
{
    double m = -1.0;
    for (double x : v) m = std::max(m, x);
    return m;
}

// The points the routing measures distance from on a single-tree box: the tree's
// kinks found in the labels and the box's two moneyness edges (a kink just outside
// the box, which no label shows, bends the price near the edge).  Empty when the box
// is not a single tree.
std::vector<double> route_points(const hwt_surrogate *s)
{
    std::vector<double> r;
    if (s->kinks.empty()) return r;
    r = s->kinks;
    r.push_back(s->box.moneyness_min);
    r.push_back(s->box.moneyness_max);
    return r;
}

}  // namespace

extern "C" {

int hwt_surrogate_train(hwt_surrogate *s, const hwt_options *samples, const hwt_yield *y,
                        const hwt_train_config *cfg, hwt_train_stats *stats)
{
    if (!s || !samples || !y || !cfg) return HWT_EINVAL;
    const int n = samples->n;
    const int batch = cfg->batch > 0 ? cfg->batch : 8192;
    const int epochs = cfg->epochs > 0 ? cfg->epochs : 1;
    const float lam = (float)std::max(cfg->err_weight, 0.0);
    const double holdout = cfg->holdout > 0 ? std::min(cfg->holdout, 0.5) : 0.05;
    const double route_tol = cfg->route_tolerance > 0 ? cfg->route_tolerance : 1e-4;
    if (n < batch) return sfail(s, HWT_EINVAL, "fewer samples than one batch");
    if (stats) memset(stats, 0, sizeof(*stats));

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
    if ((r = features_for(s, samples, y))) return r;
    std::vector<double> Fh(n), bh(n);
    std::vector<uint8_t> ib(n);
    SCUDA(s, cudaMemcpyAsync(Fh.data(), s->F.p, 8ull * n, cudaMemcpyDeviceToHost, s->stream), "F D2H");
    SCUDA(s, cudaMemcpyAsync(bh.data(), s->base.p, 8ull * n, cudaMemcpyDeviceToHost, s->stream), "base D2H");
    SCUDA(s, cudaMemcpyAsync(ib.data(), s->inbox.p, n, cudaMemcpyDeviceToHost, s->stream), "box D2H");
    SCUDA(s, cudaStreamSynchronize(s->stream), "features");
    // in-box samples, shuffled once and split into training and held-out parts
    std::vector<int32_t> idx;
    idx.reserve(n);
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
    for (int64_t i = (int64_t)idx.size() - 1; i > 0; --i) std::swap(idx[i], idx[rnd() % (unsigned long long)(i + 1)]);
    const int64_t nin = (int64_t)idx.size();
    const int64_t nhold = (int64_t)(holdout * nin);
    const int64_t ntrain = nin - nhold;
    // single-tree box: the tree's payoff kinks from the training part's labels
    s->kinks.clear();
    s->kink_delta = -1.0;
    s->route_delta.clear();
    for (auto &v : s->cal_deltas) v.clear();
    if (single_tree_box(s->box)) {
        std::vector<double> kx(ntrain), kp(ntrain);
        std::vector<int8_t> kt(ntrain);
        for (int64_t j = 0; j < ntrain; ++j) {
            const int i = idx[j];
            kx[j] = samples->strike[i] / Fh[i];
            kp[j] = price[i];
            kt[j] = samples->type[i];
        }
        s->kinks = find_kinks(kx.data(), kp.data(), kt.data(), ntrain);
        if (s->kinks.size() > (size_t)kMaxKinks) s->kinks.clear();  // not one tree after all
    }
    if (ntrain < batch) return sfail(s, HWT_EINVAL, "fewer in-box training samples than one batch");
    double sum = 0, sum2 = 0;
    for (int64_t j = 0; j < ntrain; ++j) {
        const int i = idx[j];
        const double v = (price[i] - bh[i]) / Fh[i];
        sum += v; sum2 += v * v;
    }
    s->ymean = sum / ntrain;
    s->ystd = std::max(sqrt(std::max(sum2 / ntrain - s->ymean * s->ymean, 0.0)), 1e-12);

    // the epoch's sample list: on a single-tree box, samples within kKinkBand (moneyness)
    // of a kink appear kink_oversample times (the network's largest errors sit there)
    std::vector<int32_t> tr(idx.begin(), idx.begin() + ntrain);
    const int reps = std::max(1, std::min(cfg->kink_oversample, 16));
    const std::vector<double> rp = route_points(s);
    if (reps > 1 && !s->kinks.empty()) {
        for (int64_t j = 0; j < ntrain; ++j) {
            const int i = idx[j];
            if (kink_distance(rp, samples->strike[i] / Fh[i]) < kKinkBand)
                for (int q = 1; q < reps; ++q) tr.push_back(i);
        }
    }
    // hard-sample mining: nh more slots per epoch, refilled every hard_every epochs
    // (from the first quarter of the epochs on) with the training samples the network
    // prices worst; random training samples until the first mining
    const int hard_every = cfg->hard_every > 0 && cfg->hard_fraction > 0 ? cfg->hard_every : 0;
    const int64_t nh = hard_every ? (int64_t)(std::min(cfg->hard_fraction, 0.25) * ntrain) : 0;
    const std::vector<int32_t> tr0 = tr;
    for (int64_t j = 0; j < nh; ++j) tr.push_back(idx[rnd() % (unsigned long long)ntrain]);
    const int64_t nlist = (int64_t)tr.size();
    const int64_t nbuf = std::max(nlist, nin);

    Scoped guard;
    float *yv = nullptr, *Xs = nullptr, *ys = nullptr;
    double *dprice = nullptr;
    int32_t *perm = nullptr;
    StepState *dstate = nullptr;
    float *derr = nullptr;
    bool ok = cudaMalloc(&yv, 4ull * n) == cudaSuccess && cudaMalloc(&Xs, 4ull * kInPad * nbuf) == cudaSuccess &&
              cudaMalloc(&ys, 4ull * nbuf) == cudaSuccess && cudaMalloc(&dprice, 8ull * n) == cudaSuccess &&
              cudaMalloc(&perm, 4ull * nbuf) == cudaSuccess && cudaMalloc(&dstate, sizeof(StepState)) == cudaSuccess &&
              (nh == 0 || cudaMalloc(&derr, 4ull * n) == cudaSuccess);
    guard.ptrs = {yv, Xs, ys, dprice, perm, dstate, derr};
    if (!ok) {
        cudaGetLastError();
        return sfail(s, HWT_ENOMEM, "training buffers");
    }
    SCUDA(s, cudaMemcpyAsync(dprice, price.data(), 8ull * n, cudaMemcpyHostToDevice, s->stream), "prices H2D");
    targets_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(dprice, s->F.p, s->base.p, n, s->ymean, 1.0 / s->ystd, yv);
    SCUDA(s, cudaGetLastError(), "targets");
    if ((r = ensure_act(s, batch))) return r;

    // 3. Adam with cosine decay over the training part, reshuffled every epoch
    const int steps_per_epoch = (int)(nlist / batch);
    const long total = (long)steps_per_epoch * epochs;
    const double lr0 = cfg->lr > 0 ? cfg->lr : 1e-3, lr_min = cfg->lr_min;
    long step = 0;
    double last_epoch_loss = 0;
    {
        StepState h;
        memset(&h, 0, sizeof(h));
        h.t = s->adam_t;
        SCUDA(s, cudaMemcpy(dstate, &h, sizeof(h), cudaMemcpyHostToDevice), "step state H2D");
    }
    // one training step captured as a CUDA graph (about 30 kernels), replayed per step
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
    r = train_step(s, Xs, ys, dstate, batch, lr0, lr_min, (long long)total, lam);
    {
        const cudaError_t ce2 = cudaStreamEndCapture(s->stream, &graph);
        if (r) return r;
        SCUDA(s, ce2, "end capture");
    }
    SCUDA(s, cudaGraphInstantiate(&gexec, graph, 0), "instantiate training graph");
    if (nh > 0 && !s->out2.grow((size_t)n * kOut)) return sfail(s, HWT_ENOMEM, "mining outputs");
    std::vector<float> herr(nh > 0 ? n : 0);
    std::vector<int32_t> cand;
    int64_t minings = 0;
    double hard_thr = 0.0;
    const int first_mining = epochs / 4;
    SCUDA(s, cudaEventRecord(s->ev[0], s->stream), "event");
    for (int ep = 0; ep < epochs; ++ep) {
        if (nh > 0 && ep >= first_mining && (ep - first_mining) % hard_every == 0) {
            // price every sample with the current weights, keep the nh worst training samples
            if ((r = forward_fused(s, s->xf.p, (int)n, s->out2.p))) return r;
            sample_err_kernel<<<(int)((n + 255) / 256), 256, 0, s->stream>>>(s->out2.p, yv, s->F.p, (int)n, derr);
            SCUDA(s, cudaGetLastError(), "sample error kernel");
            SCUDA(s, cudaMemcpyAsync(herr.data(), derr, 4ull * n, cudaMemcpyDeviceToHost, s->stream), "errors D2H");
            SCUDA(s, cudaStreamSynchronize(s->stream), "mining");
            if ((r = gemm_status(s))) return r;
            cand.assign(idx.begin(), idx.begin() + ntrain);
            std::nth_element(cand.begin(), cand.begin() + (nh - 1), cand.end(),
                             [&](int32_t a, int32_t b) { return herr[a] > herr[b]; });
            hard_thr = (double)herr[cand[nh - 1]] * s->ystd;
            tr.assign(tr0.begin(), tr0.end());
            tr.insert(tr.end(), cand.begin(), cand.begin() + nh);
            ++minings;
        }
        for (int64_t i = nlist - 1; i > 0; --i) std::swap(tr[i], tr[rnd() % (unsigned long long)(i + 1)]);
        SCUDA(s, cudaMemcpyAsync(perm, tr.data(), 4ull * nlist, cudaMemcpyHostToDevice, s->stream), "perm H2D");
        gather_rows_kernel<<<(int)((nlist + 255) / 256), 256, 0, s->stream>>>(s->xf.p, yv, perm, (int)nlist, Xs, ys);
        SCUDA(s, cudaStreamSynchronize(s->stream), "shuffle");  // tr is reshuffled next epoch
        SCUDA(s, cudaMemsetAsync(s->d_loss, 0, sizeof(double), s->stream), "zero loss");
        SCUDA(s, cudaMemsetAsync(&dstate->k, 0, sizeof(int), s->stream), "epoch start");
        for (int k = 0; k < steps_per_epoch; ++k, ++step)
            SCUDA(s, cudaGraphLaunch(gexec, s->stream), "training step");
        double l = 0;
        SCUDA(s, cudaMemcpyAsync(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s->stream), "loss D2H");
        SCUDA(s, cudaStreamSynchronize(s->stream), "epoch");
        last_epoch_loss = l / steps_per_epoch;
    }
    SCUDA(s, cudaEventRecord(s->ev[1], s->stream), "event");
    SCUDA(s, cudaEventSynchronize(s->ev[1]), "event");
    {
        StepState h;
        SCUDA(s, cudaMemcpy(&h, dstate, sizeof(h), cudaMemcpyDeviceToHost), "step state D2H");
        s->adam_t = (long)h.t;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]);
    if ((r = gemm_status(s))) return r;

    // 4. router calibration on the held-out samples with the fused network
    double answered = 1.0, max_ans = 0.0, p99_ans = 0.0, max_all = 0.0;
    int64_t holdout_over = 0;
    s->route_tau = INFINITY;
    s->cal_valid = 0;
    if (nhold > 0) {
        std::vector<int32_t> hold(idx.begin() + ntrain, idx.end());
        if (!s->out2.grow((size_t)nhold * kOut)) return sfail(s, HWT_ENOMEM, "held-out outputs");
        SCUDA(s, cudaMemcpyAsync(perm, hold.data(), 4ull * nhold, cudaMemcpyHostToDevice, s->stream), "perm H2D");
        gather_rows_kernel<<<(int)((nhold + 255) / 256), 256, 0, s->stream>>>(s->xf.p, nullptr, perm, (int)nhold, Xs,
                                                                              nullptr);
        if ((r = forward_fused(s, Xs, (int)nhold, s->out2.p))) return r;
        std::vector<float> o((size_t)nhold * kOut);
        SCUDA(s, cudaMemcpyAsync(o.data(), s->out2.p, 4ull * nhold * kOut, cudaMemcpyDeviceToHost, s->stream), "D2H");
        SCUDA(s, cudaStreamSynchronize(s->stream), "held-out forward");
        if ((r = gemm_status(s))) return r;
        std::vector<double> pred(nhold), err(nhold);
        for (int64_t j = 0; j < nhold; ++j) {
            const int i = hold[j];
            const double net = bh[i] + Fh[i] * ((double)o[2 * j] * s->ystd + s->ymean);
            err[j] = fabs(net - price[i]);
            if (!(err[j] <= 1e300)) err[j] = INFINITY;
            pred[j] = exp((double)o[2 * j + 1]) * s->ystd * Fh[i];
            max_all = std::max(max_all, err[j]);
        }
        // moneyness of the held-out samples on a single-tree box
        std::vector<double> xm;
        if (!rp.empty()) {
            xm.resize(nhold);
            for (int64_t j = 0; j < nhold; ++j) xm[j] = samples->strike[hold[j]] / Fh[hold[j]];
        }
        // routing that keeps every held-out answer within tol: the error head's
        // threshold tau, or on a single-tree box a distance per routing point (each
        // held-out answer above tol widens the distance of the point nearest to it
        // to reach it, so a stray error far from the kinks costs the tree only the
        // options around one point); the answered fraction and the largest and p99
        // errors of the answered samples
        int64_t over = 0;  // answered held-out samples above the training tolerance
        auto calibrate = [&](double tol, double *tau, std::vector<double> *delta, double *ans, double *mx,
                             double *p99) {
            *tau = INFINITY;
            delta->clear();
            if (lam > 0) {
                *tau = calibrate_tau(pred, err, tol, ans, mx, p99);
                return;
            }
            std::vector<double> e;
            if (!xm.empty()) {
                route_distances(rp, xm.data(), err.data(), nhold, tol, *delta);
                for (int64_t j = 0; j < nhold; ++j)
                    if (!routed_near(rp, *delta, xm[j])) e.push_back(err[j]);
            } else {
                e = err;
            }
            *ans = (double)e.size() / nhold;
            *mx = *p99 = 0.0;
            if (!e.empty()) {
                std::sort(e.begin(), e.end());
                *mx = e.back();
                *p99 = e[std::min(e.size() - 1, (size_t)floor(0.99 * (e.size() - 1)))];
            }
        };
        calibrate(route_tol, &s->route_tau, &s->route_delta, &answered, &max_ans, &p99_ans);
        s->kink_delta = max_of(s->route_delta);
        for (int64_t j = 0; j < nhold; ++j) {
            const bool kept = s->route_tau == INFINITY ? (xm.empty() || !routed_near(rp, s->route_delta, xm[j]))
                                                       : pred[j] <= s->route_tau;
            if (kept && !(err[j] <= route_tol)) ++over;
        }
        holdout_over = over;
        for (int k = 0; k < kCalTols; ++k) {
            double mx, p99;
            calibrate(kCalTol[k], &s->cal_tau[k], &s->cal_deltas[k], &s->cal_answered[k], &mx, &p99);
            s->cal_delta[k] = max_of(s->cal_deltas[k]);
        }
        s->cal_valid = 1;
    }
    s->trained = 1;
    if (stats) {
        stats->final_loss = last_epoch_loss;
        stats->train_ms = ms;
        stats->label_ms = ts.total_ms;
        stats->steps = step;
        stats->samples = ntrain;
        stats->samples_per_s = (double)step * batch / (ms * 1e-3);
        stats->y_mean = s->ymean;
        stats->y_std = s->ystd;
        stats->route_threshold = s->route_tau;
        stats->holdout_answered = answered;
        stats->holdout_max_abs = max_ans;
        stats->holdout_p99_abs = p99_ans;
        stats->holdout_all_max_abs = max_all;
        stats->holdout = nhold;
        stats->holdout_over = holdout_over;
        stats->hard_minings = minings;
        stats->hard_threshold_abs = hard_thr;
        stats->n_kinks = (int64_t)s->kinks.size();
        stats->kink_delta = s->kink_delta;
        for (int k = 0; k < kCalTols; ++k) {
            stats->ladder_tolerance[k] = kCalTol[k];
            stats->ladder_answered[k] = s->cal_valid ? s->cal_answered[k] : 0.0;
        }
    }
    return HWT_OK;
}

int hwt_surrogate_price(hwt_surrogate *s, const hwt_options *o, const hwt_yield *y, double judge_fraction,
                        uint64_t seed, int tree_mode, double judge_tolerance, double *out, hwt_surrogate_stats *stats)
{
    if (!s || !o || !y || (o->n > 0 && !out)) return HWT_EINVAL;
    if (!s->trained) return sfail(s, HWT_EINVAL, "the surrogate has not been trained or loaded");
    if (tree_mode < HWT_BATCHED_FP64 || tree_mode > HWT_BATCHED_DF64) return sfail(s, HWT_EINVAL, "tree mode must be batched");
    const int n = o->n;
    if (stats) memset(stats, 0, sizeof(*stats));
    if (n == 0) return HWT_OK;
    int r;
    SCUDA(s, cudaEventRecord(s->ev[0], s->stream), "event");
    if ((r = features_for(s, o, y, s->ev[4]))) return r;
    if (!s->out2.grow((size_t)n * kOut) || !s->price.grow(n) || !s->kind.grow(n) || !s->list.grow(n) ||
        !s->counts.grow(4) || !s->tree.grow(n) || !s->errs.grow(n) || !grow_batch(s->sub, n))
        return sfail(s, HWT_ENOMEM, "pricing buffers");
    // network on every option (rows outside the box are not used)
    if ((r = forward_fused(s, s->xf.p, n, s->out2.p))) return r;
    SCUDA(s, cudaMemsetAsync(s->counts.p, 0, 16, s->stream), "counts");
    const double jf = std::min(std::max(judge_fraction, 0.0), 1.0);
    const unsigned long long thresh = jf >= 1.0 ? ~0ull : (unsigned long long)(jf * 18446744073709551616.0);
    // routing: the training tolerance's calibration, or, with a judge tolerance, the
    // ladder's largest tolerance not above kJudgeMargin times it (the strictest if none is)
    double tau = s->route_tau, route_tol = NAN;
    const std::vector<double> *delta = &s->route_delta;
    if (judge_tolerance > 0 && s->cal_valid) {
        int k = 0;
        for (int q = 0; q < kCalTols; ++q)
            if (kCalTol[q] <= kJudgeMargin * judge_tolerance * (1.0 + 1e-12)) k = q;
        tau = s->cal_tau[k];
        delta = &s->cal_deltas[k];
        route_tol = kCalTol[k];
    }
    // flag when exp(o1) ystd F > tau; tau = +inf: the router is off, tau <= 0: nothing is answered
    const float log_tau = std::isinf(tau) ? INFINITY : (tau > 0 ? (float)log(tau / s->ystd) : -INFINITY);
    const std::vector<double> rp = route_points(s);
    const int nk = delta->size() == rp.size() ? (int)rp.size() : 0;
    if (nk > 0) {
        if (!s->dkinks.grow(2 * (kMaxKinks + 2))) return sfail(s, HWT_ENOMEM, "kink buffer");
        SCUDA(s, cudaMemcpyAsync(s->dkinks.p, rp.data(), 8ull * nk, cudaMemcpyHostToDevice, s->stream), "kinks H2D");
        SCUDA(s, cudaMemcpyAsync(s->dkinks.p + nk, delta->data(), 8ull * nk, cudaMemcpyHostToDevice, s->stream),
              "distances H2D");
    }
    decode_route_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(s->out2.p, s->F.p, s->base.p, s->inbox.p,
                                                               s->opts.strike, n, s->ymean, s->ystd, log_tau,
                                                               s->dkinks.p, s->dkinks.p + nk, nk, seed, thresh,
                                                               s->price.p, s->kind.p, s->list.p, s->counts.p);
    SCUDA(s, cudaGetLastError(), "decode kernel");
    SCUDA(s, cudaEventRecord(s->ev[1], s->stream), "event");
    int32_t cnt[4] = {0, 0, 0, 0};
    SCUDA(s, cudaMemcpyAsync(cnt, s->counts.p, 16, cudaMemcpyDeviceToHost, s->stream), "counts D2H");
    SCUDA(s, cudaStreamSynchronize(s->stream), "route");
    if ((r = gemm_status(s))) return r;
    const int m = cnt[0];
    double tree_ms = 0;
    hwt_config tc;
    memset(&tc, 0, sizeof(tc));
    tc.mode = tree_mode;
    tc.use_graph = 1;
    if (m > 0) {
        gather_options_kernel<<<(m + 255) / 256, 256, 0, s->stream>>>(dev_view(s->opts, n), s->list.p, m, s->sub.strike,
                                                                    s->sub.bm, s->sub.om, s->sub.tu, s->sub.ts, s->sub.a,
                                                                    s->sub.sg, s->sub.ty);
        SCUDA(s, cudaStreamSynchronize(s->stream), "gather");  // the tree runs on the context's stream
        hwt_options so = abi_view(s->sub, m);
        hwt_stats ts;
        r = hwt_price_device(s->ctx, &so, y, &tc, s->tree.p, &ts);
        if (r && r != HWT_EINVAL) return sfail(s, r, hwt_last_error(s->ctx));
        tree_ms = ts.total_ms;
        scatter_tree_kernel<<<(m + 255) / 256, 256, 0, s->stream>>>(s->list.p, m, s->tree.p, s->kind.p, s->price.p,
                                                                  s->errs.p);
        SCUDA(s, cudaGetLastError(), "scatter kernel");
    }
    SCUDA(s, cudaEventRecord(s->ev[2], s->stream), "event");
    std::vector<double> errs(m);
    if (m > 0) SCUDA(s, cudaMemcpyAsync(errs.data(), s->errs.p, 8ull * m, cudaMemcpyDeviceToHost, s->stream), "errs D2H");
    SCUDA(s, cudaMemcpyAsync(out, s->price.p, 8ull * n, cudaMemcpyDeviceToHost, s->stream), "prices D2H");
    SCUDA(s, cudaEventRecord(s->ev[3], s->stream), "event");
    SCUDA(s, cudaStreamSynchronize(s->stream), "price");
    // judge: |network - tree| on the sample of the network's answers
    std::vector<double> e;
    e.reserve(cnt[KIND_JUDGED]);
    double worst = 0.0;
    for (int j = 0; j < m; ++j)
        if (errs[j] >= 0.0 || errs[j] != errs[j]) {
            const double v = errs[j] != errs[j] ? INFINITY : errs[j];
            e.push_back(v);
            worst = std::max(worst, v);
        }
    int fell_back = 0;
    double fallback_ms = 0;
    int64_t n_network = (int64_t)n - cnt[KIND_OUTSIDE] - cnt[KIND_FLAGGED];
    if (judge_tolerance > 0 && worst > judge_tolerance) {
        // the network failed its judge on this batch: the tree prices the rest of
        // the network's answers too
        SCUDA(s, cudaMemsetAsync(s->counts.p, 0, 4, s->stream), "counts");
        network_list_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(s->kind.p, n, s->list.p, s->counts.p);
        int32_t m2 = 0;
        SCUDA(s, cudaMemcpyAsync(&m2, s->counts.p, 4, cudaMemcpyDeviceToHost, s->stream), "count D2H");
        SCUDA(s, cudaStreamSynchronize(s->stream), "fallback list");
        if (m2 > 0) {
            gather_options_kernel<<<(m2 + 255) / 256, 256, 0, s->stream>>>(dev_view(s->opts, n), s->list.p, m2,
                                                                         s->sub.strike, s->sub.bm, s->sub.om, s->sub.tu,
                                                                         s->sub.ts, s->sub.a, s->sub.sg, s->sub.ty);
            SCUDA(s, cudaStreamSynchronize(s->stream), "gather");
            hwt_options so = abi_view(s->sub, m2);
            hwt_stats ts;
            r = hwt_price_device(s->ctx, &so, y, &tc, s->tree.p, &ts);
            if (r && r != HWT_EINVAL) return sfail(s, r, hwt_last_error(s->ctx));
            fallback_ms = ts.total_ms;
            scatter_tree_kernel<<<(m2 + 255) / 256, 256, 0, s->stream>>>(s->list.p, m2, s->tree.p, s->kind.p, s->price.p,
                                                                       s->errs.p);
            SCUDA(s, cudaMemcpyAsync(out, s->price.p, 8ull * n, cudaMemcpyDeviceToHost, s->stream), "prices D2H");
            SCUDA(s, cudaStreamSynchronize(s->stream), "fallback");
        }
        fell_back = 1;
        n_network = 0;
    }
    if (stats) {
        float t0 = 0, t1 = 0, t2 = 0, tc0 = 0;
        cudaEventElapsedTime(&tc0, s->ev[0], s->ev[4]);
        cudaEventElapsedTime(&t0, s->ev[4], s->ev[1]);
        cudaEventElapsedTime(&t1, s->ev[0], s->ev[3]);
        cudaEventElapsedTime(&t2, s->ev[1], s->ev[2]);
        stats->n_in_box = n - cnt[KIND_OUTSIDE];
        stats->n_routed = cnt[KIND_OUTSIDE];
        stats->n_judged = (int64_t)e.size();
        stats->n_flagged = cnt[KIND_FLAGGED];
        stats->n_network = n_network;
        if (!e.empty()) {
            std::sort(e.begin(), e.end());
            double sm = 0;
            for (double v : e) sm += v;
            stats->judge_max_abs = e.back();
            stats->judge_p99_abs = e[std::min(e.size() - 1, (size_t)floor(0.99 * (e.size() - 1)))];
            stats->judge_mean_abs = sm / e.size();
        }
        stats->fell_back = fell_back;
        stats->route_tolerance = route_tol;
        stats->copy_ms = tc0;
        stats->network_ms = t0;
        stats->tree_ms = tree_ms + fallback_ms;
        stats->route_ms = t2;
        stats->total_ms = t1 + fallback_ms;
    }
    return HWT_OK;
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
    const uint32_t magic = 0x48575453u, version = 6;
    const uint64_t np = s->n_params, nk = s->kinks.size();
    const int64_t t = s->adam_t;
    // per-point routing distances: the training tolerance's, then the ladder's
    auto put_deltas = [&](const std::vector<double> &d) {
        const uint64_t c = d.size();
        return fwrite(&c, 8, 1, f) == 1 && (c == 0 || fwrite(d.data(), 8, c, f) == c);
    };
    bool ok = fwrite(&magic, 4, 1, f) == 1 && fwrite(&version, 4, 1, f) == 1 && fwrite(&s->box, sizeof(hwt_box), 1, f) == 1 &&
              fwrite(&s->ymean, 8, 1, f) == 1 && fwrite(&s->ystd, 8, 1, f) == 1 && fwrite(&s->route_tau, 8, 1, f) == 1 &&
              fwrite(&s->kink_delta, 8, 1, f) == 1 && fwrite(&nk, 8, 1, f) == 1 &&
              (nk == 0 || fwrite(s->kinks.data(), 8, nk, f) == nk) && fwrite(&s->cal_valid, 4, 1, f) == 1 &&
              fwrite(s->cal_tau, 8, kCalTols, f) == kCalTols && fwrite(s->cal_delta, 8, kCalTols, f) == kCalTols &&
              fwrite(s->cal_answered, 8, kCalTols, f) == kCalTols && put_deltas(s->route_delta);
    for (int k = 0; k < kCalTols; ++k) ok = ok && put_deltas(s->cal_deltas[k]);
    ok = ok && fwrite(&t, 8, 1, f) == 1 && fwrite(&np, 8, 1, f) == 1 && fwrite(w.data(), 4, np, f) == np &&
              fwrite(m.data(), 4, np, f) == np && fwrite(v.data(), 4, np, f) == np;
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
    double ym = 0, ysd = 1, tau = INFINITY, kd = -1.0;
    uint64_t nk = 0;
    std::vector<double> kinks;
    int cal_valid = 0;
    double cal_tau[kCalTols], cal_delta[kCalTols], cal_answered[kCalTols];
    bool ok = fread(&magic, 4, 1, f) == 1 && fread(&version, 4, 1, f) == 1 && magic == 0x48575453u && version == 6 &&
              fread(&box, sizeof(hwt_box), 1, f) == 1 && fread(&ym, 8, 1, f) == 1 && fread(&ysd, 8, 1, f) == 1 &&
              fread(&tau, 8, 1, f) == 1 && fread(&kd, 8, 1, f) == 1 && fread(&nk, 8, 1, f) == 1 && nk <= (uint64_t)kMaxKinks;
    if (ok && nk) {
        kinks.resize(nk);
        ok = fread(kinks.data(), 8, nk, f) == nk;
    }
    ok = ok && fread(&cal_valid, 4, 1, f) == 1 && fread(cal_tau, 8, kCalTols, f) == kCalTols &&
         fread(cal_delta, 8, kCalTols, f) == kCalTols && fread(cal_answered, 8, kCalTols, f) == kCalTols;
    auto get_deltas = [&](std::vector<double> &d) {
        uint64_t c = 0;
        if (fread(&c, 8, 1, f) != 1 || c > (uint64_t)kMaxKinks + 2) return false;
        d.resize(c);
        return c == 0 || fread(d.data(), 8, c, f) == c;
    };
    std::vector<double> rdelta, cdeltas[kCalTols];
    ok = ok && get_deltas(rdelta);
    for (int k = 0; k < kCalTols; ++k) ok = ok && get_deltas(cdeltas[k]);
    ok = ok && fread(&t, 8, 1, f) == 1 && fread(&np, 8, 1, f) == 1 && np == s->n_params;
    std::vector<float> w(s->n_params), m(s->n_params), v(s->n_params);
    ok = ok && fread(w.data(), 4, np, f) == np && fread(m.data(), 4, np, f) == np && fread(v.data(), 4, np, f) == np;
    fclose(f);
    if (!ok) return sfail(s, HWT_EINVAL, "checkpoint is not a surrogate of this shape");
    s->box = box;
    box_norm(box, s->fn);
    s->ymean = ym;
    s->ystd = ysd;
    s->route_tau = tau;
    s->kink_delta = kd;
    s->kinks = kinks;
    s->route_delta = rdelta;
    for (int k = 0; k < kCalTols; ++k) s->cal_deltas[k] = cdeltas[k];
    s->cal_valid = cal_valid;
    memcpy(s->cal_tau, cal_tau, sizeof(cal_tau));
    memcpy(s->cal_delta, cal_delta, sizeof(cal_delta));
    memcpy(s->cal_answered, cal_answered, sizeof(cal_answered));
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

int hwt_find_kinks(const double *x, const double *price, const int8_t *type, int64_t n, double *kinks, int32_t cap,
                   int32_t *count)
{
    if (n < 0 || cap < 0 || !count || (n > 0 && (!x || !price || !type)) || (cap > 0 && !kinks)) return HWT_EINVAL;
    const std::vector<double> k = find_kinks(x, price, type, n);
    *count = (int32_t)std::min<size_t>(k.size(), (size_t)INT32_MAX);
    if (k.size() > (size_t)cap) return HWT_EINVAL;
    for (size_t j = 0; j < k.size(); ++j) kinks[j] = k[j];
    return HWT_OK;
}

int hwt_route_distances(const double *points, int32_t n_points, const double *x, const double *err, int64_t n,
                        double tol, double *delta, double *answered)
{
    if (n_points < 0 || n < 0 || (n_points > 0 && (!points || !delta)) || (n > 0 && (!x || !err))) return HWT_EINVAL;
    const std::vector<double> pts(points, points + n_points);
    std::vector<double> d;
    route_distances(pts, x, err, n, tol, d);
    for (int32_t k = 0; k < n_points; ++k) delta[k] = d[k];
    if (answered) {
        int64_t kept = 0;
        for (int64_t j = 0; j < n; ++j) kept += routed_near(pts, d, x[j]) ? 0 : 1;
        *answered = n > 0 ? (double)kept / (double)n : 1.0;
    }
    return HWT_OK;
}

}  // extern "C"
