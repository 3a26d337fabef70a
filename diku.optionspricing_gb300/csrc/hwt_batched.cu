// Batched Hull-White trinomial-tree pricer for sm_103a.
//
// What it computes is the reference's per-option pricer (seq/Seq.hpp:24-179):
// forward induction of Arrow-Debreu prices Q with an alpha fitted to the yield
// curve at every step, then backward induction of a 100-face bond with the
// option payoff applied at the option's maturity step.  How it computes it is
// different, and rests on one identity: alpha_i is the same for every node of a
// time step, so it only rescales whole rows.  Write Q_i = s_i * Qt_i.  Then
//   r_{i+1} = G o gather(r_i),   r_0 = e_center,    G_j = exp(-(j dr) dt)
//   Sum_i   = sum_k r_i[k]       (the reference's alpha sum is s_i * Sum_i)
//   s_k     = P_k / Sum_{k-1}    with P_k = exp(-R(k dt) k dt), Sum_0 = 1
// and the backward rows of the bond are  c_i = (s_n / s_i) * ct_i  with
//   ct_i = G o P ct_{i+1},  ct_n = 100.
// At the maturity step m the payoff max(X - (s_n/s_m) ct_m, 0) (put) or
// max((s_n/s_m) ct_m - X, 0) (call) starts a new row v, rolled back the same
// way; the price is s_m * v_0[center] (or s_n * ct_0[center] when m >= n).
// So each tree is two pure stencil sweeps with no per-step reduction, log or
// exp; the alpha fit collapses to two sums (rows m-1 and n-1) per option.
//
// Work layout: trees are sized, validated and binned on the device.  Trees up to
// 256 nodes wide run on a slice of a warp (L lanes x K nodes per lane, rows in
// registers, neighbours by shuffle); wider trees get a whole block (K nodes per
// thread, warp edges exchanged through shared memory, one barrier per step).
// One persistent kernel drains the block-tree queue and then the warp-task
// queue, both ordered by descending work.
//
// Precision modes: FP64 runs the stencils in the gather form with G folded into
// the coefficients (3 FMAs per node and pass, 4 while the +-jmax edge jumps are
// live).  FP32 and MIXED run them in float in a flux form that conserves
// probability exactly (stay = 1 - up - down is never formed), with G written as
// 1 + g, and the bond phase of the backward sweep carried as a deviation from
// 100.  MIXED keeps the two alpha-fit sums, the scales, the payoff and the final
// discount in double; FP32 does those in float too.
#include <float.h>
#include <stdio.h>

#include "hwt_internal.h"
#include "hwt_model.cuh"

namespace hwt {
namespace {

constexpr unsigned FULL = 0xffffffffu;

struct ModeF64 {
    typedef double Row;
    typedef double Scal;
    static constexpr bool kFlux = false;
};
struct ModeF32 {
    typedef float Row;
    typedef float Scal;
    static constexpr bool kFlux = true;
};
struct ModeMix {
    typedef float Row;
    typedef double Scal;
    static constexpr bool kFlux = true;
};

__device__ __forceinline__ int cls_K(int cls) { return cls / kNumL + 1; }

// Named barrier `id` over the `nthreads` threads of one tree's warp group (id 0
// with the whole block is __syncthreads).
__device__ __forceinline__ void tree_barrier(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Warps that price one tree together: `nthreads` threads from `base`, synchronised
// by named barrier `bar`.
struct Group {
    int base, nthreads, bar;
};
__device__ __forceinline__ int cls_L(int cls) { return 1 << (cls % kNumL); }

// Smallest L*K >= width with K in {1,2,3,4,6,8}, L in {1..32}; ties go to the
// larger K (more trees per warp, fewer shuffles per node).  K = 5 and 7 are left
// out to keep the kernel's code (and its instruction-cache footprint) small.
__host__ __device__ int pick_warp_class(int width)
{
    const int ks[6] = {8, 6, 4, 3, 2, 1};
    int best = -1, best_slots = 1 << 30;
    for (int q = 0; q < 6; ++q) {
        const int K = ks[q];
        for (int l = 0; l < kNumL; ++l) {
            const int slots = K << l;
            if (slots >= width && slots < best_slots) {
                best_slots = slots;
                best = (K - 1) * kNumL + l;
            }
        }
    }
    return best;
}

__device__ __forceinline__ int work_bucket(unsigned long long work)
{
    // 2 buckets per octave, descending: heavy work sorts first.
    const double lw = log2((double)work + 1.0);
    int b = (int)(lw * 2.0);
    if (b > kWorkBuckets - 1) b = kWorkBuckets - 1;
    return kWorkBuckets - 1 - b;
}

// ---------------------------------------------------------------------------
// Sizing, validation and binning.
// ---------------------------------------------------------------------------

__global__ void size_kernel(EngineParams p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int key = -1;
    unsigned long long nodes = 0;
    if (i < p.opt.n) {
        Shape s;
        int st = make_shape(s, p.opt.bond_maturity[i], p.opt.option_maturity[i], p.opt.term_unit[i],
                            p.opt.term_steps[i], p.opt.a[i], p.opt.sigma[i], p.max_width);
        const int8_t ty = p.opt.type[i];
        const double X = p.opt.strike[i];
        if (st == SHAPE_OK && ty != 0 && ty != 1) st = 6;
        if (st == SHAPE_OK && !isfinite(X)) st = SHAPE_NONFINITE;
        if (st != SHAPE_OK) {
            atomicAdd(&p.s.status->bad_count, 1);
            atomicMin(&p.s.status->first_bad, ((unsigned long long)(unsigned)i << 32) | (unsigned)st);
            p.out[i] = __longlong_as_double(0x7ff8000000000000ll);
            p.s.keys[i] = -1;
        } else {
            Tree t;
            t.dt = s.dt; t.dr = s.dr; t.M = s.M; t.X = X;
            t.idx = i; t.jmax = s.jmax; t.n = s.n; t.m = s.m; t.jc = s.jc; t.width = s.width;
            t.term_unit = p.opt.term_unit[i]; t.type = ty; t.edges = (int8_t)s.edges;
            p.s.trees[i] = t;
            nodes = (unsigned long long)s.nodes;
            const int tier = s.width <= p.big_threshold ? 2 : (s.width <= kMaxBlockK * p.group_threads ? 1 : 0);
            int cls = 0;
            if (tier == 2) {
                cls = pick_warp_class(s.width);
                const int top = s.edges ? (s.width - 1) % cls_K(cls) : 0;  // slot of node W-1
                cls |= top << 6;
            }
            const unsigned long long work = (unsigned long long)s.nodes + (unsigned long long)s.width;
            key = (tier * kWorkBuckets + work_bucket(work)) * kClassSlots + cls;
            p.s.keys[i] = key;
            atomicMax(&p.s.status->max_width, s.width);
            atomicMax(&p.s.status->max_height, s.n);
        }
    }
    // warp-aggregated histogram and node count
    for (int off = 16; off > 0; off >>= 1) nodes += __shfl_xor_sync(FULL, nodes, off);
    if (lane == 0 && nodes) atomicAdd(&p.s.status->nodes, nodes);
    const unsigned peers = __match_any_sync(FULL, key);
    if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&p.s.hist[key], __popc(peers));
}

// One block: exclusive scans of the key histogram into bin starts and warp-task
// starts.  kKeyBins / blockDim bins per thread.
__global__ void scan_kernel(EngineParams p)
{
    constexpr int T = 1024;
    constexpr int PER = kKeyBins / T;
    static_assert(PER * T == kKeyBins, "bins must split evenly over the scan threads");
    __shared__ int s_a[T], s_b[T];
    const int tid = threadIdx.x;
    int cnt[PER], tsk[PER];
    int sa = 0, sb = 0;
    for (int q = 0; q < PER; ++q) {
        const int b = tid * PER + q;
        const int c = p.s.hist[b];
        const bool warp = b >= 2 * kTierBins;
        int t = 0;
        if (warp && c > 0) {
            const int G = 32 / cls_L((b % kClassSlots) & 63);  // low 6 bits of the class: K and L
            t = (c + G - 1) / G;
        }
        cnt[q] = c; tsk[q] = t; sa += c; sb += t;
    }
    s_a[tid] = sa; s_b[tid] = sb;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        int va = 0, vb = 0;
        if (tid >= off) { va = s_a[tid - off]; vb = s_b[tid - off]; }
        __syncthreads();
        s_a[tid] += va; s_b[tid] += vb;
        __syncthreads();
    }
    int ea = s_a[tid] - sa, eb = s_b[tid] - sb;
    for (int q = 0; q < PER; ++q) {
        const int b = tid * PER + q;
        p.s.bin_start[b] = ea;
        p.s.task_start[b] = eb;
        ea += cnt[q]; eb += tsk[q];
    }
    if (tid == T - 1) p.s.status->n_warp_tasks = s_b[T - 1];
    // tier boundaries: options before the first tier-1 and tier-2 bins (global
    // writes of the block are visible to it after the barrier)
    __syncthreads();
    if (tid == 0) {
        const int t1 = p.s.bin_start[kTierBins], t2 = p.s.bin_start[2 * kTierBins];
        p.s.status->n_cta = t1;
        p.s.status->n_group = t2 - t1;
    }
}

// Places every valid option at its sorted position and emits one warp task per
// G consecutive small trees of a bin.
__global__ void scatter_kernel(EngineParams p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.opt.n) return;
    const int key = p.s.keys[i];
    if (key < 0) return;
    const int q = atomicAdd(&p.s.fill[key], 1);
    const int pos = p.s.bin_start[key] + q;
    p.s.order[pos] = i;
    if (key >= 2 * kTierBins) {
        const int cls = key % kClassSlots;
        const int G = 32 / cls_L(cls & 63);
        if (q % G == 0) {
            WarpTask t;
            t.start = pos;
            const int left = p.s.hist[key] - q;
            t.count = (int16_t)(left < G ? left : G);
            t.cls = (int16_t)cls;
            p.s.tasks[p.s.task_start[key] + q / G] = t;
        }
    }
}

// ---------------------------------------------------------------------------
// Per-thread tree slice: K consecutive nodes k0 .. k0+K-1 of one tree.
// ---------------------------------------------------------------------------

template <typename R, int K>
struct Ext {  // e[s + 2] is node k0 + s; e[0..1] left neighbours, e[K+2..K+3] right
    R e[K + 4];
};

template <class Mode, int K>
struct Slice {
    typedef typename Mode::Row R;
    typedef typename Mode::Scal S;

    R r[K];                 // current row
    R c0[K], c1[K], c2[K];  // FP64: fa/fb/fc or ba/bb/bc.  Flux: up, down, g.
    R cl, cr;               // flux: up of node k0-1, down of node k0+K
    // Edge jumps (+-jmax branch two nodes away).  Nodes 0 and 2 sit at compile-time
    // slots (0 and 2 % K); node W-1 sits at slot ts = (W-1) % K, which is the same
    // for every tree a warp prices (it is part of the warp class), so the top
    // edge is handled by one uniform switch per step instead of a test per slot.
    R jlo, jhi;             // FP64: jump coefficient times the receiving node's G; flux: pu_b, pd_c
    bool n0, n2, nw1, nw3;  // this thread owns node 0 / 2 / W-1 / W-3 of an edged tree
    int ts;

    __device__ __forceinline__ void setup_owners(const Tree &t, int k0)
    {
        const int W = t.width;
        const bool e = t.edges != 0;
        n0 = e && k0 == 0;
        n2 = e && k0 <= 2 && 2 < k0 + K;
        nw1 = e && k0 <= W - 1 && W - 1 < k0 + K;
        nw3 = e && k0 <= W - 3 && W - 3 < k0 + K;
        ts = (W - 1) % K;
    }

    // Coefficients for the forward sweep of tree `t`.
    __device__ __forceinline__ void setup_forward(const Tree &t, int k0)
    {
        const int W = t.width, jc = t.jc, jmax = t.jmax;
        setup_owners(t, k0);
        jlo = jhi = (R)0;
        if constexpr (!Mode::kFlux) {
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const int k = k0 + s;
                double a = 0.0, b = 0.0, c = 0.0;
                if (k < W) {
                    const int j = k - jc;
                    const double G = column_discount(j, t.dr, t.dt);
                    const Branch me = branch(j, jmax, t.M);
                    b = G * me.stay;
                    if (k >= 1) a = G * branch(j - 1, jmax, t.M).up;
                    if (k + 1 < W) c = G * branch(j + 1, jmax, t.M).down;
                    if (t.edges && k == 2) jlo = G * pu_b(-jmax, t.M);
                    if (t.edges && k == W - 3) jhi = G * pd_c(jmax, t.M);
                }
                c0[s] = a; c1[s] = b; c2[s] = c;
                r[s] = (k == jc) ? 1.0 : 0.0;
            }
        } else {
            const float Mf = (float)t.M, drdt = (float)(t.dr * t.dt);
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const int k = k0 + s;
                float u = 0.f, d = 0.f, g = 0.f;
                if (k < W) {
                    const int j = k - jc;
                    const float x = (float)j * Mf, x2 = x * x;
                    g = expm1f(-(float)j * drdt);
                    if (j == -jmax) {
                        u = -1.0f / 3.0f - x2 + 2.0f * x;   // pm_b
                        d = 0.f;
                    } else if (j == jmax) {
                        u = 0.f;
                        d = -1.0f / 3.0f - x2 - 2.0f * x;   // pm_c
                    } else {
                        u = 1.0f / 6.0f + (x2 + x) * 0.5f;  // pu_a
                        d = 1.0f / 6.0f + (x2 - x) * 0.5f;  // pd_a
                    }
                }
                c0[s] = u; c1[s] = d; c2[s] = g;
                r[s] = (k == jc) ? 1.f : 0.f;
            }
            // neighbours' up (node k0-1) and down (node k0+K) coefficients
            cl = 0.f; cr = 0.f;
            {
                const int kl = k0 - 1, kr = k0 + K;
                if (kl >= 0 && kl < W) {
                    const int j = kl - jc;
                    const float x = (float)j * Mf, x2 = x * x;
                    cl = (j == -jmax) ? (-1.0f / 3.0f - x2 + 2.0f * x) : (j == jmax ? 0.f : 1.0f / 6.0f + (x2 + x) * 0.5f);
                }
                if (kr < W) {
                    const int j = kr - jc;
                    const float x = (float)j * Mf, x2 = x * x;
                    cr = (j == -jmax) ? 0.f : (j == jmax ? (-1.0f / 3.0f - x2 - 2.0f * x) : 1.0f / 6.0f + (x2 - x) * 0.5f);
                }
            }
            if (t.edges) {
                const float xb = (float)(-jmax) * Mf, xt = (float)jmax * Mf;
                jlo = 1.0f / 6.0f + (xb * xb - xb) * 0.5f;  // pu_b: bottom edge jumps up two
                jhi = 1.0f / 6.0f + (xt * xt + xt) * 0.5f;  // pd_c: top edge jumps down two
            }
        }
    }

    // Coefficients for the backward sweep; rows start at the bond's face value
    // (flux form: as the deviation 0 from 100).
    __device__ __forceinline__ void setup_backward(const Tree &t, int k0)
    {
        const int W = t.width, jc = t.jc, jmax = t.jmax;
        if constexpr (!Mode::kFlux) {
            jlo = jhi = 0.0;
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const int k = k0 + s;
                double a = 0.0, b = 0.0, c = 0.0;
                if (k < W) {
                    const int j = k - jc;
                    const double G = column_discount(j, t.dr, t.dt);
                    const Branch me = branch(j, jmax, t.M);
                    a = G * me.up; b = G * me.stay; c = G * me.down;
                    if (t.edges && k == 0) jlo = G * me.jump;
                    if (t.edges && k == W - 1) jhi = G * me.jump;
                }
                c0[s] = a; c1[s] = b; c2[s] = c;
                r[s] = (k < W) ? 100.0 : 0.0;
            }
        } else {
            // up, down, g and the jump probabilities are the forward's
#pragma unroll
            for (int s = 0; s < K; ++s) r[s] = (R)0;
        }
    }

    // Top-edge terms with the slot of node W-1 known at compile time.
    template <int TS>
    __device__ __forceinline__ void top_forward(R (&v)[K], const Ext<R, K> &x) const
    {
        if constexpr (TS < K) {
            constexpr int S3 = (TS + 2 * K - 2) % K;  // slot of node W-3
            if constexpr (Mode::kFlux) {
                if (nw1) v[TS] = fma(-jhi, r[TS], v[TS]);
            }
            if (nw3) v[S3] = fma(jhi, x.e[S3 + 4], v[S3]);
        }
    }

    template <int TS>
    __device__ __forceinline__ void top_backward(R (&v)[K], const Ext<R, K> &x) const
    {
        if constexpr (TS < K) {
            if constexpr (Mode::kFlux) {
                if (nw1) v[TS] = fma(jhi, x.e[TS] - x.e[TS + 2], v[TS]);
            } else {
                if (nw1) v[TS] = fma(jhi, x.e[TS], v[TS]);
            }
        }
    }

    __device__ __forceinline__ void edges_forward(R (&v)[K], const Ext<R, K> &x) const
    {
        constexpr int S2 = 2 % K;  // slot of node 2
        if constexpr (Mode::kFlux) {
            if (n0) v[0] = fma(-jlo, r[0], v[0]);
        }
        if (n2) v[S2] = fma(jlo, x.e[S2], v[S2]);
        switch (ts) {
            case 0: top_forward<0>(v, x); break;
            case 1: top_forward<1>(v, x); break;
            case 2: top_forward<2>(v, x); break;
            case 3: top_forward<3>(v, x); break;
            case 4: top_forward<4>(v, x); break;
            case 5: top_forward<5>(v, x); break;
            case 6: top_forward<6>(v, x); break;
            default: top_forward<7>(v, x); break;
        }
    }

    __device__ __forceinline__ void edges_backward(R (&v)[K], const Ext<R, K> &x) const
    {
        if constexpr (Mode::kFlux) {
            if (n0) v[0] = fma(jlo, x.e[4] - x.e[2], v[0]);
        } else {
            if (n0) v[0] = fma(jlo, x.e[4], v[0]);
        }
        switch (ts) {
            case 0: top_backward<0>(v, x); break;
            case 1: top_backward<1>(v, x); break;
            case 2: top_backward<2>(v, x); break;
            case 3: top_backward<3>(v, x); break;
            case 4: top_backward<4>(v, x); break;
            case 5: top_backward<5>(v, x); break;
            case 6: top_backward<6>(v, x); break;
            default: top_backward<7>(v, x); break;
        }
    }

    // One forward step: r <- G o gather(r), reading neighbours from x.
    __device__ __forceinline__ void forward_step(const Ext<R, K> &x, bool edge_live)
    {
        R v[K];
        if constexpr (!Mode::kFlux) {
#pragma unroll
            for (int s = 0; s < K; ++s) {
                R t = c0[s] * x.e[s + 1];
                t = fma(c1[s], x.e[s + 2], t);
                t = fma(c2[s], x.e[s + 3], t);
                v[s] = t;
            }
            if (edge_live) edges_forward(v, x);
#pragma unroll
            for (int s = 0; s < K; ++s) r[s] = v[s];
        } else {
            R f[K], h[K];
#pragma unroll
            for (int s = 0; s < K; ++s) { f[s] = c0[s] * r[s]; h[s] = c1[s] * r[s]; }
            const R fl = cl * x.e[1], hr = cr * x.e[K + 2];
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const R fin = (s == 0) ? fl : f[s - 1];
                const R hin = (s == K - 1) ? hr : h[s + 1];
                v[s] = (r[s] + (fin - f[s])) + (hin - h[s]);
            }
            if (edge_live) edges_forward(v, x);
#pragma unroll
            for (int s = 0; s < K; ++s) r[s] = fma(c2[s], v[s], v[s]);
        }
    }

    // One backward step: r <- G o P r (flux: on the deviation from `base`).
    __device__ __forceinline__ void backward_step(const Ext<R, K> &x, bool edge_live, R base)
    {
        R v[K];
        if constexpr (!Mode::kFlux) {
#pragma unroll
            for (int s = 0; s < K; ++s) {
                R t = c0[s] * x.e[s + 3];
                t = fma(c1[s], x.e[s + 2], t);
                t = fma(c2[s], x.e[s + 1], t);
                v[s] = t;
            }
            if (edge_live) edges_backward(v, x);
#pragma unroll
            for (int s = 0; s < K; ++s) r[s] = v[s];
        } else {
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const R d0 = x.e[s + 2];
                const R up = x.e[s + 3] - d0, dn = x.e[s + 1] - d0;
                v[s] = d0 + fma(c0[s], up, c1[s] * dn);
            }
            if (edge_live) edges_backward(v, x);
#pragma unroll
            for (int s = 0; s < K; ++s) r[s] = fma(c2[s], v[s] + base, v[s]);
        }
    }

    __device__ __forceinline__ S partial_sum(int k0, int W) const
    {
        S acc = (S)0;
#pragma unroll
        for (int s = 0; s < K; ++s)
            if (k0 + s < W) acc += (S)r[s];
        return acc;
    }

    // Payoff at the maturity step: value = kappa * (base + row).
    __device__ __forceinline__ void payoff(S kappa, R base, double X, int type)
    {
#pragma unroll
        for (int s = 0; s < K; ++s) {
            const S c = kappa * ((S)base + (S)r[s]);
            const S x = (S)X;
            const S p = (type == 1) ? (x - c) : (c - x);
            r[s] = (R)(p < (S)0 ? (S)0 : p);
        }
    }

    __device__ __forceinline__ R pick(int slot) const
    {
        R v = r[0];
#pragma unroll
        for (int s = 1; s < K; ++s) v = (s == slot) ? r[s] : v;
        return v;
    }
};

template <typename R, int K>
__device__ __forceinline__ void fill_ext(Ext<R, K> &x, const R (&r)[K])
{
#pragma unroll
    for (int s = 0; s < K; ++s) x.e[s + 2] = r[s];
}

// Neighbour values within a warp segment of L lanes holding one tree.  The
// shuffles use width L, so a lane never reads another tree: at the segment ends
// it gets its own values back, which only ever meet a zero coefficient (the
// tree's outer nodes branch nowhere outward) or feed nodes outside the active
// cone.
template <typename R, int K>
__device__ __forceinline__ void exchange_warp(Ext<R, K> &x, const R (&r)[K], int L)
{
    fill_ext(x, r);
    if constexpr (K >= 2) {
        x.e[1] = __shfl_up_sync(FULL, r[K - 1], 1, L);
        x.e[0] = __shfl_up_sync(FULL, r[K - 2], 1, L);
        x.e[K + 2] = __shfl_down_sync(FULL, r[0], 1, L);
        x.e[K + 3] = __shfl_down_sync(FULL, r[1], 1, L);
    } else {
        x.e[1] = __shfl_up_sync(FULL, r[0], 1, L);
        x.e[0] = __shfl_up_sync(FULL, r[0], 2, L);
        x.e[3] = __shfl_down_sync(FULL, r[0], 1, L);
        x.e[4] = __shfl_down_sync(FULL, r[0], 2, L);
    }
}

// Neighbour values across a whole block: shuffles inside each warp, the first and
// last two nodes of every warp through shared memory (double buffered, so one
// barrier per step is enough).
template <typename R, int K>
__device__ __forceinline__ void exchange_block(Ext<R, K> &x, const R (&r)[K], R *sh, int parity, const Group &gr)
{
    // shared slots are indexed by the warp's index in the block; neighbours are
    // the adjacent warps of the same group
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int w0 = gr.base >> 5, w1 = w0 + (gr.nthreads >> 5);
    R *buf = sh + parity * (32 * 4);
    if constexpr (K >= 2) {
        if (lane == 0) { buf[warp * 4 + 0] = r[0]; buf[warp * 4 + 1] = r[1]; }
        if (lane == 31) { buf[warp * 4 + 2] = r[K - 2]; buf[warp * 4 + 3] = r[K - 1]; }
    } else {
        if (lane < 2) buf[warp * 4 + lane] = r[0];
        if (lane >= 30) buf[warp * 4 + lane - 28] = r[0];
    }
    tree_barrier(gr.bar, gr.nthreads);
    exchange_warp<R, K>(x, r, 32);
    const bool hasl = warp > w0, hasr = warp + 1 < w1;
    if constexpr (K >= 2) {
        if (lane == 0) {
            x.e[1] = hasl ? buf[(warp - 1) * 4 + 3] : (R)0;
            x.e[0] = hasl ? buf[(warp - 1) * 4 + 2] : (R)0;
        }
        if (lane == 31) {
            x.e[K + 2] = hasr ? buf[(warp + 1) * 4 + 0] : (R)0;
            x.e[K + 3] = hasr ? buf[(warp + 1) * 4 + 1] : (R)0;
        }
    } else {
        if (lane == 0) {
            x.e[1] = hasl ? buf[(warp - 1) * 4 + 3] : (R)0;
            x.e[0] = hasl ? buf[(warp - 1) * 4 + 2] : (R)0;
        }
        if (lane == 1) x.e[0] = hasl ? buf[(warp - 1) * 4 + 3] : (R)0;
        if (lane == 31) {
            x.e[3] = hasr ? buf[(warp + 1) * 4 + 0] : (R)0;
            x.e[4] = hasr ? buf[(warp + 1) * 4 + 1] : (R)0;
        }
        if (lane == 30) x.e[4] = hasr ? buf[(warp + 1) * 4 + 0] : (R)0;
    }
}

// Scalars of one tree after its forward sweep.
template <typename S>
struct Scales {
    S kappa;  // s_n / s_m, applied at the maturity step
    S final;  // s_m (payoff) or s_n (bond only)
};

template <typename S>
__device__ __forceinline__ Scales<S> tree_scales(const Tree &t, S sum_m1, S sum_n1, const DevYield &yc)
{
    Scales<S> sc;
    const S dt = (S)t.dt;
    const S *rates;
    if constexpr (sizeof(S) == 8) rates = (const S *)yc.rate; else rates = (const S *)yc.rate_f;
    const S Pn = discount_at_step<S>(t.n, dt, t.term_unit, rates, yc.day, yc.n);
    const S sn = Pn / sum_n1;
    if (t.m >= 0 && t.m < t.n) {
        S sm = (S)1;
        if (t.m >= 1) {
            const S Pm = discount_at_step<S>(t.m, dt, t.term_unit, rates, yc.day, yc.n);
            sm = Pm / sum_m1;
        }
        sc.kappa = sn / sm;
        sc.final = sm;
    } else {
        sc.kappa = (S)1;
        sc.final = sn;
    }
    return sc;
}

__device__ __forceinline__ bool pays_at(const Tree &t) { return t.m >= 0 && t.m < t.n; }

// ---------------------------------------------------------------------------
// Small trees: 32/L trees per warp, L lanes x K nodes each.
// ---------------------------------------------------------------------------
template <class Mode, int K>
__device__ void price_warp_task(const EngineParams &p, const WarpTask &task)
{
    typedef typename Mode::Row R;
    typedef typename Mode::Scal S;
    constexpr unsigned NONE = 0x7fffffffu;
    const int lane = threadIdx.x & 31;
    const int L = cls_L(task.cls & 63);
    const int g = lane / L, lis = lane & (L - 1);
    const bool valid = g < task.count;
    Tree t;
    if (valid) {
        t = p.s.trees[p.s.order[task.start + g]];
    } else {
        t.n = 0; t.m = -1; t.width = 1; t.jc = 0; t.jmax = 1; t.edges = 0; t.idx = -1;
        t.dt = 1.0; t.dr = 0.0; t.M = -0.5; t.X = 0.0; t.type = 0; t.term_unit = 365;
    }
    const int k0 = lis * K;
    const int W = t.width;
    Slice<Mode, K> sl;
    Ext<R, K> x;

    // ---- forward sweep: rows 1 .. n-1; the sums of rows m-1 and n-1 are kept.
    // Rows of trees that are done keep being updated (their segment is isolated by
    // the width-L shuffles), so the step loop carries no per-tree predicates.
    sl.setup_forward(t, k0);
    sl.ts = (task.cls >> 6) & 7;  // the warp's common top-edge slot
    const int e_f = (int)__reduce_min_sync(FULL, (valid && t.edges) ? (unsigned)t.jmax : NONE);
    const int rm = (t.m >= 2 && t.m < t.n) ? t.m - 1 : -1;  // row m-1 (row 0 sums to 1)
    const int rn = (t.n >= 2) ? t.n - 1 : -1;               // row n-1
    S sum_m1 = (S)1, sum_n1 = (S)1;
    const int fsteps = (int)__reduce_max_sync(FULL, (unsigned)(t.n > 1 ? t.n - 1 : 0));
    int i = 0;
    while (i < fsteps) {
        unsigned mine = NONE;
        if (rm > i) mine = (unsigned)rm;
        if (rn > i && (unsigned)rn < mine) mine = (unsigned)rn;
        const int ev = (int)__reduce_min_sync(FULL, mine);  // next row whose sum someone needs
        const int stop = ev < fsteps ? ev : fsteps;          // steps i .. stop-1 produce rows .. stop
        for (; i < stop; ++i) {
            exchange_warp<R, K>(x, sl.r, L);
            sl.forward_step(x, i >= e_f);
        }
        if (ev <= fsteps) {
            S acc = sl.partial_sum(k0, W);
            for (int off = 1; off < L; off <<= 1) acc += __shfl_xor_sync(FULL, acc, off);
            if (rm == ev) sum_m1 = acc;
            if (rn == ev) sum_n1 = acc;
        }
    }
    const Scales<S> sc = tree_scales<S>(t, sum_m1, sum_n1, p.yc);

    // ---- backward sweep from each tree's own height; rows of trees that have not
    // started yet are put back to the face value after every step.
    sl.setup_backward(t, k0);
    const int e_b = (int)__reduce_min_sync(FULL, (valid && t.edges) ? (unsigned)t.jmax : NONE);
    const int bsteps = (int)__reduce_max_sync(FULL, (unsigned)(t.n > 0 ? t.n : 0));
    const int n_min = (int)__reduce_min_sync(FULL, valid ? (unsigned)t.n : (unsigned)bsteps);
    const R face = Mode::kFlux ? (R)0 : (R)100;
    R base = Mode::kFlux ? (R)100 : (R)0;
    const bool pays = valid && pays_at(t);
    i = bsteps - 1;
    while (i >= 0) {
        // next maturity step at or below i (one per tree), -1 if none left
        const int pm = (int)__reduce_max_sync(FULL, (pays && t.m <= i) ? (unsigned)(t.m + 1) : 0u) - 1;
        const int lo = pm > 0 ? pm : 0;
        for (; i >= lo; --i) {
            exchange_warp<R, K>(x, sl.r, L);
            sl.backward_step(x, i >= e_b, base);
            if (i >= n_min && i >= t.n) {
#pragma unroll
                for (int s = 0; s < K; ++s) sl.r[s] = (k0 + s < W) ? face : (R)0;
            }
            if (i == pm && pays && t.m == i) {
                sl.payoff(sc.kappa, base, t.X, t.type);
                base = (R)0;
            }
        }
    }

    // ---- price at the root node
    const int owner = t.jc / K, slot = t.jc - owner * K;
    const R v = sl.pick(slot);
    if (valid && lis == owner) {
        double price;
        if (t.n <= 0) price = 100.0;
        else if (pays_at(t)) price = (double)(sc.final * (S)v);
        else price = (double)(sc.final * ((S)base + (S)v));
        p.out[t.idx] = price;
    }
}

// ---------------------------------------------------------------------------
// Wide trees: one whole block per tree, K nodes per thread.
// ---------------------------------------------------------------------------
template <class Mode, int K>
__device__ void price_block_tree(const EngineParams &p, const Tree &t, const Group &gr, typename Mode::Row *sh_x,
                                 typename Mode::Scal *sh_red)
{
    typedef typename Mode::Row R;
    typedef typename Mode::Scal S;
    const int tid = threadIdx.x - gr.base, lane = tid & 31, warp = tid >> 5, nw = gr.nthreads >> 5;
    const int aw0 = gr.base >> 5;  // first warp of the group in the block
    const int k0 = tid * K;
    const int W = t.width, jc = t.jc;
    const int wk0 = warp * 32 * K, wk1 = wk0 + 32 * K;  // this warp's node range
    Slice<Mode, K> sl;
    Ext<R, K> x;
    int parity = 0;

    sl.setup_forward(t, k0);
    S sum_m1 = (S)1, sum_n1 = (S)1;
    const int fsteps = t.n > 1 ? t.n - 1 : 0;
    for (int i = 0; i < fsteps; ++i) {
        exchange_block<R, K>(x, sl.r, sh_x, parity, gr);
        parity ^= 1;
        // rows outside the cone of row i+1 stay zero: skip whole warps there
        const int reach = (i + 1 < jc) ? i + 1 : jc;
        const bool active = wk1 > jc - reach && wk0 <= jc + reach && wk0 < W;
        if (active) sl.forward_step(x, t.edges && i >= t.jmax);
        const int row = i + 1;
        if (row == t.m - 1 || row == t.n - 1) {
            S acc = sl.partial_sum(k0, W);
            for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(FULL, acc, off);
            if (lane == 0) sh_red[aw0 + warp] = acc;
            tree_barrier(gr.bar, gr.nthreads);
            S tot = (S)0;
            for (int w = 0; w < nw; ++w) tot += sh_red[aw0 + w];
            tree_barrier(gr.bar, gr.nthreads);
            if (row == t.m - 1) sum_m1 = tot;
            if (row == t.n - 1) sum_n1 = tot;
        }
    }
    const Scales<S> sc = tree_scales<S>(t, sum_m1, sum_n1, p.yc);

    sl.setup_backward(t, k0);
    R base = Mode::kFlux ? (R)100 : (R)0;
    for (int i = t.n - 1; i >= 0; --i) {
        exchange_block<R, K>(x, sl.r, sh_x, parity, gr);
        parity ^= 1;
        const int reach = (i < t.jmax) ? i : t.jmax;
        const bool active = wk1 > jc - reach && wk0 <= jc + reach && wk0 < W;
        if (active) sl.backward_step(x, t.edges && i >= t.jmax, base);
        if (i == t.m) {
            sl.payoff(sc.kappa, base, t.X, t.type);
            base = (R)0;
        }
    }

    const int owner = jc / K, slot = jc - owner * K;
    const R v = sl.pick(slot);
    if (tid == owner) {
        double price;
        if (t.n <= 0) price = 100.0;
        else if (pays_at(t)) price = (double)(sc.final * (S)v);
        else price = (double)(sc.final * ((S)base + (S)v));
        p.out[t.idx] = price;
    }
}

// K = nodes per thread for a tree on group `gr` (width <= 8 * gr.nthreads).
template <class Mode>
__device__ __forceinline__ void dispatch_block_tree(const EngineParams &p, const Tree &t, const Group &gr,
                                                    typename Mode::Row *sh_x, typename Mode::Scal *sh_red)
{
    // K rounded up to 1, 2, 4 or 8 (warps left past the width skip their steps)
    const int K = (t.width + gr.nthreads - 1) / gr.nthreads;
    if (K <= 1) price_block_tree<Mode, 1>(p, t, gr, sh_x, sh_red);
    else if (K <= 2) price_block_tree<Mode, 2>(p, t, gr, sh_x, sh_red);
    else if (K <= 4) price_block_tree<Mode, 4>(p, t, gr, sh_x, sh_red);
    else price_block_tree<Mode, 8>(p, t, gr, sh_x, sh_red);
}

template <class Mode>
__global__ void __launch_bounds__(kPricingThreads, 1) price_kernel(EngineParams p)
{
    typedef typename Mode::Row R;
    typedef typename Mode::Scal S;
    __shared__ R sh_x[2 * 32 * 4];
    __shared__ S sh_red[32];
    __shared__ int sh_task[1 + 16];
    unsigned long long t_start = 0;
    if (p.record_busy && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));

    // Tier 0: trees wider than a group holds, one per block, heaviest first.
    const int n_cta = p.s.status->n_cta;
    for (;;) {
        if (threadIdx.x == 0) sh_task[0] = atomicAdd(&p.s.status->cta_counter, 1);
        __syncthreads();
        const int tsk = sh_task[0];
        __syncthreads();
        if (tsk >= n_cta) break;
        const Tree t = p.s.trees[p.s.order[tsk]];
        const Group gr{0, (int)blockDim.x, 0};
        dispatch_block_tree<Mode>(p, t, gr, sh_x, sh_red);
        __syncthreads();  // shared buffers are reused by the next tree
    }

    // Tier 1: each group of group_threads threads prices its own trees.
    {
        const int n_group = p.s.status->n_group;
        const int gsize = p.group_threads;
        const int g = (int)threadIdx.x / gsize;
        const Group gr{g * gsize, gsize, 1 + g};
        for (;;) {
            if ((int)threadIdx.x == gr.base) sh_task[1 + g] = atomicAdd(&p.s.status->group_counter, 1);
            tree_barrier(gr.bar, gr.nthreads);
            const int tsk = sh_task[1 + g];
            tree_barrier(gr.bar, gr.nthreads);
            if (tsk >= n_group) break;
            const Tree t = p.s.trees[p.s.order[n_cta + tsk]];
            dispatch_block_tree<Mode>(p, t, gr, sh_x, sh_red);
            tree_barrier(gr.bar, gr.nthreads);
        }
    }

    // Phase 2: warp tasks, each warp on its own.
    const int n_tasks = p.s.status->n_warp_tasks;
    const int lane = threadIdx.x & 31;
    for (;;) {
        int tsk = 0;
        if (lane == 0) tsk = atomicAdd(&p.s.status->warp_counter, 1);
        tsk = __shfl_sync(FULL, tsk, 0);
        if (tsk >= n_tasks) break;
        const WarpTask wt = p.s.tasks[tsk];
        switch (cls_K(wt.cls & 63)) {
            case 1: price_warp_task<Mode, 1>(p, wt); break;
            case 2: price_warp_task<Mode, 2>(p, wt); break;
            case 3: price_warp_task<Mode, 3>(p, wt); break;
            case 4: price_warp_task<Mode, 4>(p, wt); break;
            case 6: price_warp_task<Mode, 6>(p, wt); break;
            default: price_warp_task<Mode, 8>(p, wt); break;
        }
    }
    if (p.record_busy) {
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t_end;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_end));
            p.s.cta_busy[blockIdx.x] = t_end - t_start;
        }
    }
}

}  // namespace

int warp_class_of(int width, int *K, int *L)
{
    const int c = pick_warp_class(width);
    if (c < 0) return -1;
    if (K) *K = c / kNumL + 1;
    if (L) *L = 1 << (c % kNumL);
    return c;
}

int sizing_launches() { return 3; }

cudaError_t launch_sizing(const EngineParams &p, cudaStream_t stream)
{
    const int n = p.opt.n;
    cudaError_t e;
    if ((e = cudaMemsetAsync(p.s.hist, 0, sizeof(int32_t) * kKeyBins * 2, stream)) != cudaSuccess) return e;
    // status: zero counters, first_bad = all ones
    if ((e = cudaMemsetAsync(p.s.status, 0, sizeof(RunStatus), stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(&p.s.status->first_bad, 0xff, 8, stream)) != cudaSuccess) return e;
    if (n > 0) {
        size_kernel<<<(n + 255) / 256, 256, 0, stream>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    scan_kernel<<<1, 1024, 0, stream>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (n > 0) {
        scatter_kernel<<<(n + 255) / 256, 256, 0, stream>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_pricing(const EngineParams &p, int mode, int grid, cudaStream_t stream)
{
    switch (mode) {
        case MODE_BATCHED_FP64: price_kernel<ModeF64><<<grid, kPricingThreads, 0, stream>>>(p); break;
        case MODE_BATCHED_FP32: price_kernel<ModeF32><<<grid, kPricingThreads, 0, stream>>>(p); break;
        case MODE_BATCHED_MIXED: price_kernel<ModeMix><<<grid, kPricingThreads, 0, stream>>>(p); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int pricing_blocks_per_sm(int mode)
{
    const int block_threads = kPricingThreads;
    int nb = 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (mode) {
        case MODE_BATCHED_FP64: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, price_kernel<ModeF64>, block_threads, 0); break;
        case MODE_BATCHED_FP32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, price_kernel<ModeF32>, block_threads, 0); break;
        case MODE_BATCHED_MIXED: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, price_kernel<ModeMix>, block_threads, 0); break;
        default: break;
    }
    return e == cudaSuccess ? nb : 0;
}

}  // namespace hwt
