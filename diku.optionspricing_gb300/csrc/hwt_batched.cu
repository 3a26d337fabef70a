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
// discount in double precision, as double-float pairs on the FP32 pipes (the
// curve's discount factors come from the sizing pass, in double); FP32 does those
// in float too.
#include <float.h>
#include <stdio.h>

#include <atomic>
#include <type_traits>

#include "hwt_df64.cuh"
#include "hwt_internal.h"
#include "hwt_model.cuh"

namespace hwt {
namespace {

constexpr unsigned FULL = 0xffffffffu;

struct ModeF64 {
    typedef double Row;
    typedef double Scal;
    static constexpr bool kSizingDiscounts = false;  // P(n dt), P(m dt) from the sizing pass
    static constexpr bool kWide = false;  // K = 32 warp tasks (coefficients in shared memory)
    static constexpr bool kScratchPayoff = false;
    static constexpr bool kFlux = false;
};
struct ModeF32 {
    typedef float Row;
    typedef float Scal;
    static constexpr bool kSizingDiscounts = false;  // P(n dt), P(m dt) from the sizing pass
    static constexpr bool kWide = true;  // K = 32 warp tasks (coefficients in shared memory)
    static constexpr bool kScratchPayoff = false;
    static constexpr bool kFlux = true;
};
struct ModeMix {
    typedef float Row;
    typedef df64 Scal;    // double precision without the FP64 pipe (GB300 issues it at 1/64 of FP32)
    static constexpr bool kSizingDiscounts = true;  // P(n dt), P(m dt) from the sizing pass
    static constexpr bool kWide = true;  // K = 32 warp tasks (coefficients in shared memory)
    static constexpr bool kScratchPayoff = true;  // payoff through shared-memory scratch
    static constexpr bool kFlux = true;
};
struct ModeDF64 {
    typedef df64 Row;     // gather form like double rows, arithmetic on the FP32 pipes
    typedef double Scal;
    static constexpr bool kSizingDiscounts = true;  // P(n dt), P(m dt) from the sizing pass
    static constexpr bool kWide = false;  // K = 32 warp tasks (coefficients in shared memory)
    static constexpr bool kScratchPayoff = false;
    static constexpr bool kFlux = false;
};

// Width-w warp shuffles for every row type (df64 moves as two floats).
template <typename T>
__device__ __forceinline__ T shfl_up(T v, unsigned d, int w) { return __shfl_up_sync(0xffffffffu, v, d, w); }
template <typename T>
__device__ __forceinline__ T shfl_down(T v, unsigned d, int w) { return __shfl_down_sync(0xffffffffu, v, d, w); }
__device__ __forceinline__ df64 shfl_up(df64 v, unsigned d, int w)
{
    return df64_make(__shfl_up_sync(0xffffffffu, v.hi, d, w), __shfl_up_sync(0xffffffffu, v.lo, d, w));
}
__device__ __forceinline__ df64 shfl_down(df64 v, unsigned d, int w)
{
    return df64_make(__shfl_down_sync(0xffffffffu, v.hi, d, w), __shfl_down_sync(0xffffffffu, v.lo, d, w));
}

template <typename T>
__device__ __forceinline__ T shfl_xor(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ df64 shfl_xor(df64 v, int m)
{
    return df64_make(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
}

// Scalar types: double, float, or double-float pairs (df64) for float rows.
template <typename S>
constexpr bool kPairScal = std::is_same<S, df64>::value;

// A row value as a scalar (exact).
template <typename S, typename R>
__device__ __forceinline__ S to_scal(R x)
{
    if constexpr (kPairScal<S>) return df64_make(x, 0.f);
    else return (S)x;
}

// a + b of two row values as a scalar (exact for float rows).
template <typename S, typename R>
__device__ __forceinline__ S scal_sum(R a, R b)
{
    if constexpr (kPairScal<S>) return exact_sum(a, b);
    else return (S)a + (S)b;
}

// a x + b y + c z in the gather form: two FMAs after a product for double rows
// (this order is the one the FP64 results are pinned with), the compensated
// three-term product for df64 rows.
__device__ __forceinline__ double gather3(double a, double x, double b, double y, double c, double z)
{
    return fma(c, z, fma(b, y, a * x));
}
__device__ __forceinline__ df64 gather3(df64 a, df64 x, df64 b, df64 y, df64 c, df64 z) { return dot3(a, x, b, y, c, z); }

__device__ __forceinline__ int cls_K(int cls)
{
    const int k = cls / kNumL;
    return k < 8 ? k + 1 : (k == 8 ? 12 : (k == 9 ? 16 : 32));
}

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

// A warp task's class word: K index q and L index l as q * kNumL + l (bits 0-6),
// top-edge slot ts (bits 7-11).  Its sort-key slot packs the same triple densely:
// kNumL * (sum of the K values before K_q) + ts * kNumL + l, so slot % kNumL = l.
__device__ __forceinline__ int class_slot_base(int q)
{
    // kNumL x prefix sums of {1, 2, ..., 8, 12, 16, 32}
    return kNumL * (q <= 8 ? q * (q + 1) / 2 : (q == 9 ? 48 : (q == 10 ? 64 : 96)));
}
__device__ __forceinline__ int class_slot(int cls)
{
    const int q = (cls & kClsMask) / kNumL, l = (cls & kClsMask) % kNumL, ts = (cls >> kTsShift) & 31;
    return class_slot_base(q) + ts * kNumL + l;
}
__device__ __forceinline__ int slot_class(int slot)
{
    int q = 0;
#pragma unroll
    for (int t = 1; t < kNumK; ++t) q += slot >= class_slot_base(t);
    const int rest = slot - class_slot_base(q);
    return (q * kNumL + rest % kNumL) | ((rest / kNumL) << kTsShift);
}

// Smallest L*K >= width with K in the allowed set (bits of k_mask over
// {1, 2, ..., 8, 12, 16, 32}), L in {1..32}; ties go to the larger K (more trees per
// warp, fewer shuffles per node).  Each K used adds its code to the working set
// of the instruction cache, so float rows (whose warps are issue-bound) use only
// 1, 2, 4, 8, 16 and 32 by default; double rows (FP64-pipe-bound) use 1 .. 8.
__host__ __device__ int pick_warp_class(int width, int k_mask)
{
    const int ks[kNumK] = {1, 2, 3, 4, 5, 6, 7, 8, 12, 16, 32};  // the K values of kWarpK
    int best = -1, best_slots = 1 << 30;
    // K = 32 last: it wins only where nothing else fits (coefficients in shared
    // memory cost more than in registers)
    for (int i = 0; i < kNumK; ++i) {
        const int q = i < kNumK - 1 ? kNumK - 2 - i : kNumK - 1;
        const int K = ks[q];
        if (!((k_mask >> q) & 1)) continue;
        for (int l = 0; l < kNumL; ++l) {
            const int slots = K << l;
            if (slots >= width && slots < best_slots) {
                best_slots = slots;
                best = q * kNumL + l;
            }
        }
    }
    return best;
}

// Descending log buckets, `per` per octave: heavy work (tall trees) sorts first.
// (A float logarithm: buckets only order the work, and the double one costs the
// FP64-bound sizing pass about a tenth of its time.)
__device__ __forceinline__ int desc_bucket(double v, int per)
{
    int b = (int)(log2f((float)v + 1.0f) * (float)per);
    if (b > kBuckets - 1) b = kBuckets - 1;
    return kBuckets - 1 - b;
}

// Bucket of a tree inside its tier for sort order `sort` (HWT_SORT_*): the
// default orders the group tiers by work and the warp tier by height, tallest
// first; 'H'/'h' and 'W'/'w' order every tier by height or width, descending /
// ascending; 'i' keeps one bucket per tier (trees in arrival order, close to input
// order).
__device__ __forceinline__ int sort_bucket(int sort, bool warp_tier, int n, int width, long long nodes)
{
    const int per = warp_tier ? 8 : 4;
    switch (sort) {
        case 'H': return desc_bucket((double)n, per);
        case 'h': return kBuckets - 1 - desc_bucket((double)n, per);
        case 'W': return desc_bucket((double)width, per);
        case 'w': return kBuckets - 1 - desc_bucket((double)width, per);
        case 'i': return 0;
        default: return warp_tier ? desc_bucket((double)n, per) : desc_bucket((double)nodes + (double)width, per);
    }
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
    int wmax = 0, hmax = 0;
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
            t.disc = make_float4(0.f, 0.f, 0.f, 0.f);
            if (p.curve_discounts) {
                // the curve's discount factors at steps n and m, once per option
                // in double, for the pricing pass's double-float scales
                const df64 pn(discount_at_step<double>(s.n, s.dt, t.term_unit, p.yc.rate, p.yc.day, p.yc.n));
                const df64 pm((s.m >= 1 && s.m < s.n)
                                  ? discount_at_step<double>(s.m, s.dt, t.term_unit, p.yc.rate, p.yc.day, p.yc.n)
                                  : 1.0);
                t.disc = make_float4(pn.hi, pn.lo, pm.hi, pm.lo);
            }
            p.s.trees[i] = t;
            nodes = (unsigned long long)s.nodes;
            // warp tier up to the warp-task width; wider trees go to the smallest
            // group (not below group_threads) that holds them at max_group_k nodes
            // per thread
            const int warp_max = p.big_threshold < 32 * p.max_warp_k ? p.big_threshold : 32 * p.max_warp_k;
            int tier = kWarpTier;
            if (s.width > warp_max) {
                tier = 0;
                for (int t = kGroupTiers - 1; t > 0; --t) {
                    const int gs = kPricingThreads >> t;
                    if (gs >= p.group_threads && s.width <= p.max_group_k * gs) { tier = t; break; }
                }
            }
            int cls = 0;
            if (tier == kWarpTier) {
                cls = pick_warp_class(s.width, p.warp_k_mask);
                const int top = s.edges ? (s.width - 1) % cls_K(cls) : 0;  // slot of node W-1
                cls |= top << kTsShift;
            }
            // group tiers: one tree per task, by work (4 buckets per octave); warp
            // tier: trees of one class in lockstep, by height (8 per octave, <= 9% apart)
            // (a K = 32 task costs about twice a K = 16 one of the same height: it is
            // ordered as one twice as tall, so that it starts early enough)
            const int hw = (tier == kWarpTier && cls_K(cls) == kWideK) ? 2 * s.n : s.n;
            const int bucket = sort_bucket(p.sort, tier == kWarpTier, p.sort == 0 || p.sort == '-' ? hw : s.n, s.width,
                                           (long long)s.nodes);
            if (tier == kWarpTier) key = kWarpTier * kBuckets + bucket * kClassSlots + class_slot(cls);
            else key = tier * kBuckets + bucket;
            p.s.keys[i] = key;
            wmax = s.width;
            hmax = s.n;
        }
    }
    // warp-aggregated: one atomic per warp, not 32 on the same address
    wmax = (int)__reduce_max_sync(FULL, (unsigned)wmax);
    hmax = (int)__reduce_max_sync(FULL, (unsigned)hmax);
    if (lane == 0 && wmax > 0) {
        atomicMax(&p.s.status->max_width, wmax);
        atomicMax(&p.s.status->max_height, hmax);
    }
    // warp-aggregated histogram and node count
    for (int off = 16; off > 0; off >>= 1) nodes += __shfl_xor_sync(FULL, nodes, off);
    if (lane == 0 && nodes) atomicAdd(&p.s.status->nodes, nodes);
    const unsigned peers = __match_any_sync(FULL, key);
    if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&p.s.hist[key], __popc(peers));
}

// Zeroes the key histogram and fill counters and resets the run status (one
// launch instead of three memsets).
__global__ void reset_kernel(EngineParams p)
{
    int4 *h = reinterpret_cast<int4 *>(p.s.hist);  // hist | fill, 2 kKeyBins counters
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kKeyBins / 2; i += gridDim.x * blockDim.x)
        h[i] = make_int4(0, 0, 0, 0);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        RunStatus z = {};
        z.first_bad = ~0ull;
        *p.s.status = z;
    }
}

// Exclusive scans of the key histogram into bin starts and warp-task starts, one
// bin per thread (coalesced), in kScanBlocks blocks: each block writes the starts
// within itself and its totals; the last block to finish (a fence and a counter,
// no waiting) turns the totals into block offsets, which the scatter adds.
__device__ __forceinline__ int bin_tasks(int b, int c)
{
    if (b < kWarpTier * kBuckets || c == 0) return 0;  // group tiers: no warp tasks
    // G = 32 / L = 2^(5 - l) trees per task, l = slot % kNumL (kClassSlots is a
    // multiple of kNumL); shifts, not divisions: this runs for every bin
    const int sh = 5 - (b - kWarpTier * kBuckets) % kNumL;
    return (c + (1 << sh) - 1) >> sh;
}

__device__ __forceinline__ int warp_inclusive_scan(int v, int lane)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int u = __shfl_up_sync(FULL, v, off);
        if (lane >= off) v += u;
    }
    return v;
}

__global__ void __launch_bounds__(kScanBlock) scan_kernel(EngineParams p)
{
    constexpr int NW = kScanBlock / 32;
    __shared__ int s_a[NW], s_b[NW];
    __shared__ int s_last;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * kScanBlock + threadIdx.x;
    const int c = p.s.hist[b];
    const int t = bin_tasks(b, c);
    const int ia = warp_inclusive_scan(c, lane), it = warp_inclusive_scan(t, lane);
    if (lane == 31) { s_a[warp] = ia; s_b[warp] = it; }
    __syncthreads();
    if (warp == 0) {
        const int a = s_a[lane], x = s_b[lane];
        const int xa = warp_inclusive_scan(a, lane), xt = warp_inclusive_scan(x, lane);
        s_a[lane] = xa - a;
        s_b[lane] = xt - x;
        if (lane == 31) {
            p.s.bin_start[kScanOffsets + blockIdx.x] = xa;  // the block's totals
            p.s.task_start[kScanOffsets + blockIdx.x] = xt;
        }
    }
    __syncthreads();
    p.s.bin_start[b] = s_a[warp] + ia - c;
    p.s.task_start[b] = s_b[warp] + it - t;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&p.s.status->scan_blocks_done, 1) == kScanBlocks - 1;
    __syncthreads();
    if (!s_last) return;
    // last block: exclusive scan of the block totals, one per thread
    __threadfence();
    const int x = threadIdx.x;
    const int ba = x < kScanBlocks ? __ldcg(p.s.bin_start + kScanOffsets + x) : 0;
    const int bt = x < kScanBlocks ? __ldcg(p.s.task_start + kScanOffsets + x) : 0;
    const int ja = warp_inclusive_scan(ba, lane), jt = warp_inclusive_scan(bt, lane);
    if (lane == 31) { s_a[warp] = ja; s_b[warp] = jt; }
    __syncthreads();
    if (warp == 0) {
        const int a = s_a[lane], y = s_b[lane];
        const int xa = warp_inclusive_scan(a, lane), xt = warp_inclusive_scan(y, lane);
        s_a[lane] = xa - a;
        s_b[lane] = xt - y;
        if (lane == 31) p.s.status->n_warp_tasks = xt;
    }
    __syncthreads();
    if (x < kScanBlocks) {
        p.s.bin_start[kScanOffsets + x] = s_a[warp] + ja - ba;
        p.s.task_start[kScanOffsets + x] = s_b[warp] + jt - bt;
    }
    // tier boundaries: the group tiers' bins all lie in scan block 0 (offset 0)
    static_assert((kGroupTiers + 1) * kBuckets <= kScanBlock, "tier bins in the first scan block");
    if (x < kGroupTiers) {
        const int a = __ldcg(p.s.bin_start + x * kBuckets), e = __ldcg(p.s.bin_start + (x + 1) * kBuckets);
        p.s.status->tier_start[x] = a;
        p.s.status->tier_count[x] = e - a;
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
    const int blk = kScanOffsets + key / kScanBlock;
    const int pos = p.s.bin_start[key] + p.s.bin_start[blk] + q;
    p.s.order[pos] = i;
    if (key >= kWarpTier * kBuckets) {
        const int sh = 5 - (key - kWarpTier * kBuckets) % kNumL;  // G = 2^sh trees per task
        const int G = 1 << sh;
        if ((q & (G - 1)) == 0) {
            WarpTask t;
            t.start = pos;
            const int left = p.s.hist[key] - q;
            t.count = (int16_t)(left < G ? left : G);
            t.cls = (int16_t)slot_class((key - kWarpTier * kBuckets) % kClassSlots);
            p.s.tasks[p.s.task_start[key] + p.s.task_start[blk] + (q >> sh)] = t;
        }
    }
}

// ---------------------------------------------------------------------------
// Per-thread tree slice: K consecutive nodes k0 .. k0+K-1 of one tree.
// ---------------------------------------------------------------------------

// Values of the two nodes left of a thread's slice (l1 = k0-1, l2 = k0-2) and the
// two right of it (r1 = k0+K, r2 = k0+K+1), all from the current row.
template <typename R>
struct Halo {
    R l1, l2, r1, r2;
};

// A thread's K node values in registers.  Float rows with an even K are held as
// K/2 pairs (node s, node s + K/2), so the flux stencils run on the paired FP32
// instructions (two FMAs per issue slot): the pair of right neighbours of pair p
// is pair p+1, except across the slice's middle.
template <typename R, int K,
          bool PAIRED = (std::is_same<R, float>::value || std::is_same<R, df64>::value) && K % 2 == 0>
struct Nodes {
    static constexpr bool kPaired = false;
    R v[K];
    __device__ __forceinline__ R &operator[](int s) { return v[s]; }
    __device__ __forceinline__ const R &operator[](int s) const { return v[s]; }
};
template <int K>
struct Nodes<float, K, true> {
    static constexpr bool kPaired = true;
    static constexpr int H = K / 2;
    float2 v[H];
    __device__ __forceinline__ float &operator[](int s) { return s < H ? v[s].x : v[s - H].y; }
    __device__ __forceinline__ const float &operator[](int s) const { return s < H ? v[s].x : v[s - H].y; }
    __device__ __forceinline__ float2 pair(int q) const { return v[q]; }
};

// One double-float node inside the paired storage (its hi and lo sit in two pairs).
struct DF64Ref {
    float &hi, &lo;
    __device__ __forceinline__ operator df64() const { return df64_make(hi, lo); }
    __device__ __forceinline__ DF64Ref &operator=(df64 x)
    {
        hi = x.hi;
        lo = x.lo;
        return *this;
    }
    __device__ __forceinline__ DF64Ref &operator+=(df64 x) { return *this = df64_make(hi, lo) + x; }
};

// Double-float rows with an even K: the same pairing, hi and lo parts in separate
// pairs, so the compensated products run on the paired instructions.
template <int K>
struct Nodes<df64, K, true> {
    static constexpr bool kPaired = true;
    static constexpr int H = K / 2;
    float2 hi[H], lo[H];
    __device__ __forceinline__ DF64Ref operator[](int s)
    {
        return s < H ? DF64Ref{hi[s].x, lo[s].x} : DF64Ref{hi[s - H].y, lo[s - H].y};
    }
    __device__ __forceinline__ df64 operator[](int s) const
    {
        return s < H ? df64_make(hi[s].x, lo[s].x) : df64_make(hi[s - H].y, lo[s - H].y);
    }
    __device__ __forceinline__ df64x2 pair(int q) const
    {
        df64x2 r;
        r.hi = hi[q];
        r.lo = lo[q];
        return r;
    }
    __device__ __forceinline__ void set_pair(int q, const df64x2 &x)
    {
        hi[q] = x.hi;
        lo[q] = x.lo;
    }
};

// Adds d * s to lane (S < H ? x : y) of a double-float pair (a scalar fix-up of one node).
template <int S, int H>
__device__ __forceinline__ void fma_lane(df64x2 &v, df64 d, df64 s)
{
    if constexpr (S < H) {
        const df64 t = fma(d, s, df64_make(v.hi.x, v.lo.x));
        v.hi.x = t.hi;
        v.lo.x = t.lo;
    } else {
        const df64 t = fma(d, s, df64_make(v.hi.y, v.lo.y));
        v.hi.y = t.hi;
        v.lo.y = t.lo;
    }
}

// One float-row node's payoff, kappa (base + r) against the strike x, in double
// precision with float operations:
//   s = base + r exactly (FastTwoSum: |r| <= base = 100 before the payoff)
//   c = kappa s as kh sh + [exact error of kh sh] + kl sh + kh sl
//   x - c = (xh - kh sh) + ((xl - err) - cross)
// xh - kh sh is exact where x and c are close (Sterbenz), the only case where the
// difference needs the low parts; the omitted kl sl is below u^2 |c| (4e-13 per
// 100 face).
__device__ __forceinline__ float payoff_value(float r, float base, df64 kappa, df64 x, int type)
{
    const float sh = __fadd_rn(base, r);
    const float sl = __fsub_rn(r, __fsub_rn(sh, base));
    const float ph = __fmul_rn(kappa.hi, sh);
    const float pl = __fmaf_rn(kappa.hi, sh, -ph);
    const float cr = __fmaf_rn(kappa.lo, sh, __fmul_rn(kappa.hi, sl));
    const float d = __fadd_rn(__fsub_rn(x.hi, ph), __fsub_rn(__fsub_rn(x.lo, pl), cr));
    const float p = (type == 1) ? d : -d;
    return p < 0.f ? 0.f : p;
}

// The switch cases on the top edge's slot, 0..31 (cases a slice cannot reach stay
// empty: see kTopSlot).
#define HWT_TOP_CASES(X)                                                                          \
    X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) \
    X(17) X(18) X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27) X(28) X(29) X(30) X(31)

// Coefficients of a K = 32 slice in shared memory (three arrays of 32 x 32 floats
// would not fit in registers beside the row): pair q of a lane at base[q * 32],
// base offset by the lane, so a warp's access to pair q is 256 contiguous bytes.
struct SmemPairs {
    float2 *base;
    __device__ __forceinline__ float2 &operator[](int q) const { return base[q * 32]; }
};
template <int K>
struct SmemNodes {
    static constexpr bool kPaired = true;
    static constexpr int H = K / 2;
    SmemPairs v;
    __device__ __forceinline__ float &operator[](int s) const { return s < H ? v[s].x : v[s - H].y; }
    // A step's read of pair q: a volatile shared load, so the compiler cannot keep
    // the constant coefficients in registers across the step loop (which is what
    // their place in shared memory is for)
    __device__ __forceinline__ float2 pair(int q) const
    {
        float2 c;
        const unsigned a = (unsigned)__cvta_generic_to_shared(v.base + q * 32);
        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(c.x), "=f"(c.y) : "r"(a) : "memory");
        return c;
    }
};
template <typename R, int K>
struct CoefStore {
    typedef Nodes<R, K> type;
};
template <>
struct CoefStore<float, kWideK> {
    typedef SmemNodes<kWideK> type;
};

template <class Mode, int K>
struct Slice {
    typedef typename Mode::Row R;
    typedef typename Mode::Scal S;

    Nodes<R, K> r;                            // current row, nodes k0 .. k0+K-1
    typename CoefStore<R, K>::type c0, c1, c2;  // FP64: fa/fb/fc or ba/bb/bc.  Flux: up, -down of the next node, g.

    // K = 32: the warp's shared-memory region for the coefficients (kWideWarpFloat2).
    __device__ __forceinline__ void bind_coefficients(float2 *warp_region, int lane)
    {
        if constexpr (K == kWideK && std::is_same<R, float>::value) {
            c0.v.base = warp_region + lane;
            c1.v.base = warp_region + (K / 2) * 32 + lane;
            c2.v.base = warp_region + 2 * (K / 2) * 32 + lane;
        }
    }
    R cl, cd0;              // flux: up of node k0-1, -down of node k0
    // Edge jumps (+-jmax branch two nodes away).  Nodes 0, 1 and 2 sit at compile-time
    // slots (0, 1 % K, 2 % K) and their terms are part of the step loop (flux rows: the
    // bottom jump rides on links 0 and 1, node 0's up coefficient holding pu_b); node
    // W-1 sits at slot ts = (W-1) % K, known only at run time, so the top-edge terms
    // are applied after the in-place step from old values saved before it, through a
    // switch on ts.  Warp tasks group trees by ts (it is part of the warp class),
    // which keeps the switch uniform across the warp.
    R jlo, jhi;             // FP64: jump coefficient times the receiving node's G; flux: pu_b, pd_c (1 + g_{W-1})
    R jg3;                  // flux: pd_c (1 + g_{W-3}), the top jump discounted at the node it lands on
    bool n0, n1, n2, nw1, nw3;  // this thread owns node 0 / 1 / 2 / W-1 / W-3 of an edged tree
    int ts;

    __device__ __forceinline__ void setup_owners(const Tree &t, int k0)
    {
        const int W = t.width;
        const bool e = t.edges != 0;
        n0 = e && k0 == 0;
        n1 = e && k0 <= 1 && 1 < k0 + K;
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
        jlo = jhi = jg3 = (R)0;
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
            float dn[K];  // down coefficient of node k0+s
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const int k = k0 + s;
                float u = 0.f, d = 0.f, g = 0.f;
                if (k < W) {
                    const int j = k - jc;
                    const float x = (float)j * Mf, x2 = x * x;
                    g = expm1f(-(float)j * drdt);
                    if (j == -jmax) {
                        // pm_b, plus pu_b on an edged tree: node 0's jump up two crosses
                        // this link and the next one (the step adds it to the next)
                        u = -1.0f / 3.0f - x2 + 2.0f * x;
                        if (t.edges) u += 1.0f / 6.0f + (x2 - x) * 0.5f;
                        d = 0.f;
                    } else if (j == jmax) {
                        u = 0.f;
                        d = -1.0f / 3.0f - x2 - 2.0f * x;   // pm_c
                    } else {
                        u = 1.0f / 6.0f + (x2 + x) * 0.5f;  // pu_a
                        d = 1.0f / 6.0f + (x2 - x) * 0.5f;  // pd_a
                    }
                }
                c0[s] = u; dn[s] = d; c2[s] = g;
                r[s] = (k == jc) ? 1.f : 0.f;
            }
            // neighbours' up (node k0-1) and down (node k0+K) coefficients
            float cr = 0.f;
            cl = 0.f;
            {
                const int kl = k0 - 1, kr = k0 + K;
                if (kl >= 0 && kl < W) {
                    const int j = kl - jc;
                    const float x = (float)j * Mf, x2 = x * x;
                    cl = (j == -jmax) ? (-1.0f / 3.0f - x2 + 2.0f * x) : (j == jmax ? 0.f : 1.0f / 6.0f + (x2 + x) * 0.5f);
                    if (j == -jmax && t.edges) cl += 1.0f / 6.0f + (x2 - x) * 0.5f;
                }
                if (kr < W) {
                    const int j = kr - jc;
                    const float x = (float)j * Mf, x2 = x * x;
                    cr = (j == -jmax) ? 0.f : (j == jmax ? (-1.0f / 3.0f - x2 - 2.0f * x) : 1.0f / 6.0f + (x2 - x) * 0.5f);
                }
            }
            // c1 holds the next node's down coefficient, negated: the net flux from
            // node k to node k+1 is then fma(c0, r_k, c1 r_{k+1})
            cd0 = -dn[0];
#pragma unroll
            for (int s = 0; s < K; ++s) c1[s] = -((s < K - 1) ? dn[s + 1] : cr);
            if (t.edges) {
                const float xb = (float)(-jmax) * Mf, xt = (float)jmax * Mf;
                jlo = 1.0f / 6.0f + (xb * xb - xb) * 0.5f;  // pu_b: bottom edge jumps up two
                // pd_c (top edge jumps down two), times the discount 1 + g of the node it
                // leaves (W-1) and of the node it reaches (W-3): the top-edge terms are
                // added to the discounted row, one fused multiply-add each
                const float pdc = 1.0f / 6.0f + (xt * xt + xt) * 0.5f;
                jhi = fmaf(pdc, expm1f(-(float)jmax * drdt), pdc);
                jg3 = fmaf(pdc, expm1f(-(float)(jmax - 2) * drdt), pdc);
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

    // Old value of the node `d` nodes away from slot S (d in -2..2), from the row
    // or the halo.
    template <int S, int D>
    __device__ __forceinline__ R old_at(const Halo<R> &h) const
    {
        constexpr int q = S + D;
        if constexpr (q >= 0 && q < K) return r[q];
        else if constexpr (q == -1) return h.l1;
        else if constexpr (q == -2) return h.l2;
        else if constexpr (q == K) return h.r1;
        else return h.r2;
    }

    // Old values the top-edge terms need, per compile-time slot TS of node W-1.
    // Seen from the thread owning node W-1: w1 = node W-1, w3 = node W-3.  Seen
    // from the thread owning node W-3 (possibly the previous thread): w1b = node W-1.
    // Slots node W-1 can take: W = 2 jc + 1 is odd, so for an even K the slot
    // (W-1) % K is even; the other switch cases stay empty (less code to fetch).
    template <int TS>
    static constexpr bool kTopSlot = TS < K && (K % 2 == 1 || TS % 2 == 0);

    template <int TS>
    __device__ __forceinline__ void save_top(const Halo<R> &h, R &w1, R &w3, R &w1b) const
    {
        if constexpr (kTopSlot<TS>) {
            constexpr int S3 = (TS + 2 * K - 2) % K;  // slot of node W-3
            w1 = r[TS];
            w3 = old_at<TS, -2>(h);
            w1b = old_at<S3, 2>(h);
        }
    }

    __device__ __forceinline__ void top_values(const Halo<R> &h, R &w1, R &w3, R &w1b) const
    {
        switch (ts) {
#define HWT_SAVE_TOP(T) \
    case T: save_top<T>(h, w1, w3, w1b); break;
            HWT_TOP_CASES(HWT_SAVE_TOP)
#undef HWT_SAVE_TOP
            default: break;
        }
    }

    // Adds c to the finished value at slot S (gather-form rows: c already carries G).
    template <int S>
    __device__ __forceinline__ void add_at(R c)
    {
        r[S] += c;
    }

    template <int TS, bool FWD>
    __device__ __forceinline__ void top_fix(R w1, R w3, R w1b)
    {
        if constexpr (kTopSlot<TS>) {
            constexpr int S3 = (TS + 2 * K - 2) % K;
            if constexpr (Mode::kFlux) {
                // the discounts are in jhi and jg3
                if constexpr (FWD) {
                    if (nw1) r[TS] = fma(-jhi, w1, r[TS]);
                    if (nw3) r[S3] = fma(jg3, w1b, r[S3]);
                } else {
                    if (nw1) r[TS] = fma(jhi, w3 - w1, r[TS]);
                }
            } else if constexpr (FWD) {
                if (nw3) add_at<S3>(jhi * w1b);
            } else {
                if (nw1) add_at<TS>(jhi * w3);
            }
        }
    }

    template <bool FWD>
    __device__ __forceinline__ void top_fixes(R w1, R w3, R w1b)
    {
        switch (ts) {
#define HWT_TOP_FIX(T) \
    case T: top_fix<T, FWD>(w1, w3, w1b); break;
            HWT_TOP_CASES(HWT_TOP_FIX)
#undef HWT_TOP_FIX
            default: break;
        }
    }

    // Top-edge fixes of the step just taken, then the halo of the next step and its
    // top-edge values: one switch on ts where a step would otherwise take two.
    // (exchange_warp is defined after Slice; X is that function, passed in.)
    template <bool FWD, class X>
    __device__ __forceinline__ void fix_then_next(R &w1, R &w3, R &w1b, Halo<R> &h, X &&exchange)
    {
        switch (ts) {
#define HWT_FIX_NEXT(T)                                  \
    case T:                                              \
        if constexpr (kTopSlot<T>) {                     \
            top_fix<T, FWD>(w1, w3, w1b);                \
            h = exchange(K < 3 || T < 2 || !Mode::kFlux); \
            save_top<T>(h, w1, w3, w1b);                 \
        }                                                \
        break;
            HWT_TOP_CASES(HWT_FIX_NEXT)
#undef HWT_FIX_NEXT
            default: break;
        }
    }

    // One forward step, in place: r <- G o gather(r).  TOP = false leaves the
    // top-edge terms to the caller (fix_then_next).
    template <bool TOP = true>
    __device__ __forceinline__ void forward_step(const Halo<R> &h, bool edge_live)
    {
        constexpr int S2 = 2 % K;  // slot of node 2
        R w1 = (R)0, w3 = (R)0, w1b = (R)0;
        // bottom-edge jump: gather rows add it at node 2 (its weight jin, zero on other
        // threads); flux rows carry it on link 1, owned by node 1's thread (jl1)
        const R jin = (edge_live && n2) ? jlo : (R)0;
        const R src2 = old_at<S2, -2>(h);  // node 0 seen from node 2 (read before the update)
        const R jl1 = n1 ? jlo : (R)0;
        // K <= 2: link 1 also starts a thread (the one whose first node is node 2), which
        // computes its flux from the left halo and adds the same term (node 0 = l2)
        const R jl2 = (K <= 2 && n2 && !n1) ? jlo : (R)0;
        if (TOP && edge_live) top_values(h, w1, w3, w1b);
        if constexpr (!Mode::kFlux && Nodes<R, K>::kPaired) {
            // double-float rows on pairs (node q, node q+H): the compensated products
            // of two nodes per instruction; the prices are bitwise the scalar loop's
            constexpr int H = K / 2;
            df64x2 prev, last;
            prev.hi = make_float2(h.l1.hi, r.hi[H - 1].x);  // left neighbours of pair 0
            prev.lo = make_float2(h.l1.lo, r.lo[H - 1].x);
            last.hi = make_float2(r.hi[0].y, h.r1.hi);      // right neighbours of pair H-1
            last.lo = make_float2(r.lo[0].y, h.r1.lo);
#pragma unroll
            for (int q = 0; q < H; ++q) {
                const df64x2 cur = r.pair(q);
                df64x2 v = dot3x2(c0.pair(q), prev, c1.pair(q), cur, c2.pair(q), (q == H - 1) ? last : r.pair(q + 1));
                if (q == S2 % H) fma_lane<S2, H>(v, jin, src2);
                r.set_pair(q, v);
                prev = cur;
            }
        } else if constexpr (!Mode::kFlux) {
            R prev = h.l1;
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const R cur = r[s];
                const R nxt = (s < K - 1) ? r[s + 1] : h.r1;
                R v = gather3(c0[s], prev, c1[s], cur, c2[s], nxt);
                if (s == S2) v = fma(jin, src2, v);
                r[s] = v;
                prev = cur;
            }
        } else if constexpr (Nodes<R, K>::kPaired) {
            // the same operations on pairs (node p, node p+H); a - b as fma(b, -1, a)
            // rounds as the subtraction, so the results are the unpaired ones
            constexpr int H = K / 2;
            constexpr int S1 = 1 % K, Q1 = S1 % H;  // node 1's slot and pair
            const float2 m1 = make_float2(-1.f, -1.f);
            // bottom edge: node 0's jump up two rides on links 0 (its coefficient) and
            // 1 (this term, node 0's old value, added to link 1's flux)
            const float jq = edge_live ? jl1 * old_at<S1, -1>(h) : 0.f;
            const float2 jadd = (S1 >= H) ? make_float2(0.f, jq) : make_float2(jq, 0.f);
            // pair H-1's right neighbours are node H (pair 0's second) and the halo
            const float2 nl = make_float2(r.v[0].y, h.r1);
            const float2 e_last = __ffma2_rn(c0.pair(H - 1), r.v[H - 1],
                                             (edge_live && Q1 == H - 1) ? __ffma2_rn(c1.pair(H - 1), nl, jadd)
                                                                        : __fmul2_rn(c1.pair(H - 1), nl));
            const float lk = (K <= 2 && edge_live) ? fma(cd0, r[0], jl2 * h.l2) : cd0 * r[0];
            float2 ep = make_float2(fma(cl, h.l1, lk), e_last.x);  // links k0-1 and k0+H-1
#pragma unroll
            for (int q = 0; q < H; ++q) {
                const float2 e =
                    (q == H - 1) ? e_last
                                 : __ffma2_rn(c0.pair(q), r.v[q],
                                              (edge_live && q == Q1) ? __ffma2_rn(c1.pair(q), r.v[q + 1], jadd)
                                                                     : __fmul2_rn(c1.pair(q), r.v[q + 1]));
                const float2 v = __fadd2_rn(r.v[q], __ffma2_rn(e, m1, ep));
                r.v[q] = __ffma2_rn(c2.pair(q), v, v);
                ep = e;
            }
        } else {
            // net flux e_k = up_k r_k - down_{k+1} r_{k+1} across each link, computed
            // once and used by both ends (the row's sum is kept exactly)
            constexpr int S1 = 1 % K;  // node 1's slot
            const R jq = edge_live ? jl1 * old_at<S1, -1>(h) : (R)0;  // node 0's jump, on link 1
            R eprev = fma(cl, h.l1, (K <= 2 && edge_live) ? fma(cd0, r[0], jl2 * h.l2) : cd0 * r[0]);
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const R cur = r[s];
                const R nxt = (s < K - 1) ? r[s + 1] : h.r1;
                const R e = fma(c0[s], cur, (edge_live && s == S1) ? fma(c1[s], nxt, jq) : c1[s] * nxt);
                const R v = cur + (eprev - e);
                r[s] = fma(c2[s], v, v);
                eprev = e;
            }
        }
        if (TOP && edge_live) top_fixes<true>(w1, w3, w1b);
    }

    // One backward step, in place: r <- G o P r (flux: on the deviation from `base`).
    template <bool TOP = true>
    __device__ __forceinline__ void backward_step(const Halo<R> &h, bool edge_live, R base)
    {
        R w1 = (R)0, w3 = (R)0, w1b = (R)0;
        const R j0 = (edge_live && n0) ? jlo : (R)0;  // bottom-edge jump weight of node 0
        const R o2 = old_at<0, 2>(h);                 // node 2 seen from node 0 (read before the update)
        const R o1 = old_at<0, 1>(h);                 // node 1 seen from node 0
        if (TOP && edge_live) top_values(h, w1, w3, w1b);
        R prev = h.l1;
        if constexpr (!Mode::kFlux && Nodes<R, K>::kPaired) {
            constexpr int H = K / 2;
            df64x2 pv, last;
            pv.hi = make_float2(h.l1.hi, r.hi[H - 1].x);
            pv.lo = make_float2(h.l1.lo, r.lo[H - 1].x);
            last.hi = make_float2(r.hi[0].y, h.r1.hi);
            last.lo = make_float2(r.lo[0].y, h.r1.lo);
#pragma unroll
            for (int q = 0; q < H; ++q) {
                const df64x2 cur = r.pair(q);
                df64x2 v = dot3x2(c0.pair(q), (q == H - 1) ? last : r.pair(q + 1), c1.pair(q), cur, c2.pair(q), pv);
                if (q == 0) fma_lane<0, H>(v, j0, o2);
                r.set_pair(q, v);
                pv = cur;
            }
        } else if constexpr (!Mode::kFlux) {
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const R cur = r[s];
                const R nxt = (s < K - 1) ? r[s + 1] : h.r1;
                R v = gather3(c0[s], nxt, c1[s], cur, c2[s], prev);
                if (s == 0) v = fma(j0, o2, v);
                r[s] = v;
                prev = cur;
            }
        } else if constexpr (Nodes<R, K>::kPaired) {
            // paired as the forward step; -down of node p is c1 of node p-1
            constexpr int H = K / 2;
            const float2 m1 = make_float2(-1.f, -1.f);
            const float2 b2 = make_float2(base, base);
            const float2 d_last = __ffma2_rn(r.v[H - 1], m1, make_float2(r.v[0].y, h.r1));
            float2 dp = make_float2(r[0] - prev, d_last.x);  // differences at nodes k0-1 and k0+H-1
#pragma unroll
            for (int q = 0; q < H; ++q) {
                const float2 d = (q == H - 1) ? d_last : __ffma2_rn(r.v[q], m1, r.v[q + 1]);
                const float2 nd = (q == 0) ? make_float2(cd0, c1.pair(H - 1).x) : c1.pair(q - 1);
                float2 v = __ffma2_rn(nd, dp, __ffma2_rn(c0.pair(q), d, r.v[q]));
                if (edge_live && q == 0) v.x = fma(j0, o2 - o1, v.x);  // up two: r2 - r1 (r1 - r0 in up)
                r.v[q] = __ffma2_rn(c2.pair(q), __fadd2_rn(v, b2), v);
                dp = d;
            }
        } else {
            // differences D_k = r_{k+1} - r_k, each computed once:
            // v_k = r_k + up_k D_k - down_k D_{k-1}, as two fused multiply-adds
            R dprev = r[0] - prev;
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const R cur = r[s];
                const R nxt = (s < K - 1) ? r[s + 1] : h.r1;
                const R d = nxt - cur;
                const R ndown = (s == 0) ? cd0 : c1[s - 1];  // -down of this node
                R v = fma(ndown, dprev, fma(c0[s], d, cur));
                if (s == 0) v = fma(j0, o2 - o1, v);  // up two: r2 - r1 (r1 - r0 in up)
                r[s] = fma(c2[s], v + base, v);
                dprev = d;
            }
        }
        if (TOP && edge_live) top_fixes<false>(w1, w3, w1b);
    }

    __device__ __forceinline__ S partial_sum(int k0, int W) const
    {
        if constexpr (kPairScal<S>) {
            // float rows summed exactly: running TwoSums, their errors gathered
            float hi = 0.f, lo = 0.f;
#pragma unroll
            for (int s = 0; s < K; ++s) {
                if (k0 + s < W) {
                    float e;
                    hi = two_sum(hi, r[s], e);
                    lo = __fadd_rn(lo, e);
                }
            }
            return fast_two_sum(hi, lo);
        } else if constexpr (std::is_same<R, df64>::value) {
            // double-float rows summed in double-float (terms of one sign), one
            // conversion to the double scalar
            df64 acc = df64_make(0.f, 0.f);
#pragma unroll
            for (int s = 0; s < K; ++s)
                if (k0 + s < W) acc = acc + (R)r[s];
            return (S)acc;
        } else {
            S acc = (S)0;
#pragma unroll
            for (int s = 0; s < K; ++s)
                if (k0 + s < W) acc += (S)(R)r[s];
            return acc;
        }
    }

    // Payoff at the maturity step: value = kappa * (base + row).
    __device__ __forceinline__ void payoff(S kappa, R base, double X, int type)
    {
        if constexpr (kPairScal<S>) {
            // Through the thread's shared-memory scratch (16 floats, stride 32): the
            // row out, one rolled loop over the nodes, the row back; the code is that
            // of one node whatever K (unrolled over K, the per-node arithmetic cost
            // the step loops of other warps their instruction-cache lines: mixed rows
            // ran 3-12% slower than float rows beside K = 32 tasks)
            extern __shared__ float payoff_scratch[];
            float *scr = payoff_scratch + (threadIdx.x >> 5) * (32 * kPayoffScratch) + (threadIdx.x & 31);
            const df64 x(X);
            constexpr int HALF = K < kPayoffScratch ? K : kPayoffScratch;
#pragma unroll
            for (int h0 = 0; h0 < K; h0 += HALF) {
#pragma unroll
                for (int s = 0; s < HALF; ++s) scr[s * 32] = r[h0 + s];
#pragma unroll 1
                for (int s = 0; s < HALF; ++s) scr[s * 32] = payoff_value(scr[s * 32], base, kappa, x, type);
#pragma unroll
                for (int s = 0; s < HALF; ++s) r[h0 + s] = scr[s * 32];
            }
        } else {
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const S c = kappa * ((S)base + (S)(R)r[s]);
                const S x = (S)X;
                const S p = (type == 1) ? (x - c) : (c - x);
                r[s] = (R)(p < (S)0 ? (S)0 : p);
            }
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

// Halo within a warp segment of L lanes holding one tree.  The shuffles use width
// L, so a lane never reads another tree: at the segment ends it gets its own
// values back, which only ever meet a zero coefficient (the tree's outer nodes
// branch nowhere outward) or feed nodes outside the active cone.  The second
// neighbours are needed only while the edge jumps are live.
template <typename R, int K>
__device__ __forceinline__ Halo<R> exchange_warp(const Nodes<R, K> &r, int L, bool two)
{
    Halo<R> h;
    if constexpr (K >= 2) {
        h.l1 = shfl_up(r[K - 1], 1, L);
        h.r1 = shfl_down(r[0], 1, L);
        h.l2 = two ? shfl_up(r[K - 2], 1, L) : (R)0;
        h.r2 = two ? shfl_down(r[1], 1, L) : (R)0;
    } else {
        h.l1 = shfl_up(r[0], 1, L);
        h.r1 = shfl_down(r[0], 1, L);
        h.l2 = two ? shfl_up(r[0], 2, L) : (R)0;
        h.r2 = two ? shfl_down(r[0], 2, L) : (R)0;
    }
    return h;
}

// Halo across a warp group: shuffles inside each warp, the first and last two
// nodes of every warp through shared memory (double buffered, so one barrier per
// step is enough).
template <typename R, int K>
__device__ __forceinline__ Halo<R> exchange_block(const Nodes<R, K> &r, R *sh, int parity, const Group &gr)
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
    Halo<R> h = exchange_warp<R, K>(r, 32, true);
    const bool hasl = warp > w0, hasr = warp + 1 < w1;
    if constexpr (K >= 2) {
        if (lane == 0) {
            h.l1 = hasl ? buf[(warp - 1) * 4 + 3] : (R)0;
            h.l2 = hasl ? buf[(warp - 1) * 4 + 2] : (R)0;
        }
        if (lane == 31) {
            h.r1 = hasr ? buf[(warp + 1) * 4 + 0] : (R)0;
            h.r2 = hasr ? buf[(warp + 1) * 4 + 1] : (R)0;
        }
    } else {
        if (lane == 0) {
            h.l1 = hasl ? buf[(warp - 1) * 4 + 3] : (R)0;
            h.l2 = hasl ? buf[(warp - 1) * 4 + 2] : (R)0;
        }
        if (lane == 1) h.l2 = hasl ? buf[(warp - 1) * 4 + 3] : (R)0;
        if (lane == 31) {
            h.r1 = hasr ? buf[(warp + 1) * 4 + 0] : (R)0;
            h.r2 = hasr ? buf[(warp + 1) * 4 + 1] : (R)0;
        }
        if (lane == 30) h.r2 = hasr ? buf[(warp + 1) * 4 + 0] : (R)0;
    }
    return h;
}

// Scalars of one tree after its forward sweep.
template <typename S>
struct Scales {
    S kappa;  // s_n / s_m, applied at the maturity step
    S final;  // s_m (payoff) or s_n (bond only)
};

template <typename S, bool kSizingDisc>
__device__ __forceinline__ Scales<S> tree_scales(const Tree &t, S sum_m1, S sum_n1, const EngineParams &p)
{
    Scales<S> sc;
    if constexpr (kSizingDisc && std::is_same<S, double>::value) {
        // double scalars, discount factors from the sizing pass (double-float rows:
        // no curve lookups or exponentials on the FP64 pipe here)
        const float4 d = t.idx >= 0 ? p.s.trees[t.idx].disc : make_float4(1.f, 0.f, 1.f, 0.f);
        const double sn = (double)df64_make(d.x, d.y) / sum_n1;
        if (t.m >= 0 && t.m < t.n) {
            const double sm = (t.m >= 1) ? (double)df64_make(d.z, d.w) / sum_m1 : 1.0;
            sc.kappa = sn / sm;
            sc.final = sm;
        } else {
            sc.kappa = 1.0;
            sc.final = sn;
        }
    } else if constexpr (kPairScal<S>) {
        // discount factors from the sizing pass (read here, not with the tree
        // record, so they hold no registers through the forward sweep)
        const float4 d = t.idx >= 0 ? p.s.trees[t.idx].disc : make_float4(1.f, 0.f, 1.f, 0.f);
        const df64 sn = df64_make(d.x, d.y) / sum_n1;
        if (t.m >= 0 && t.m < t.n) {
            const df64 sm = (t.m >= 1) ? df64_make(d.z, d.w) / sum_m1 : df64_make(1.f, 0.f);
            sc.kappa = sn / sm;
            sc.final = sm;
        } else {
            sc.kappa = df64_make(1.f, 0.f);
            sc.final = sn;
        }
    } else {
        const DevYield &yc = p.yc;
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
    }
    return sc;
}

__device__ __forceinline__ bool pays_at(const Tree &t) { return t.m >= 0 && t.m < t.n; }

// ---------------------------------------------------------------------------
// Small trees: 32/L trees per warp, L lanes x K nodes each.
// ---------------------------------------------------------------------------
template <class Mode, int K>
__device__ void price_warp_task(const EngineParams &p, const WarpTask &task, float2 *wide)
{
    typedef typename Mode::Row R;
    typedef typename Mode::Scal S;
    constexpr unsigned NONE = 0x7fffffffu;
    const int lane = threadIdx.x & 31;
    const int L = cls_L(task.cls & kClsMask);
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

    // ---- forward sweep: rows 1 .. n-1; the sums of rows m-1 and n-1 are kept.
    // Rows of trees that are done keep being updated (their segment is isolated by
    // the width-L shuffles), so the step loop carries no per-tree predicates.
    sl.bind_coefficients(wide, lane);
    sl.setup_forward(t, k0);
    sl.ts = (task.cls >> kTsShift) & 31;  // the warp's common top-edge slot
    // While the edge jumps are live the second neighbours (l2, r2) are read only
    // when node W-1 sits in slot 0 or 1 (node W-3 in the previous lane) or K < 3;
    // otherwise float rows skip the step's two extra shuffles (double-float rows
    // measured 1-2% slower without them, so they keep them).
    const bool wide_halo = K < 3 || sl.ts < 2 || !Mode::kFlux;
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
        if constexpr (!Mode::kFlux) {
            // 64-bit rows (FP64-pipe-bound or 31 float operations a node): the
            // top-edge lookups cost little beside the row update
            for (; i < stop; ++i) {
                const bool live = i >= e_f;
                const Halo<R> h = exchange_warp<R, K>(sl.r, L, live && wide_halo);
                sl.forward_step(h, live);
            }
        } else {
            for (; i < stop && i < e_f; ++i) {
                const Halo<R> h = exchange_warp<R, K>(sl.r, L, false);
                sl.forward_step(h, false);
            }
            if (i < stop) {
                // edge jumps live: one switch on the top-edge slot per step (two would
                // cost the issue-bound float rows about a fifth of their time)
                auto xch = [&](bool two) { return exchange_warp<R, K>(sl.r, L, two); };
                Halo<R> h = xch(wide_halo);
                R w1 = (R)0, w3 = (R)0, w1b = (R)0;
                sl.top_values(h, w1, w3, w1b);
                for (; i < stop; ++i) {
                    sl.template forward_step<false>(h, true);
                    if (i + 1 < stop) sl.template fix_then_next<true>(w1, w3, w1b, h, xch);
                    else sl.template top_fixes<true>(w1, w3, w1b);
                }
            }
        }
        if (ev <= fsteps) {
            S acc = sl.partial_sum(k0, W);
            for (int off = 1; off < L; off <<= 1) acc += shfl_xor(acc, off);
            if (rm == ev) sum_m1 = acc;
            if (rn == ev) sum_n1 = acc;
        }
    }
    const Scales<S> sc = tree_scales<S, Mode::kSizingDiscounts>(t, sum_m1, sum_n1, p);

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
        auto after_step = [&](int row) {
            if (row >= n_min && row >= t.n) {
#pragma unroll
                for (int s = 0; s < K; ++s) sl.r[s] = (k0 + s < W) ? face : (R)0;
            }
            if (row == pm && pays && t.m == row) {
                sl.payoff(sc.kappa, base, t.X, t.type);
                base = (R)0;
            }
        };
        if constexpr (!Mode::kFlux) {
            for (; i >= lo; --i) {
                const bool live = i >= e_b;
                const Halo<R> h = exchange_warp<R, K>(sl.r, L, live && wide_halo);
                sl.backward_step(h, live, base);
                after_step(i);
            }
        } else {
            if (i >= lo && i >= e_b) {
                // edge jumps live: one switch on the top-edge slot per step, except where
                // rows are reset or paid off between the fixes and the next exchange
                auto xch = [&](bool two) { return exchange_warp<R, K>(sl.r, L, two); };
                Halo<R> h = xch(wide_halo);
                R w1 = (R)0, w3 = (R)0, w1b = (R)0;
                sl.top_values(h, w1, w3, w1b);
                for (; i >= lo && i >= e_b; --i) {
                    sl.template backward_step<false>(h, true, base);
                    const bool more = i - 1 >= lo && i - 1 >= e_b;
                    if (more && i < n_min && i != pm) {
                        sl.template fix_then_next<false>(w1, w3, w1b, h, xch);
                    } else {
                        sl.template top_fixes<false>(w1, w3, w1b);
                        after_step(i);
                        if (more) {
                            h = xch(wide_halo);
                            sl.top_values(h, w1, w3, w1b);
                        }
                    }
                }
            }
            for (; i >= lo; --i) {
                const Halo<R> h = exchange_warp<R, K>(sl.r, L, false);
                sl.backward_step(h, false, base);
                after_step(i);
            }
        }
    }

    // ---- price at the root node
    const int owner = t.jc / K, slot = t.jc - owner * K;
    const R v = sl.pick(slot);
    if (valid && lis == owner) {
        double price;
        if (t.n <= 0) price = 100.0;
        else if (pays_at(t)) price = (double)(sc.final * to_scal<S>(v));
        else price = (double)(sc.final * scal_sum<S>(base, v));
        p.out[t.idx] = price;
    }
}

// K = 32 tasks in a function of their own: inlined into the kernel, their code
// changed the register allocation of the K = 16 path (mixed rows 4% slower even
// with no K = 32 task in the batch).
template <class Mode>
__device__ __noinline__ void price_wide_task(const EngineParams &p, const WarpTask &task, float2 *wide)
{
    price_warp_task<Mode, kWideK>(p, task, wide);
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
    int parity = 0;

    sl.setup_forward(t, k0);
    S sum_m1 = (S)1, sum_n1 = (S)1;
    const int fsteps = t.n > 1 ? t.n - 1 : 0;
    for (int i = 0; i < fsteps; ++i) {
        const Halo<R> h = exchange_block<R, K>(sl.r, sh_x, parity, gr);
        parity ^= 1;
        // rows outside the cone of row i+1 stay zero: skip whole warps there
        const int reach = (i + 1 < jc) ? i + 1 : jc;
        const bool active = wk1 > jc - reach && wk0 <= jc + reach && wk0 < W;
        if (active) sl.forward_step(h, t.edges && i >= t.jmax);
        const int row = i + 1;
        if (row == t.m - 1 || row == t.n - 1) {
            S acc = sl.partial_sum(k0, W);
            for (int off = 16; off > 0; off >>= 1) acc += shfl_xor(acc, off);
            if (lane == 0) sh_red[aw0 + warp] = acc;
            tree_barrier(gr.bar, gr.nthreads);
            S tot = (S)0;
            for (int w = 0; w < nw; ++w) tot += sh_red[aw0 + w];
            tree_barrier(gr.bar, gr.nthreads);
            if (row == t.m - 1) sum_m1 = tot;
            if (row == t.n - 1) sum_n1 = tot;
        }
    }
    const Scales<S> sc = tree_scales<S, Mode::kSizingDiscounts>(t, sum_m1, sum_n1, p);

    sl.setup_backward(t, k0);
    R base = Mode::kFlux ? (R)100 : (R)0;
    for (int i = t.n - 1; i >= 0; --i) {
        const Halo<R> h = exchange_block<R, K>(sl.r, sh_x, parity, gr);
        parity ^= 1;
        const int reach = (i < t.jmax) ? i : t.jmax;
        const bool active = wk1 > jc - reach && wk0 <= jc + reach && wk0 < W;
        if (active) sl.backward_step(h, t.edges && i >= t.jmax, base);
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
        else if (pays_at(t)) price = (double)(sc.final * to_scal<S>(v));
        else price = (double)(sc.final * scal_sum<S>(base, v));
        p.out[t.idx] = price;
    }
}

// K = nodes per thread for a tree on group `gr` (width <= 8 * gr.nthreads, or
// 16 * gr.nthreads for float rows).  More nodes per thread spread the step's fixed
// cost (halo exchange, barrier, loop control) over more nodes.
template <class Mode>
__device__ __forceinline__ void dispatch_block_tree(const EngineParams &p, const Tree &t, const Group &gr,
                                                    typename Mode::Row *sh_x, typename Mode::Scal *sh_red)
{
    // K rounded up to 1, 2, 4, 8 (12, 16) (warps left past the width skip their steps)
    const int K = (t.width + gr.nthreads - 1) / gr.nthreads;
    if (K <= 1) price_block_tree<Mode, 1>(p, t, gr, sh_x, sh_red);
    else if (K <= 2) price_block_tree<Mode, 2>(p, t, gr, sh_x, sh_red);
    else if (K <= 4) price_block_tree<Mode, 4>(p, t, gr, sh_x, sh_red);
    else if (K <= 8 || !Mode::kFlux) price_block_tree<Mode, 8>(p, t, gr, sh_x, sh_red);
    else if constexpr (Mode::kFlux) {
        if (K <= 12) price_block_tree<Mode, 12>(p, t, gr, sh_x, sh_red);
        else price_block_tree<Mode, 16>(p, t, gr, sh_x, sh_red);
    }
}

template <class Mode>
__global__ void __launch_bounds__(kPricingThreads, 1) price_kernel(EngineParams p)
{
    typedef typename Mode::Row R;
    typedef typename Mode::Scal S;
    __shared__ R sh_x[2 * 32 * 4];
    __shared__ S sh_red[32];
    __shared__ int sh_task[16];  // one per group of every group tier
    unsigned long long t_start = 0;
    if (p.record_busy && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
    // dynamic shared memory of this launch: mixed rows need their payoff scratch
    // (a launch without it does no work and is reported), K = 32 tasks their
    // coefficients (checked per task below)
    unsigned dyn_bytes;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn_bytes));
    if constexpr (Mode::kScratchPayoff) {
        if (dyn_bytes < (unsigned)kScratchSmemBytes) {
            if (threadIdx.x == 0) atomicExch(&p.s.status->wide_smem_missing, 1);
            return;
        }
    }

    // Group tiers, heaviest first: tier t prices one tree per group of 512 >> t
    // threads.  Group g of tier t uses named barrier and task slot 2^t - 1 + g
    // (0: the whole block; 1-2: halves; 3-6: quarters; 7-14: eighths), so groups of
    // different tiers never share one while some threads are still in the earlier
    // tier.
    for (int tier = 0; tier < kGroupTiers; ++tier) {
        const int count = p.s.status->tier_count[tier];
        if (count == 0) continue;
        const int start = p.s.status->tier_start[tier];
        const int gsize = kPricingThreads >> tier;
        const int g = (int)threadIdx.x / gsize;
        const int slot = (1 << tier) - 1 + g;
        const Group gr{g * gsize, gsize, slot};
        for (;;) {
            if ((int)threadIdx.x == gr.base) sh_task[slot] = atomicAdd(&p.s.status->tier_counter[tier], 1);
            tree_barrier(gr.bar, gr.nthreads);
            const int tsk = sh_task[slot];
            tree_barrier(gr.bar, gr.nthreads);
            if (tsk >= count) break;
            const Tree t = p.s.trees[p.s.order[start + tsk]];
            dispatch_block_tree<Mode>(p, t, gr, sh_x, sh_red);
            tree_barrier(gr.bar, gr.nthreads);  // shared buffers are reused by the next tree
        }
    }

    // Warp tier: warp tasks, each warp on its own.
    const int n_tasks = p.s.status->n_warp_tasks;
    const int lane = threadIdx.x & 31;
    // this warp's coefficient region for K = 32 tasks (float rows: the kernel is
    // launched with kWideSmemBytes of dynamic shared memory)
    extern __shared__ float2 wide_coef[];
    float2 *wide = wide_coef + (Mode::kScratchPayoff ? kScratchSmemBytes / 8 : 0) + (threadIdx.x >> 5) * kWideWarpFloat2;
    // a K = 32 task runs only if this launch has its coefficient space (a task in a
    // launch without it is skipped and reported, never run out of bounds)
    const bool wide_ok = dyn_bytes >= (unsigned)((Mode::kScratchPayoff ? kScratchSmemBytes : 0) + kWideSmemBytes);
    for (;;) {
        int tsk = 0;
        if (lane == 0) tsk = atomicAdd(&p.s.status->warp_counter, 1);
        tsk = __shfl_sync(FULL, tsk, 0);
        if (tsk >= n_tasks) break;
        const WarpTask wt = p.s.tasks[tsk];
        switch (cls_K(wt.cls & kClsMask)) {
            case 1: price_warp_task<Mode, 1>(p, wt, wide); break;
            case 2: price_warp_task<Mode, 2>(p, wt, wide); break;
            case 3: price_warp_task<Mode, 3>(p, wt, wide); break;
            case 4: price_warp_task<Mode, 4>(p, wt, wide); break;
            case 5: price_warp_task<Mode, 5>(p, wt, wide); break;
            case 6: price_warp_task<Mode, 6>(p, wt, wide); break;
            case 7: price_warp_task<Mode, 7>(p, wt, wide); break;
            case 8: price_warp_task<Mode, 8>(p, wt, wide); break;
            default:
                if constexpr (Mode::kFlux) {
                    const int k = cls_K(wt.cls & kClsMask);
                    if (k == 12) price_warp_task<Mode, 12>(p, wt, wide);
                    else if (k == 16 || !Mode::kWide) price_warp_task<Mode, 16>(p, wt, wide);
                    else if constexpr (Mode::kWide) {
                        if (wide_ok) price_wide_task<Mode>(p, wt, wide);
                        else if (lane == 0) atomicExch(&p.s.status->wide_smem_missing, 1);
                    }
                }
                break;
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

int resolve_k_mask(int mode, int requested, int *max_k)
{
    const bool dbl = mode == MODE_BATCHED_FP64 || mode == MODE_BATCHED_DF64;  // 64-bit rows: K <= 8
    const int allowed = dbl ? kKMaskFP64 : kKMaskAll;
    int m = requested & allowed;
    // defaults: every K for the FP64-pipe-bound double rows; the issue-bound
    // double-float rows, like float rows, do better with fewer K (less code)
    if (m == 0) m = mode == MODE_BATCHED_FP64 ? kKMaskFP64 : (mode == MODE_BATCHED_DF64 ? kKMaskFP64Alt : kKMaskFloat);
    int mk = 1;
    for (int q = 0; q < kNumK; ++q)
        if ((m >> q) & 1) mk = kWarpK[q];
    if (max_k) *max_k = mk;
    return m;
}

int run_k_mask(int mode, int requested, int big_threshold, int *max_k)
{
    int m = resolve_k_mask(mode, requested, max_k);
    const int k32 = 1 << (kNumK - 1);
    if ((m & k32) && (m & ~k32) && big_threshold <= 512) {
        m &= ~k32;
        int mk = 1;
        for (int q = 0; q < kNumK; ++q)
            if ((m >> q) & 1) mk = kWarpK[q];
        if (max_k) *max_k = mk;
    }
    return m;
}

int warp_layout(int width, int k_mask, int *K, int *L)
{
    const int c = pick_warp_class(width, k_mask);
    if (c < 0) return -1;
    *K = kWarpK[c / kNumL];
    *L = 1 << (c % kNumL);
    return 0;
}

int pricing_smem_bytes(int mode, int k_mask)
{
    const bool wide = (k_mask >> (kNumK - 1)) & 1;
    if (mode == MODE_BATCHED_FP32) return wide ? kWideSmemBytes : 0;
    if (mode == MODE_BATCHED_MIXED) return kScratchSmemBytes + (wide ? kWideSmemBytes : 0);
    return 0;
}

int sizing_launches() { return 4; }

cudaError_t launch_sizing(const EngineParams &p, cudaStream_t stream)
{
    const int n = p.opt.n;
    cudaError_t e;
    reset_kernel<<<48, 512, 0, stream>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (n > 0) {
        // 64-thread blocks: the FP64-bound sizing of a 30,000-option batch reaches
        // every SM (256-thread blocks left a quarter of them idle)
        size_kernel<<<(n + 63) / 64, 64, 0, stream>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    scan_kernel<<<kScanBlocks, kScanBlock, 0, stream>>>(p);
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
        case MODE_BATCHED_FP32:
            // the K = 32 coefficient space only when the run's K mask allows K = 32
            // (otherwise the L1 keeps that shared-memory carve-out)
            price_kernel<ModeF32><<<grid, kPricingThreads, pricing_smem_bytes(mode, p.warp_k_mask), stream>>>(p);
            break;
        case MODE_BATCHED_MIXED:
            price_kernel<ModeMix><<<grid, kPricingThreads, pricing_smem_bytes(mode, p.warp_k_mask), stream>>>(p);
            break;
        case MODE_BATCHED_DF64: price_kernel<ModeDF64><<<grid, kPricingThreads, 0, stream>>>(p); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Float rows' kernels take kWideSmemBytes of dynamic shared memory (K = 32
// coefficients); the attribute is set once per device, before any launch or
// occupancy query (every launch path asks for the occupancy first).  Setting it
// twice from two threads is harmless.
static bool wide_smem_enabled()
{
    static std::atomic<int> done[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (done[dev].load()) return true;
    const bool ok =
        cudaFuncSetAttribute(price_kernel<ModeF32>, cudaFuncAttributeMaxDynamicSharedMemorySize, kWideSmemBytes) ==
            cudaSuccess &&
        cudaFuncSetAttribute(price_kernel<ModeMix>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kScratchSmemBytes + kWideSmemBytes) == cudaSuccess;
    if (ok) done[dev].store(1);
    return ok;
}

int pricing_blocks_per_sm(int mode)
{
    const int block_threads = kPricingThreads;
    int nb = 0;
    cudaError_t e = cudaErrorInvalidValue;
    if ((mode == MODE_BATCHED_FP32 || mode == MODE_BATCHED_MIXED) && !wide_smem_enabled()) {
        cudaGetLastError();
        return 0;
    }
    switch (mode) {
        case MODE_BATCHED_FP64: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, price_kernel<ModeF64>, block_threads, 0); break;
        case MODE_BATCHED_FP32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, price_kernel<ModeF32>, block_threads, kWideSmemBytes); break;
        case MODE_BATCHED_MIXED:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, price_kernel<ModeMix>, block_threads,
                                                              kScratchSmemBytes + kWideSmemBytes);
            break;
        case MODE_BATCHED_DF64: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, price_kernel<ModeDF64>, block_threads, 0); break;
        default: break;
    }
    return e == cudaSuccess ? nb : 0;
}

}  // namespace hwt
