// Internal structures shared by the batched engine, the plain kernel and the
// C-ABI host code.  Not part of the public interface (include/hwtree.h is).
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

namespace hwt {

// Precision policy of a pricing run.
enum Mode : int {
    MODE_PLAIN_FP64 = 0,    // one block per option, per-step alpha fit as the reference does
    MODE_BATCHED_FP64 = 1,  // binned persistent engine, double rows
    MODE_BATCHED_FP32 = 2,  // float rows, float sums and scales
    MODE_BATCHED_MIXED = 3, // float rows; sums, scales, payoff and final discount in double precision
    MODE_BATCHED_DF64 = 4,  // double-float rows on the FP32 pipes, double sums and scales
};
constexpr int kNumModes = 5;

// Device copy of the option records (SoA, common/Options.hpp:48-58 with real=double).
struct DevOptions {
    int32_t n;
    const double *strike, *bond_maturity, *option_maturity;
    const uint16_t *term_unit, *term_steps;
    const double *a, *sigma;
    const int8_t *type;
};

// Device copy of the yield curve (common/Yield.hpp:14-40): zero rates and days.
struct DevYield {
    int32_t n;
    const double *rate;
    const float *rate_f;
    const int32_t *day;
};

// One option's tree as the sizing pass leaves it for the pricing pass.
struct Tree {
    double dt, dr, M, X;
    float4 disc;        // P(n dt), P(m dt) as double-float pairs (hi, lo, hi, lo), when sizing is asked for them
    int32_t idx;        // position in the caller's arrays
    int32_t jmax, n, m; // edge index, height, maturity step
    int32_t jc, width;  // half-width and width of the nodes that can carry value
    uint16_t term_unit;
    int8_t type;        // 0 = CALL, 1 = PUT
    int8_t edges;       // 1 when the +-jmax edge branching is reached
};

// A group of small trees priced together by one warp: `count` trees of the same
// warp class starting at `start` in the sorted order.
struct WarpTask {
    int32_t start;
    int16_t count;
    int16_t cls;
};

// Warp classes: L lanes per tree (power of two), K nodes per lane; L*K >= width.
// class = index of K in kWarpK * kNumL + log2(L); FP64 rows stop at K = 8; K = 32
// (float rows only, trees of 513..1024 nodes) keeps its coefficients in shared
// memory.  A call may restrict the K values used with a mask over kWarpK's indices.
constexpr int kWarpK[] = {1, 2, 3, 4, 5, 6, 7, 8, 12, 16, 32};
constexpr int kNumK = 11;
constexpr int kKMaskFP64 = 0xFF;      // default K set of double rows: 1 .. 8
constexpr int kKMaskFP64Alt = 0xAF;   // autotuner's alternative: 1, 2, 3, 4, 6, 8
constexpr int kKMaskFloat = 0x68B;    // default K set of float rows: 1, 2, 4, 8, 16, 32
constexpr int kKMaskFloatAlt = 0x7AF; // autotuner's alternative: 1, 2, 3, 4, 6, 8, 12, 16, 32
constexpr int kKMaskAll = 0x7FF;
constexpr int kNumL = 6;                       // L = 1, 2, 4, 8, 16, 32
constexpr int kClsMask = 127;                  // class word: K and L indices in bits 0-6,
constexpr int kTsShift = 7;                    // the top edge's slot (0..31) from bit 7
constexpr int kMaxWarpWidth = 32 * 32;         // wider trees go to warp groups or whole blocks
constexpr int kWideK = 32;                     // warp tasks of this K read coefficients from shared memory
constexpr int kWideWarpFloat2 = 3 * (kWideK / 2) * 32;  // float2 per warp: up, -down, g pairs
constexpr int kWideSmemBytes = (512 / 32) * kWideWarpFloat2 * 8;  // 192 KB per 512-thread block
// Mixed rows compute the payoff in a rolled loop through 16 floats of shared-memory
// scratch per thread (32 KB per block), ahead of the K = 32 coefficients.
constexpr int kPayoffScratch = 16;
constexpr int kScratchSmemBytes = 512 * kPayoffScratch * 4;
constexpr int kMaxBlockK = 8;                  // nodes per thread for whole-block trees
constexpr int kMaxGroupKFloat = 16;            // nodes per thread for warp-group trees, float rows
constexpr int kPricingThreads = 512;           // threads of every pricing block
constexpr int kMaxTreeWidth = kMaxBlockK * kPricingThreads;  // widest tree accepted

// Sort keys.  Group tiers t = 0..3 (trees priced by a group of 512 >> t threads:
// the whole block, halves, quarters, eighths): bins [t kBuckets, (t+1) kBuckets),
// by work.  Warp tier (small trees packed into warp tasks): kWarpTier kBuckets +
// height bucket * kClassSlots + class slot, one slot per warp class (K, L) and
// slot ts < K of the top edge node: 6 (L values) x (1+2+...+8+12+16+32) = 576 slots.
// Descending inside a tier.
constexpr int kGroupTiers = 4;
constexpr int kWarpTier = kGroupTiers;
constexpr int kBuckets = 128;
constexpr int kClassSlots = kNumL * 96;
constexpr int kKeyBinsUsed = kWarpTier * kBuckets + kBuckets * kClassSlots;  // keys are below this
constexpr int kScanBlock = 1024;  // bins per block of the histogram scan
constexpr int kScanBlocks = (kKeyBinsUsed + kScanBlock - 1) / kScanBlock;
// bin_start / task_start hold the starts within each scan block for bins below
// kScanOffsets and each scan block's offset at kScanOffsets + block
constexpr int kScanOffsets = kScanBlocks * kScanBlock;
constexpr int kKeyBins = kScanOffsets + (kScanBlocks + 63) / 64 * 64;  // counters per array
static_assert(kScanBlocks <= kScanBlock && kKeyBins % 4 == 0 && kClassSlots % kNumL == 0, "bin layout");

// Per-run status written by the device (read back after each run).
struct RunStatus {
    unsigned long long first_bad; // (index << 32) | reason of the lowest rejected option; all ones if none
    unsigned long long nodes;     // active nodes of one pass, summed over valid options
    int32_t bad_count;            // options rejected by validation
    int32_t tier_start[kGroupTiers];    // first sorted position of each group tier
    int32_t tier_count[kGroupTiers];    // trees priced by groups of 512 >> t threads
    int32_t tier_counter[kGroupTiers];  // work-queue heads of the group tiers
    int32_t n_warp_tasks;         // warp tier: warp tasks
    int32_t warp_counter;
    int32_t max_width;            // widest / tallest valid tree
    int32_t max_height;
    int32_t scan_blocks_done;     // histogram scan blocks finished (the last one adds the offsets)
    int32_t wide_smem_missing;    // a launch lacked the shared memory its work needs (work skipped)
};

struct Scratch {
    Tree *trees;            // [cap]
    int32_t *keys;          // [cap]
    int32_t *order;         // [cap] sorted position -> option
    WarpTask *tasks;        // [cap]
    int32_t *hist;          // [kKeyBins], followed in memory by fill
    int32_t *fill;          // [kKeyBins]
    int32_t *bin_start;     // [kKeyBins]
    int32_t *task_start;    // [kKeyBins]
    RunStatus *status;      // [1]
    unsigned long long *cta_busy; // [max grid] per-CTA busy cycles (tail imbalance)
};

struct EngineParams {
    DevOptions opt;
    DevYield yc;
    Scratch s;
    double *out;
    int32_t max_width;
    int32_t group_threads;  // smallest warp group (64..512 threads) a wide tree is given
    int32_t big_threshold;  // widths above this go to warp groups or whole blocks
    int32_t max_warp_k;     // largest K of a warp task (8 for double rows, 16 for float)
    int32_t warp_k_mask;    // K values warp tasks may use (bits over kWarpK's indices)
    int32_t max_group_k;    // largest K of a warp-group tree: 8 double rows, 16 float
    int32_t sort;           // HWT_SORT_* order inside the tiers (0 / '-': heaviest first)
    int32_t record_busy;
    int32_t curve_discounts;  // sizing stores Tree::disc (modes with double-float scalars)
};

// Resolves a requested K mask for `mode` (0 = the mode's default) and the largest
// K it allows.
int resolve_k_mask(int mode, int requested, int *max_k);
// The K mask a run uses: the resolved one without K = 32 when the widest warp-task
// tree is at most 512 nodes and another K is allowed (K = 32 then has no tree to
// take, and the launch needs no coefficient space in shared memory).
int run_k_mask(int mode, int requested, int big_threshold, int *max_k);
// Warp-task layout of a tree of `width` nodes under K mask `k_mask`: nodes per lane
// and lanes (the sizing kernel's choice); -1 if no allowed K fits.
int warp_layout(int width, int k_mask, int *K, int *L);
// Dynamic shared memory a pricing launch of `mode` with this K mask needs.
int pricing_smem_bytes(int mode, int k_mask);

// Launchers (hwt_batched.cu / hwt_plain.cu).  All enqueue on `stream`; none syncs.
cudaError_t launch_sizing(const EngineParams &p, cudaStream_t stream);
cudaError_t launch_pricing(const EngineParams &p, int mode, int grid, cudaStream_t stream);
int pricing_blocks_per_sm(int mode);
cudaError_t launch_plain(const EngineParams &p, int max_width, int max_height, cudaStream_t stream);
size_t plain_smem_bytes(int max_width, int max_height);
int sizing_launches();

}  // namespace hwt
