/*
 * hwtree.h - C ABI of the GB300 Hull-White trinomial-tree batch pricer.
 *
 * Drop-in boundary for the batch pricing path of the reference project
 * (MartinMetaksov/diku.OptionsPricing).  The reference has no FFI; its pricing
 * entry points are C++ calls:
 *   seq::computeOptions(const Options&, const Yield&, std::vector<real>&)
 *       seq/Seq.hpp:181-190
 *   cuda::option::KernelRunBase::run(const Options&, const Yield&,
 *       std::vector<real>&, int blockSize, SortType, bool isTest)
 *       cuda-option/Kernel.cuh:303-314
 *   cuda::multi::KernelRunBase::run(...)  cuda-multi/Kernel.cuh:375-404
 * Each is replaced by hwt_price() below; the records are the reference's SoA
 * option and yield arrays (common/Options.hpp:48-58, common/Yield.hpp:14-18)
 * with real = double.  include/hwtree.hpp wraps this ABI in the reference's own
 * C++ record and call shapes.
 *
 * Plain C types only; no exceptions or process exits cross this boundary.  All
 * functions return HWT_OK (0) or a negative HWT_E* code; hwt_last_error() gives
 * the message.  One context per host thread; calls on one context are
 * serialised by the caller.
 */
#ifndef HWTREE_H
#define HWTREE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: hwt_train_config, hwt_train_stats and hwt_surrogate_stats grew (hard-sample
 * mining, held-out violations, options copy time); hwt_struct_size added. */
#define HWT_ABI_VERSION 2

/* Status codes. */
#define HWT_OK 0
#define HWT_EINVAL (-1)      /* bad argument or option record (a <= 0, zero steps, bad type, too wide) */
#define HWT_ECUDA (-2)       /* CUDA runtime error */
#define HWT_ENOMEM (-3)      /* device or pinned host allocation failed */
#define HWT_EUNSUPPORTED (-4)/* mode not available for these inputs */
#define HWT_ENODEV (-5)      /* no CUDA device */
#define HWT_ETIMEOUT (-6)    /* a bounded device-side wait ran out; the kernel gave up and the
                                context stays usable */

/* Pricing modes.  The reference selects precision at compile time
 * (common/Real.hpp:9-21); here it is a run-time argument. */
#define HWT_PLAIN_FP64 0     /* one block per option, reference step structure, double */
#define HWT_BATCHED_FP64 1   /* binned persistent engine, double */
#define HWT_BATCHED_FP32 2   /* binned persistent engine, float throughout */
#define HWT_BATCHED_MIXED 3  /* float rows; alpha-fit sums, scales, payoff, discount in double precision */
#define HWT_BATCHED_DF64 4   /* double-float rows (hi + lo floats, ~48 bits) on the FP32 pipes,
                                double sums, scales, payoff, discount; within 1e-10 relative + 1e-12
                                absolute of FP64 (the absolute floor matters only at prices near 0) */

/* Sort orders of the reference's -s flag (common/Options.hpp:15-22).  They set the
 * order in which the engine schedules trees inside each of its tiers (whole-block
 * trees, warp-group trees, warp tasks); results never depend on them.  NONE (and
 * 0) is the engine's own order: heaviest work first, warp tasks by class and
 * height.  INPUT keeps the arrival order inside each tier and class (no binning by
 * size), the baseline for A/B runs against the sorted orders. */
#define HWT_SORT_NONE '-'
#define HWT_SORT_WIDTH_DESC 'W'
#define HWT_SORT_WIDTH_ASC 'w'
#define HWT_SORT_HEIGHT_DESC 'H'
#define HWT_SORT_HEIGHT_ASC 'h'
#define HWT_SORT_INPUT 'i'

/* Option records, SoA, one entry per option (common/Options.hpp:48-58).
 * strike = StrikePrices, bond_maturity = Maturities [years], option_maturity =
 * Lengths [years], term_unit = TermUnits [days], term_steps = TermStepCounts
 * [steps per term unit year], a = ReversionRates, sigma = Volatilities,
 * type = Types (0 = CALL, 1 = PUT). */
typedef struct hwt_options {
    int32_t n;
    const double *strike;
    const double *bond_maturity;
    const double *option_maturity;
    const uint16_t *term_unit;
    const uint16_t *term_steps;
    const double *a;
    const double *sigma;
    const int8_t *type;
} hwt_options;

/* Yield curve (common/Yield.hpp:14-18): continuously compounded zero rates
 * (Prices) at whole-day maturities (TimeSteps), ascending days. */
typedef struct hwt_yield {
    int32_t n;
    const double *rate;
    const int32_t *day;
} hwt_yield;

/* Tuning knobs; zero fields take the context's (tuned or default) values.
 * block_size plays the part of the reference's -b flag (common/Args.hpp:43). */
typedef struct hwt_config {
    int32_t mode;          /* HWT_* mode */
    int32_t block_size;    /* smallest warp group (64, 128, 256 or 512 threads) that prices one
                              wide tree; each tree gets the smallest group at least this large
                              that holds it at 8 (FP64 rows) or 16 (float rows) nodes per thread */
    int32_t sort;          /* HWT_SORT_* schedule order (0 = HWT_SORT_NONE) */
    int32_t big_threshold; /* widths above this leave warp tasks for warp groups (<= 256 for
                              double rows, <= 1024 for float rows; 0 = the default) */
    int32_t use_graph;     /* 1 = replay a captured CUDA graph (default), 0 = direct launches */
    int32_t record_busy;   /* 1 = record per-block busy time for the tail-imbalance stat */
    int32_t warp_k_mask;   /* nodes-per-lane values warp tasks may use: bit q allows the q-th of
                              {1, 2, 3, 4, 5, 6, 7, 8, 12, 16, 32}; 12, 16 and 32 apply to float
                              rows only (32: trees of up to 1,024 nodes on one warp, coefficients
                              in shared memory); 0 = the mode's default (FP64: 1..8; double-float:
                              1, 2, 3, 4, 6, 8; float rows: 1, 2, 4, 8, 16, 32) */
} hwt_config;

/* Run statistics, filled when a non-NULL pointer is passed.  Times are CUDA-event
 * times on the context's stream. */
typedef struct hwt_stats {
    double total_ms;        /* whole call on the stream: copies + sizing + pricing */
    double pricing_ms;      /* pricing kernel only */
    double sizing_ms;       /* sizing / validation / binning kernels */
    int64_t nodes;          /* active tree nodes of one pass, summed over options */
    int64_t h2d_bytes;      /* bytes copied host -> device by this call */
    int64_t d2h_bytes;      /* bytes copied device -> host by this call */
    int64_t device_bytes;   /* device memory held by the context */
    int32_t kernel_launches;/* kernels of this library launched by this call */
    int32_t n_block_trees;  /* trees priced by a whole block */
    int32_t n_warp_tasks;   /* warp tasks (groups of small trees) */
    int32_t grid;           /* pricing blocks launched */
    int32_t block_size;     /* threads per pricing block (512) */
    int32_t max_width;      /* widest tree in the batch */
    int32_t max_height;     /* tallest tree in the batch */
    int32_t graph_replayed; /* 1 if the kernels ran from a captured graph */
    double busy_max_ms;     /* per-block busy time: max (record_busy only) */
    double busy_mean_ms;    /* per-block busy time: mean (record_busy only) */
} hwt_stats;

typedef struct hwt_ctx hwt_ctx;

/* Library ABI version (HWT_ABI_VERSION). */
int hwt_abi_version(void);

/* Size in bytes of the named record as this library was built ("hwt_options",
 * "hwt_yield", "hwt_config", "hwt_stats", "hwt_box", "hwt_train_config",
 * "hwt_train_stats", "hwt_surrogate_stats"), 0 for any other name: a binding
 * checks its own layouts against it before passing a record. */
size_t hwt_struct_size(const char *name);

/* Creates a context on CUDA device `device`: stream, events, and buffers that
 * grow with the largest batch seen.  tune_cache: path of the autotuner's cache
 * file (read now, written by hwt_autotune), or NULL.  Returns NULL on failure;
 * hwt_create_status() then says why.  Replaces the reference's per-call Thrust
 * allocations (cuda/CudaDomain.cuh:114-130) and cudaSetDevice
 * (cuda-option/CudaOptionMain.cu:104-105). */
hwt_ctx *hwt_create(int device, const char *tune_cache);
int hwt_create_status(void);
void hwt_destroy(hwt_ctx *ctx);
const char *hwt_last_error(const hwt_ctx *ctx);

/* Prices n options held in HOST memory; out_prices (n doubles, host) receives
 * the prices in input order.  Replaces seq::computeOptions (seq/Seq.hpp:181)
 * and KernelRunBase::run (cuda-option/Kernel.cuh:303-314,
 * cuda-multi/Kernel.cuh:375-404).  n == 0 is a no-op.  A rejected option makes
 * the call return HWT_EINVAL; its price is NaN and the message names the first
 * rejected index. */
int hwt_price(hwt_ctx *ctx, const hwt_options *opts, const hwt_yield *yield, int mode,
              double *out_prices, hwt_stats *stats);

/* As hwt_price with explicit configuration (the reference's blockSize and
 * SortType arguments, cuda-option/Kernel.cuh:303-305). */
int hwt_price_ex(hwt_ctx *ctx, const hwt_options *opts, const hwt_yield *yield,
                 const hwt_config *cfg, double *out_prices, hwt_stats *stats);

/* Prices options whose arrays are already in DEVICE memory of the context's
 * device; out_prices is a device pointer.  The yield curve is host memory.
 * Runs on the context's stream and waits for it, so device inputs may be reused
 * on return.  No host<->device copies of option data. */
int hwt_price_device(hwt_ctx *ctx, const hwt_options *dev_opts, const hwt_yield *yield,
                     const hwt_config *cfg, double *dev_out_prices, hwt_stats *stats);

/* Allocation-free variant of hwt_price_device, with no counterpart in the
 * reference.  For callers that cannot call cudaMalloc (device memory owned by
 * another allocator; latency-bound paths where cudaMalloc/cudaFree, which may
 * synchronise the device, are not allowed): no context, no allocation of any
 * kind; the scratch the pricing kernels need lives in a static device array of
 * the library (about 5 MB on every GPU that loads it, until exit).
 *   dev_opts, dev_yield: HOST structs whose array members are DEVICE pointers of
 *     the current device (n is read on the host); dev_out_prices: device pointer
 *   mode: HWT_BATCHED_FP64, HWT_BATCHED_FP32 or HWT_BATCHED_MIXED
 *   stream: cudaStream_t to run on (NULL: the default stream); the call waits for it
 * At most 32768 options and 1024 curve nodes per call, else HWT_EINVAL.  Every
 * call looks up the array's device address in the CUDA context current at the
 * call (none is kept, so a context re-created after cudaDeviceReset is safe);
 * the first lookup in a context loads the library's device code, so make the
 * first call in a context before any stream capture.  Calls share the array:
 * calls that overlap on the GPU race.  Returns HWT_EINVAL if an option is
 * invalid (its price is NaN) or a curve rate is not finite.  Warp-task layout:
 * hwt_warp_layout(mode, width, 0, 512, ...) for the float modes and
 * (mode, width, 0, 256, ...) for HWT_BATCHED_FP64 describe this entry point. */
int hwt_price_device_noalloc(const hwt_options *dev_opts, const hwt_yield *dev_yield, int mode,
                             double *dev_out_prices, void *stream);

/* Tree shape of each option as the reference computes it
 * (common/OptionConstants.hpp:29-53, seq/Seq.hpp:125), on the host, no GPU:
 * jmax, height n, width 2*jmax+1 and maturity step (int)(t/dt).  Any output
 * pointer may be NULL.  Returns HWT_EINVAL if an option is invalid (its entries
 * are then -1). */
int hwt_shape(const hwt_options *opts, int32_t *jmax, int32_t *height, int32_t *width,
              int32_t *maturity_step);

/* Active nodes of one pass of one option's tree, sum_{i<n} (2 min(i,jmax) + 1):
 * the work unit of the roofline accounting. */
int64_t hwt_active_nodes(int32_t height, int32_t jmax);

/* How the batched engine lays out a tree `width` nodes wide for `mode` (a batched
 * mode) with this K mask and widest-warp-task threshold (0 = the defaults, as a
 * context without tuning uses them; hwt_price_device_noalloc uses threshold 512
 * for the float modes and 256 for FP64): *K nodes per lane on *L lanes of a warp task,
 * or *K = *L = 0 when the tree goes to a warp group.  Host only, no GPU.
 * HWT_EINVAL for a non-batched mode or a width outside 1..4096. */
int hwt_warp_layout(int mode, int32_t width, int32_t warp_k_mask, int32_t big_threshold, int32_t *K,
                    int32_t *L);

/* Autotuner: prices the batch with each candidate configuration (block size,
 * block-tree threshold), keeps the fastest for `mode` in the context, writes it
 * to the context's tune cache (if any) and returns it in *best. */
int hwt_autotune(hwt_ctx *ctx, const hwt_options *opts, const hwt_yield *yield, int mode,
                 int repeats, hwt_config *best);

/* Current default configuration of the context for `mode`. */
int hwt_get_config(const hwt_ctx *ctx, int mode, hwt_config *cfg);

/* Measured FP64 and FP32 fused-multiply-add peaks of the context's GPU in
 * TFLOP/s (2 flops per FMA), from dependent-chain microbenchmarks timed with
 * CUDA events.  The roofline denominators of the tree kernels. */
int hwt_measure_peaks(hwt_ctx *ctx, double *fp64_tflops, double *fp32_tflops);

/* ---- Learned surrogate -------------------------------------------------------
 * An 8 -> 4 x 256 (SiLU) -> 2 MLP over standardised (option maturity, bond
 * maturity, strike / forward bond price, a, sigma, steps per year, call/put) and a
 * zero pad.  Output 0 is price / forward bond price (or, with box.residual, the
 * tree price minus the Hull-White closed-form price over the forward bond price),
 * standardised; output 1 estimates log |output-0 error| and routes the options it
 * does not trust to the tree.  Layer 0 is fp32 (CUDA cores); layers 1-4 use bf16
 * weights with fp32 accumulation on the tensor cores.  Trained on prices from the
 * batched FP64 tree; inference runs the whole network in one fused tensor-core
 * kernel.  Options outside the training box and options the error head flags go
 * to the tree, and a random sample of the network's answers is repriced by the
 * tree as its judge.  The reference has no learned part; these entry points have
 * no reference counterpart. */
typedef struct hwt_box {
    double t_min, t_max;             /* option maturity [years] */
    double span_min, span_max;       /* bond maturity - option maturity [years] */
    double moneyness_min, moneyness_max; /* strike / forward bond price */
    double a_min, a_max, sigma_min, sigma_max;
    int32_t steps_min, steps_max;    /* steps per year */
    int32_t term_unit;               /* the only term unit inside the box */
    int32_t residual;                /* 1: the network learns (tree price - Hull-White closed-form
                                        price) / forward bond price, a control variate; 0: price /
                                        forward bond price */
} hwt_box;

typedef struct hwt_train_config {
    int32_t epochs;                  /* passes over the samples (default 1) */
    int32_t batch;                   /* samples per Adam step (default 8192) */
    double lr, lr_min;               /* cosine decay from lr to lr_min over all steps */
    uint64_t seed;                   /* shuffling and the held-out split */
    double err_weight;               /* weight of the error head's loss; 0: head untrained, no routing */
    double route_tolerance;          /* price error (per 100 face) that the network's answers must keep
                                        on the held-out samples; sets the routing threshold of the error
                                        head or, on a single-tree box, a routing distance around each
                                        payoff kink and box edge, so that every held-out answer the
                                        network keeps is within it (default 1e-4) */
    double holdout;                  /* fraction of in-box samples held out for that (default 0.05) */
    int32_t kink_oversample;         /* single-tree box: samples within 0.005 in moneyness of a payoff
                                        kink appear this many times per epoch (1 or 0: once) */
    int32_t hard_every;              /* hard-sample mining: every this many epochs (0: off), from the
                                        first quarter of the epochs on, the network prices every training
                                        sample and ... */
    double hard_fraction;            /* ... this fraction of them, those with the largest errors, is
                                        repeated once more per epoch until the next mining (max 0.25) */
} hwt_train_config;

typedef struct hwt_train_stats {
    double final_loss;               /* mean loss of the last epoch, standardised units */
    double train_ms, label_ms;       /* training time; time the tree took to price the labels */
    int64_t steps, samples;          /* Adam steps; in-box samples trained on */
    double samples_per_s;
    double y_mean, y_std;            /* target standardisation */
    double route_threshold;          /* predicted price error above which an option goes to the tree
                                        (+inf: routing off) */
    double holdout_answered;         /* fraction of held-out samples the network answers */
    double holdout_max_abs, holdout_p99_abs; /* |network - tree| over those it answers */
    double holdout_all_max_abs;      /* |network - tree| over all held-out samples */
    int64_t holdout;                 /* held-out samples */
    int64_t n_kinks;                 /* single-tree box: payoff kinks found in the labels */
    double kink_delta;               /* the largest routing distance (moneyness) around a kink or box
                                        edge; options within a point's own distance go to the tree
                                        (< 0: no kink routing) */
    double ladder_tolerance[12];     /* the routing also calibrated at these tolerances ... */
    double ladder_answered[12];      /* ... answering these fractions of the held-out samples */
    int64_t holdout_over;            /* held-out samples the network answers above route_tolerance
                                        (0 by construction) */
    int64_t hard_minings;            /* hard-sample minings run */
    double hard_threshold_abs;       /* smallest price error in the last mined set */
} hwt_train_stats;

typedef struct hwt_surrogate_stats {
    int64_t n_in_box, n_routed, n_judged;  /* n_routed: outside the box; n_judged: the judge's sample */
    int32_t fell_back;               /* 1: the judge saw an error above the tolerance and the tree
                                        priced the network's answers too */
    int32_t pad;
    double judge_max_abs, judge_p99_abs, judge_mean_abs; /* |network - tree| on the judged sample */
    double network_ms;               /* features, fused network and routing on the device */
    double tree_ms;                  /* the tree's own pricing calls (routed, judged, fallback) */
    double route_ms;                 /* from routing to the tree's answers scattered back */
    double total_ms;                 /* the whole call on the stream, copies included */
    int64_t n_flagged;               /* in-box options the routing sent to the tree */
    int64_t n_network;               /* options answered by the network */
    double route_tolerance;          /* the ladder tolerance the call routed with (NaN: the training one) */
    double copy_ms;                  /* host-to-device copy of the options */
} hwt_surrogate_stats;

typedef struct hwt_surrogate hwt_surrogate;

hwt_surrogate *hwt_surrogate_create(hwt_ctx *ctx, const hwt_box *box, uint64_t seed);
void hwt_surrogate_destroy(hwt_surrogate *s);
const char *hwt_surrogate_last_error(const hwt_surrogate *s);
/* Prices the (host) samples with the batched FP64 tree, trains on the in-box ones
 * but a held-out slice, and sets the routing threshold on that slice. */
int hwt_surrogate_train(hwt_surrogate *s, const hwt_options *samples, const hwt_yield *yield,
                        const hwt_train_config *cfg, hwt_train_stats *stats);
/* Routing tolerance: with judge_tolerance > 0 the call routes with the calibration
 * (of the training ladder: 2.5e-5, 5e-5, 9e-5, 1e-4, 1.8e-4, 2e-4, 4.5e-4, 5e-4,
 * 9e-4, 1e-3, 1.8e-3, 2e-3) for the largest tolerance not above 0.9 judge_tolerance,
 * a margin that sends the answers just under the judge's tolerance to the tree;
 * otherwise with the training's route_tolerance.
 * Prices host options: network inside the box unless the option is flagged - by
 * the error head, or, on a single-tree box (every tree parameter pinned, so the
 * price is piecewise linear in the strike), by a strike within the calibrated
 * distance of one of the tree's payoff kinks, which training finds in its labels -
 * tree (tree_mode: a batched mode) outside the box, for flagged options
 * and for the judge's sample (fraction judge_fraction of the in-box options the
 * network answers, drawn from `seed`), whose options get the tree price.  If
 * judge_tolerance > 0 and the judge's largest |network - tree| exceeds it, the
 * tree prices the network's other answers as well (stats->fell_back = 1), so the
 * answer is never worse than the tolerance on the judged sample. */
int hwt_surrogate_price(hwt_surrogate *s, const hwt_options *opts, const hwt_yield *yield, double judge_fraction,
                        uint64_t seed, int tree_mode, double judge_tolerance, double *out_prices,
                        hwt_surrogate_stats *stats);
/* Checkpoint: box, target scaling, routing threshold, weights and Adam state. */
int hwt_surrogate_save(const hwt_surrogate *s, const char *path);
int hwt_surrogate_load(hwt_surrogate *s, const char *path);
/* Parameters: layer l has W_l [fan_in][fan_out] then b_l [fan_out]; fan_in 8
 * (7 features + a zero pad row) for the first layer, fan_out 2 for the last; get
 * (set = 0) or set them. */
int64_t hwt_surrogate_param_count(const hwt_surrogate *s);
int hwt_surrogate_params(hwt_surrogate *s, float *params, int64_t count, int set);
/* Forward pass on host standardised features x [n][7] into out [n][2]: path 0 =
 * the fused inference kernel, 1 = the layer-by-layer training kernels.
 * hwt_surrogate_forward is path 0. */
int hwt_surrogate_forward(hwt_surrogate *s, const float *x, int n, float *out);
int hwt_surrogate_forward_ex(hwt_surrogate *s, const float *x, int n, float *out, int path);
/* The fused inference kernel on DEVICE buffers of the surrogate's device: dev_x
 * [n][8] standardised features with a zero eighth column (16-byte aligned rows),
 * dev_out [n][2]; waits for the kernel and returns its CUDA-event time in
 * *kernel_ms (may be NULL). */
int hwt_surrogate_forward_device(hwt_surrogate *s, const float *dev_x, int n, float *dev_out, double *kernel_ms);
/* Loss and gradients (no update) of the training path on x [n][7] and standardised
 * targets y [n]: 0.5 mean (o0 - y)^2 + err_weight 0.5 mean (o1 - log(|o0 - y| +
 * 1e-3))^2, the error-head target held constant; gradients in the params layout.
 * The hook the gradient check against the CPU oracle uses. */
int hwt_surrogate_loss_grads(hwt_surrogate *s, const float *x, const float *y, int n, double err_weight,
                             double *loss, float *grads);
/* Fault injection for tests of the failure path (no GPU fault involved): mode 1
 * makes every tensor-core kernel wait, before its first MMA, on an mbarrier phase
 * that nothing completes; mode 2 does so after its first K block's MMAs were
 * committed; 0 turns it off.  The bounded wait runs out (about a second), the
 * kernel waits for what it issued, frees its tensor memory and returns, and the
 * call returns HWT_ETIMEOUT with the context still usable. */
int hwt_surrogate_inject_stall(hwt_surrogate *s, int mode);

/* Host helpers of the single-tree routing (no GPU), the same code the training runs.
 *
 * hwt_find_kinks: payoff kinks of one tree from labelled samples of options that
 * share it - x[i] the moneyness (strike / forward bond price), price[i] the tree's
 * price, type[i] 0 (call) or 1 (put).  The price is piecewise linear in the strike;
 * a slope change above 1e-3 (price per unit of moneyness) between neighbouring
 * samples of one type marks a kink, and detections closer than 1e-4 are merged to
 * their midpoint.  Writes the kinks, ascending, to kinks[cap] and their number to
 * *count; HWT_EINVAL if more than cap were found (the samples are not one tree).
 *
 * hwt_route_distances: the routing calibration - for each of the n_points routing
 * points (moneyness), the distance that reaches every sample (moneyness x[i],
 * absolute price error err[i]) above tol whose nearest point it is, -1 where there
 * is none; *answered = the fraction of the samples outside every point's distance
 * (those the network keeps, all within tol; 1 for n = 0). */
int hwt_find_kinks(const double *x, const double *price, const int8_t *type, int64_t n, double *kinks, int32_t cap,
                   int32_t *count);
int hwt_route_distances(const double *points, int32_t n_points, const double *x, const double *err, int64_t n,
                        double tol, double *delta, double *answered);

/* ---- Input files ------------------------------------------------------------
 * Replace trinom::Options(const std::string&) and trinom::Yield(const
 * std::string&) (common/Options.hpp:73-98, common/Yield.hpp:20-38), which read
 * the "[..]" arrays value by value with iostream extraction.  hwt_read_options
 * parses the eight arrays with host threads (values correctly rounded, the same
 * doubles as the reference's reader; integer fields must be integral and in
 * range; types 0 or 1), or reads a binary cache file written by
 * hwt_write_options_bin (recognised by its magic), into arrays the library
 * allocates; hwt_free_options releases them.  On error the message goes to
 * err[err_len] (may be NULL).  No GPU is needed. */
int hwt_read_options(const char *path, hwt_options *out, char *err, int err_len);
void hwt_free_options(hwt_options *opts);
int hwt_write_options_bin(const char *path, const hwt_options *opts);
int hwt_read_yield(const char *path, hwt_yield *out, char *err, int err_len);
void hwt_free_yield(hwt_yield *yield);

#ifdef __cplusplus
}
#endif

#endif /* HWTREE_H */
