// hwt_price_device_noalloc: batched pricing that allocates nothing.
//
// Some callers cannot call cudaMalloc: a process whose device memory is already
// owned by another allocator (a framework's caching pool that holds the GPU), or
// a latency-bound service for which cudaMalloc/cudaFree, which may synchronise
// the device, are not allowed on the pricing path.  For them this entry point
// runs the same validation, binning and pricing kernels as hwt_price_device, but
// every piece of scratch memory (tree records, sort keys, sorted order, warp
// tasks, histogram bins, run status, float copy of the curve) lives in the
// file-scope array below, at most kNoAllocMaxOptions options per call.  The
// caller passes device pointers for the options, the yield curve and the prices.
//
// The array is a __device__ variable: every GPU that loads the library holds it
// (about 5 MB) until the process exits.  In host code its name is only a
// host-side stand-in, so every call looks up its device address with
// cudaGetSymbolAddress, in the CUDA context current at the call (the caller's
// device current), and passes that address to the kernels.  An address is valid
// only in the context it was looked up in, so none is kept between calls: a
// context created after cudaDeviceReset, or a non-primary context made current
// by the caller, gets its own.  The first lookup in a context also loads the
// library's device code there, so make the first call in a context before any
// stream capture.  All calls share the array and it keeps the last call's
// contents (the counters that must start at zero are cleared by every call), so
// calls that overlap on the GPU - from two streams or two host threads at once -
// race and must be serialised by the caller.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/hwtree.h"
#include "hwt_internal.h"

using namespace hwt;

namespace {

constexpr int kNoAllocMaxOptions = 32768;
constexpr int kNoAllocMaxYield = 1024;
constexpr size_t kAlign = 256;

constexpr size_t up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Byte offsets of the pieces inside the static scratch array.
constexpr size_t kOffTrees = 0;
constexpr size_t kOffKeys = up(kOffTrees + sizeof(Tree) * kNoAllocMaxOptions);
constexpr size_t kOffOrder = up(kOffKeys + 4ull * kNoAllocMaxOptions);
constexpr size_t kOffTasks = up(kOffOrder + 4ull * kNoAllocMaxOptions);
constexpr size_t kOffHist = up(kOffTasks + sizeof(WarpTask) * kNoAllocMaxOptions);  // hist then fill
constexpr size_t kOffBinStart = up(kOffHist + 2ull * 4 * kKeyBins);
constexpr size_t kOffTaskStart = up(kOffBinStart + 4ull * kKeyBins);
constexpr size_t kOffStatus = up(kOffTaskStart + 4ull * kKeyBins);
constexpr size_t kOffRateF = up(kOffStatus + sizeof(RunStatus));
constexpr size_t kOffCurveBad = up(kOffRateF + 4ull * kNoAllocMaxYield);  // non-finite curve rates seen
constexpr size_t kScratchBytes = up(kOffCurveBad + 4);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Float copy of the curve; *bad is raised for a rate that is not finite.
__global__ void curve_to_float(const double *rate, int n, float *rate_f, int *bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double r = rate[i];
    if (!isfinite(r)) atomicExch(bad, 1);
    rate_f[i] = (float)r;
}

int fail_cuda(cudaError_t e)
{
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? HWT_ENOMEM : HWT_ECUDA;
}

}  // namespace

extern "C" int hwt_price_device_noalloc(const hwt_options *dev_opts, const hwt_yield *dev_yield, int mode,
                                        double *dev_out_prices, void *stream)
{
    if (!dev_opts || !dev_yield) return HWT_EINVAL;
    if (mode != HWT_BATCHED_FP64 && mode != HWT_BATCHED_FP32 && mode != HWT_BATCHED_MIXED) return HWT_EUNSUPPORTED;
    const int n = dev_opts->n;
    if (n < 0 || n > kNoAllocMaxOptions) return HWT_EINVAL;  // more than 32768 options per call
    if (dev_yield->n <= 0 || dev_yield->n > kNoAllocMaxYield || !dev_yield->rate || !dev_yield->day) return HWT_EINVAL;
    if (n == 0) return HWT_OK;
    if (!dev_out_prices || !dev_opts->strike || !dev_opts->bond_maturity || !dev_opts->option_maturity ||
        !dev_opts->term_unit || !dev_opts->term_steps || !dev_opts->a || !dev_opts->sigma || !dev_opts->type)
        return HWT_EINVAL;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda(e);
    cudaStream_t st = (cudaStream_t)stream;
    // set-up: the array's device address in the current context
    void *scratch = nullptr;
    if ((e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch)) != cudaSuccess) return fail_cuda(e);
    unsigned char *base = (unsigned char *)scratch;

    EngineParams p;
    memset(&p, 0, sizeof(p));
    p.opt.n = n;
    p.opt.strike = dev_opts->strike;
    p.opt.bond_maturity = dev_opts->bond_maturity;
    p.opt.option_maturity = dev_opts->option_maturity;
    p.opt.term_unit = dev_opts->term_unit;
    p.opt.term_steps = dev_opts->term_steps;
    p.opt.a = dev_opts->a;
    p.opt.sigma = dev_opts->sigma;
    p.opt.type = dev_opts->type;
    p.yc.n = dev_yield->n;
    p.yc.rate = dev_yield->rate;
    p.yc.day = dev_yield->day;
    p.yc.rate_f = (const float *)(base + kOffRateF);
    p.s.trees = (Tree *)(base + kOffTrees);
    p.s.keys = (int32_t *)(base + kOffKeys);
    p.s.order = (int32_t *)(base + kOffOrder);
    p.s.tasks = (WarpTask *)(base + kOffTasks);
    p.s.hist = (int32_t *)(base + kOffHist);
    p.s.fill = p.s.hist + kKeyBins;
    p.s.bin_start = (int32_t *)(base + kOffBinStart);
    p.s.task_start = (int32_t *)(base + kOffTaskStart);
    p.s.status = (RunStatus *)(base + kOffStatus);
    p.s.cta_busy = nullptr;
    p.out = dev_out_prices;
    p.max_width = kMaxTreeWidth;
    p.group_threads = mode == HWT_BATCHED_FP64 ? 128 : 64;
    p.warp_k_mask = run_k_mask(mode, 0, 512, &p.max_warp_k);
    p.max_group_k = mode == HWT_BATCHED_FP64 ? kMaxBlockK : kMaxGroupKFloat;
    p.sort = 0;
    p.big_threshold = 32 * (p.max_warp_k < 16 ? p.max_warp_k : 16);  // warp tasks up to 512 nodes
    p.record_busy = 0;
    p.curve_discounts = mode == HWT_BATCHED_MIXED ? 1 : 0;

    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail_cuda(e);
    const int per = pricing_blocks_per_sm(mode);
    if (per < 1) return HWT_EUNSUPPORTED;

    int *curve_bad = (int *)(base + kOffCurveBad);
    if ((e = cudaMemsetAsync(curve_bad, 0, sizeof(int), st)) != cudaSuccess) return fail_cuda(e);
    curve_to_float<<<(dev_yield->n + 255) / 256, 256, 0, st>>>(dev_yield->rate, dev_yield->n, (float *)(base + kOffRateF),
                                                               curve_bad);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e);
    // launch_sizing clears the histogram, fill counters and run status itself
    if ((e = launch_sizing(p, st)) != cudaSuccess) return fail_cuda(e);
    if ((e = launch_pricing(p, mode, per * sms, st)) != cudaSuccess) return fail_cuda(e);
    RunStatus status;
    int bad_curve = 0;
    if ((e = cudaMemcpyAsync(&status, p.s.status, sizeof(RunStatus), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail_cuda(e);
    if ((e = cudaMemcpyAsync(&bad_curve, curve_bad, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail_cuda(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e);
    if (status.wide_smem_missing) return HWT_ECUDA;
    if (bad_curve) return HWT_EINVAL;  // a curve rate is not finite: every price is suspect
    return status.bad_count > 0 ? HWT_EINVAL : HWT_OK;
}
