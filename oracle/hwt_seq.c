/*
 * ORACLE - test infrastructure, not the product.
 *
 * A plain-C restatement of the reference's CPU pricer for the batch pricing path
 * (seq/Seq.hpp:24-190 with common/OptionConstants.hpp:29-53 and
 * common/Domain.hpp:11-169).  Only tests/, the smoke check and bench.py's CPU
 * baseline load it, always to check results against or as the timed CPU
 * reference; the GPU product never calls it and has no CPU fallback.
 *
 * Pinned against the reference's own golden vectors (data/out/*.out for the
 * double build, data/out32/*.out for the float build, copied under tests/golden/)
 * and against the reference's seq/ compiled from its sources (oracle/Makefile).
 *
 * Two instantiations of the same body: oracle_price_f64 (reference -DUSE_DOUBLE)
 * and oracle_price_f32 (reference default float build).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#else
static void omp_set_num_threads(int n) { (void)n; }
#endif

#define SFX_(a, b) a##b
#define SFXX(a, b) SFX_(a, b)

#define REAL double
#define SFX(name) SFXX(name, _f64)
#define ROUNDR(x) round((x))
#define REALMAX DBL_MAX
#define REALMIN DBL_MIN
#include "hwt_seq_body.h"
#undef REAL
#undef SFX
#undef ROUNDR
#undef REALMAX
#undef REALMIN

#define REAL float
#define SFX(name) SFXX(name, _f32)
#define ROUNDR(x) roundf((x))
#define REALMAX FLT_MAX
#define REALMIN FLT_MIN
#include "hwt_seq_body.h"
#undef REAL
#undef SFX
#undef ROUNDR
#undef REALMAX
#undef REALMIN

/* Threads the OpenMP runtime will use for the CPU baseline. */
int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
