// Hull-White one-factor trinomial tree: per-option model math shared by host and
// device code.  Every expression that feeds the tree's shape or coefficients is
// evaluated in double with the same operations, in the same order, as the
// reference's double build, so the integer structure (jmax, height, maturity step)
// and the branching probabilities are bit-identical to it:
//   per-option constants   common/OptionConstants.hpp:29-53
//   yield interpolation    common/Domain.hpp:11-46
//   branching probs A/B/C  common/Domain.hpp:51-96
//   maturity step          seq/Seq.hpp:125
#pragma once

#include <stdint.h>
#include <math.h>

#ifdef __CUDACC__
#define HWT_HD __host__ __device__ __forceinline__
#else
#define HWT_HD inline
#endif

namespace hwt {

// Shape and constants of one option's tree.
struct Shape {
    double dt, dr, M;     // step [years], rate spacing, exp(-a dt) - 1
    int32_t jmax;         // (int)(-0.184 / M) + 1
    int32_t n;            // height: steps to bond maturity (0 when non-positive)
    int32_t m;            // maturity step (int)(t / dt); payoff applies iff 0 <= m < n
    int32_t jc;           // min(jmax, n): half-width of the nodes that can carry value
    int32_t width;        // 2 * jc + 1 nodes actually used
    int32_t edges;        // 1 when the +-jmax edge branching is reachable (jc == jmax)
    int64_t nodes;        // active nodes per pass: sum_{i<n} (2 min(i, jmax) + 1)
};

// Validation codes for one option's inputs (mirrors what makes the reference's
// constants undefined: a <= 0 gives M >= 0, zero steps or term unit divide by 0).
enum ShapeStatus : int32_t { SHAPE_OK = 0, SHAPE_BAD_A = 1, SHAPE_BAD_STEPS = 2, SHAPE_BAD_UNIT = 3,
                             SHAPE_TOO_WIDE = 4, SHAPE_NONFINITE = 5 };

HWT_HD int64_t active_nodes(int32_t n, int32_t jmax)
{
    if (n <= 0) return 0;
    if (n <= jmax + 1) return (int64_t)n * n;                      // never reaches the edges
    const int64_t j1 = (int64_t)jmax + 1;
    return j1 * j1 + (int64_t)(n - jmax - 1) * (2 * (int64_t)jmax + 1);
}

// OptionConstants.hpp:29-53 in double.  Returns a ShapeStatus.
HWT_HD int32_t make_shape(Shape &s, double bond_maturity, double option_maturity, uint16_t term_unit,
                          uint16_t term_steps, double a, double sigma, int32_t max_width)
{
    if (term_unit == 0) return SHAPE_BAD_UNIT;
    if (term_steps == 0) return SHAPE_BAD_STEPS;
    if (!(a > 0.0)) return SHAPE_BAD_A;
    if (!isfinite(bond_maturity) || !isfinite(option_maturity) || !isfinite(sigma) || !isfinite(a))
        return SHAPE_NONFINITE;
    // ceil(365.0 / term_unit) (:33) in integers: the double quotient is exact when
    // term_unit divides 365 and otherwise lies at least 1/term_unit from an integer,
    // so the two agree, and the sizing pass saves a double division per option
    const int units_per_year = (365 + term_unit - 1) / term_unit;
    const double nreal = term_steps * units_per_year * bond_maturity;   // :35 (int * double)
    if (nreal > 1.0e7) return SHAPE_TOO_WIDE;
    s.n = (int32_t)nreal;
    if (s.n < 0) s.n = 0;
    s.dt = units_per_year / (double)term_steps;                         // :37
    const double V = sigma * sigma * (1.0 - exp(-2.0 * a * s.dt)) / (2.0 * a);   // :43
    s.dr = sqrt(3.0 * V);                                               // :44
    s.M = exp(-a * s.dt) - 1.0;                                         // :45
    const double jq = -0.184 / s.M;
    if (!(jq < 1.0e9)) return SHAPE_TOO_WIDE;
    s.jmax = (int32_t)jq + 1;                                           // :51
    const double mq = option_maturity / s.dt;                           // seq/Seq.hpp:125
    s.m = (mq >= 2147483647.0) ? 2147483647 : (mq <= -2147483648.0 ? (-2147483647 - 1) : (int32_t)mq);
    s.jc = s.jmax < s.n ? s.jmax : s.n;
    s.width = 2 * s.jc + 1;
    s.edges = (s.jc == s.jmax) ? 1 : 0;
    s.nodes = active_nodes(s.n, s.jmax);
    if (s.width > max_width) return SHAPE_TOO_WIDE;
    return SHAPE_OK;
}

// getYieldAtYear (Domain.hpp:11-46), double, curve days are whole days.
template <typename R>
HWT_HD R yield_at_year(R t, int term_unit, const R *rates, const int32_t *days, int size)
{
    const int t_days = (int)round(t * (R)term_unit);
    int first = 0, second = 0;
    for (int i = 0; i < size; ++i) {
        if (days[i] >= t_days) { second = i; break; }
        first = i;
    }
    if (first == second) return rates[0];
    if (first == size - 1) return rates[size - 1];
    const int32_t t1 = days[first], t2 = days[second];
    const R p1 = rates[first], p2 = rates[second];
    const R coefficient = (R)(t_days - t1) / (R)(t2 - t1);
    return p1 + coefficient * (p2 - p1);
}

// Discount factor the alpha fit matches at step k: exp(-R(k dt) * k dt).  For
// k >= 2 this is computeAlpha's P with ti = (i + 2) * dt (Domain.hpp:98-104); for
// k = 1 it is the first step's exp(-alpha_0 dt) with alpha_0 = R(dt) (Seq.hpp:58).
template <typename R>
HWT_HD R discount_at_step(int k, R dt, int term_unit, const R *rates, const int32_t *days, int size)
{
    const R tk = (R)k * dt;
    const R r = yield_at_year<R>(tk, term_unit, rates, days, size);
    return exp(-r * tk);
}

// Branching probabilities, Hull & White (1996) exhibit 1, written with the same
// operations as Domain.hpp:51-96 so the double values are identical.
HWT_HD double pu_a(int j, double M) { return 1.0 / 6.0 + (j * j * M * M + j * M) * 0.5; }
HWT_HD double pm_a(int j, double M) { return 2.0 / 3.0 - j * j * M * M; }
HWT_HD double pd_a(int j, double M) { return 1.0 / 6.0 + (j * j * M * M - j * M) * 0.5; }
HWT_HD double pu_b(int j, double M) { return 1.0 / 6.0 + (j * j * M * M - j * M) * 0.5; }
HWT_HD double pm_b(int j, double M) { return -1.0 / 3.0 - j * j * M * M + 2.0 * j * M; }
HWT_HD double pd_b(int j, double M) { return 7.0 / 6.0 + (j * j * M * M - 3.0 * j * M) * 0.5; }
HWT_HD double pu_c(int j, double M) { return 7.0 / 6.0 + (j * j * M * M + 3.0 * j * M) * 0.5; }
HWT_HD double pm_c(int j, double M) { return -1.0 / 3.0 - j * j * M * M - 2.0 * j * M; }
HWT_HD double pd_c(int j, double M) { return 1.0 / 6.0 + (j * j * M * M + j * M) * 0.5; }

// Where the value of node j goes in one step, in the three-plus-one form the
// stencils use.  up: to j+1, stay: to j, down: to j-1, jump: to j+2 (bottom edge)
// or j-2 (top edge).  Interior nodes: (pu_a, pm_a, pd_a, 0).  Bottom edge j=-jmax
// branches up-two/up-one/middle (Seq.hpp:72-78): up=pm_b, stay=pd_b, jump=pu_b.
// Top edge j=+jmax branches middle/down-one/down-two (Seq.hpp:79-85): stay=pu_c,
// down=pm_c, jump=pd_c.
struct Branch {
    double up, stay, down, jump;
};

HWT_HD Branch branch(int j, int jmax, double M)
{
    Branch b;
    if (j == -jmax) {
        b.up = pm_b(j, M); b.stay = pd_b(j, M); b.down = 0.0; b.jump = pu_b(j, M);
    } else if (j == jmax) {
        b.up = 0.0; b.stay = pu_c(j, M); b.down = pm_c(j, M); b.jump = pd_c(j, M);
    } else {
        b.up = pu_a(j, M); b.stay = pm_a(j, M); b.down = pd_a(j, M); b.jump = 0.0;
    }
    return b;
}

// Per-column discount of the alpha-free tree: exp(-(j dr) dt), the same
// expression as the reference's exp(-jval.rate * c.dt) (Seq.hpp:103).
HWT_HD double column_discount(int j, double dr, double dt) { return exp(-(j * dr) * dt); }

}  // namespace hwt
