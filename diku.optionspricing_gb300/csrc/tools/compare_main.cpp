// hwt-compare: the reference's Compare harness (test/Compare.cpp:9-18,
// test/Compare.hpp:8-24) restated without Catch.  Reads two "[..]" arrays from
// stdin, test first then gold, and checks every element the way Catch's
// Approx::custom().margin(1000 * eps) does: pass if |test - gold| <= 1000 * eps
// or |test - gold| <= 100 * FLT_EPSILON * |gold|.  eps is DBL_EPSILON, or
// FLT_EPSILON with --fp32 (the reference's float build).  Also prints the error
// distribution (max / p99 absolute, max relative).  Exit status 0 = all equal.
//   --abs TOL   replace the margin by an absolute tolerance TOL (no relative term)
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>

#include "hwtree.hpp"

int main(int argc, char **argv)
{
    bool fp32 = false;
    double abs_tol = -1.0;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--fp32")) fp32 = true;
        else if (!std::strcmp(argv[i], "--abs") && i + 1 < argc) abs_tol = std::atof(argv[++i]);
        else {
            std::cerr << "usage: hwt-compare [--fp32] [--abs TOL] < test_and_gold" << std::endl;
            return 2;
        }
    }
    std::vector<double> test, gold;
    hwtree::Arrays::read_array(std::cin, test);
    hwtree::Arrays::read_array(std::cin, gold);
    if (test.size() != gold.size()) {
        std::cout << "FAILED: sizes differ (" << test.size() << " vs " << gold.size() << ")" << std::endl;
        return 1;
    }
    const double margin = 1000.0 * (fp32 ? (double)FLT_EPSILON : DBL_EPSILON);
    const double rel = 100.0 * (double)FLT_EPSILON;
    size_t bad = 0, first_bad = (size_t)-1;
    double max_abs = 0, max_rel = 0;
    std::vector<double> errs(test.size());
    for (size_t i = 0; i < test.size(); ++i) {
        const double d = std::fabs(test[i] - gold[i]);
        errs[i] = d;
        max_abs = std::max(max_abs, d);
        if (gold[i] != 0.0) max_rel = std::max(max_rel, d / std::fabs(gold[i]));
        bool ok;
        if (abs_tol >= 0) ok = d <= abs_tol;
        else ok = (test[i] + margin >= gold[i] && gold[i] + margin >= test[i]) ||
                  (d <= rel * std::fabs(gold[i]));
        if (!ok || std::isnan(test[i]) != std::isnan(gold[i])) {
            if (bad == 0) first_bad = i;
            ++bad;
        }
    }
    double p99 = 0;
    if (!errs.empty()) {
        std::vector<double> s = errs;
        const size_t k = std::min(s.size() - 1, (size_t)std::floor(0.99 * (s.size() - 1)));
        std::nth_element(s.begin(), s.begin() + k, s.end());
        p99 = s[k];
    }
    std::printf("compared %zu values: max abs %.3e, p99 abs %.3e, max rel %.3e\n", test.size(), max_abs, p99, max_rel);
    if (bad) {
        std::printf("FAILED: %zu value(s) outside tolerance; first at index %zu: %.17g vs %.17g\n", bad, first_bad,
                    test[first_bad], gold[first_bad]);
        return 1;
    }
    std::printf("All tests passed (%zu assertions)\n", test.size());
    return 0;
}
