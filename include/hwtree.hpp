// hwtree.hpp - header-only C++ adapter over the C ABI (hwtree.h) in the shapes
// of the reference project's records and pricing calls, so C++ callers of the
// reference switch by changing a namespace:
//   trinom::Options / trinom::Yield   common/Options.hpp:48-125, common/Yield.hpp:14-40
//   trinom::Arrays::read/write_array  common/Arrays.hpp:15-46 (same text format)
//   seq::computeOptions               seq/Seq.hpp:181-190
//   KernelRunBase::run                cuda-option/Kernel.cuh:303-314
// Records hold doubles (the reference's real under -DUSE_DOUBLE).  Errors are
// C++ exceptions on this side of the ABI, as in the reference.
#pragma once

#include <cmath>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <cstring>
#include <vector>

#include "hwtree.h"

namespace hwtree {

// common/Options.hpp:15-22, plus INPUT (arrival order, no binning by size)
enum class SortType : char { WIDTH_DESC = 'W', WIDTH_ASC = 'w', HEIGHT_DESC = 'H', HEIGHT_ASC = 'h', NONE = '-', INPUT = 'i' };

// common/Options.hpp:24-46: 0 = CALL, 1 = PUT; other values are rejected on read.
enum class OptionType : int8_t { CALL = 0, PUT = 1 };

inline std::ostream &operator<<(std::ostream &os, const OptionType t) { return os << static_cast<int>(t); }

inline std::istream &operator>>(std::istream &is, OptionType &t)
{
    int c;
    is >> c;
    t = static_cast<OptionType>(c);
    if (t != OptionType::CALL && t != OptionType::PUT) throw std::out_of_range("Invalid OptionType read from stream.");
    return is;
}

// Text arrays "[a, b, c]" (common/Arrays.hpp:15-46): read until ']', write with
// max_digits10 and std::fixed.
struct Arrays {
    template <class T, class = decltype(std::declval<std::istream &>() >> std::declval<T &>())>
    static void read_array(std::istream &in, std::vector<T> &array)
    {
        T x;
        char c;
        in >> c;
        while (!in.eof()) {
            in >> x >> c;
            array.push_back(x);
            if (c == ']') break;
        }
    }

    template <class T, class = decltype(std::declval<std::ostream &>() << std::declval<T>())>
    static void write_array(std::ostream &out, const std::vector<T> &array)
    {
        out.precision(std::numeric_limits<T>::max_digits10);
        if (array.empty()) {
            out << "[]" << std::endl;
            return;
        }
        out << '[' << std::fixed << array[0];
        for (size_t i = 1; i < array.size(); ++i) out << ", " << std::fixed << array[i];
        out << ']' << std::endl;
    }
};

// common/Options.hpp:48-125
struct Options {
    int N = 0;
    std::vector<double> StrikePrices, Maturities, Lengths;
    std::vector<uint16_t> TermUnits, TermStepCounts;
    std::vector<double> ReversionRates, Volatilities;
    std::vector<OptionType> Types;

    explicit Options(const int count)
    {
        N = count;
        StrikePrices.reserve(N); Maturities.reserve(N); Lengths.reserve(N); TermUnits.reserve(N);
        TermStepCounts.reserve(N); ReversionRates.reserve(N); Volatilities.reserve(N); Types.reserve(N);
    }

    // Reads a .in text file (or the library's binary cache) with the library's
    // threaded reader (hwt_read_options); same values as the stream reader.
    explicit Options(const std::string &filename)
    {
        if (filename.empty()) throw std::invalid_argument("File not specified.");
        hwt_options o;
        char err[512];
        const int rc = hwt_read_options(filename.c_str(), &o, err, (int)sizeof(err));
        if (rc != HWT_OK) {
            if (std::strncmp(err, "Invalid OptionType", 18) == 0) throw std::out_of_range(err);
            throw std::invalid_argument(err);
        }
        const size_t n = (size_t)o.n;
        StrikePrices.assign(o.strike, o.strike + n);
        Maturities.assign(o.bond_maturity, o.bond_maturity + n);
        Lengths.assign(o.option_maturity, o.option_maturity + n);
        TermUnits.assign(o.term_unit, o.term_unit + n);
        TermStepCounts.assign(o.term_steps, o.term_steps + n);
        ReversionRates.assign(o.a, o.a + n);
        Volatilities.assign(o.sigma, o.sigma + n);
        Types.resize(n);
        for (size_t i = 0; i < n; ++i) Types[i] = static_cast<OptionType>(o.type[i]);
        N = (int)n;
        hwt_free_options(&o);
    }

    // Writes the binary cache file the reader above recognises.
    void writeBinary(const std::string &filename) const
    {
        const hwt_options o = view();
        if (hwt_write_options_bin(filename.c_str(), &o) != HWT_OK)
            throw std::invalid_argument("cannot write '" + filename + "'");
    }

    void writeToFile(const std::string &filename) const
    {
        if (filename.empty()) throw std::invalid_argument("File not specified.");
        std::ofstream out(filename);
        if (!out) throw std::invalid_argument("File does not exist.");
        Arrays::write_array(out, StrikePrices);
        Arrays::write_array(out, Maturities);
        Arrays::write_array(out, Lengths);
        Arrays::write_array(out, TermUnits);
        Arrays::write_array(out, TermStepCounts);
        Arrays::write_array(out, ReversionRates);
        Arrays::write_array(out, Volatilities);
        Arrays::write_array(out, Types);
    }

    hwt_options view() const
    {
        hwt_options o;
        o.n = (int32_t)StrikePrices.size();
        o.strike = StrikePrices.data();
        o.bond_maturity = Maturities.data();
        o.option_maturity = Lengths.data();
        o.term_unit = TermUnits.data();
        o.term_steps = TermStepCounts.data();
        o.a = ReversionRates.data();
        o.sigma = Volatilities.data();
        o.type = reinterpret_cast<const int8_t *>(Types.data());
        return o;
    }
};

// common/Yield.hpp:14-40
struct Yield {
    int N = 0;
    std::vector<double> Prices;
    std::vector<int32_t> TimeSteps;

    Yield() = default;
    explicit Yield(const std::string &filename)
    {
        if (filename.empty()) throw std::invalid_argument("File not specified.");
        std::ifstream in(filename);
        if (!in) throw std::invalid_argument("File does not exist.");
        Arrays::read_array(in, Prices);
        Arrays::read_array(in, TimeSteps);
        N = (int)Prices.size();
        if (TimeSteps.size() != Prices.size()) throw std::invalid_argument("Yield file has arrays of different lengths.");
    }

    hwt_yield view() const
    {
        hwt_yield y;
        y.n = (int32_t)Prices.size();
        y.rate = Prices.data();
        y.day = TimeSteps.data();
        return y;
    }
};

// Owns one pricer context (stream, device buffers, tuned configuration).
class Pricer {
  public:
    explicit Pricer(int device = 0, const char *tune_cache = nullptr)
    {
        ctx_ = hwt_create(device, tune_cache);
        if (!ctx_) throw std::runtime_error("hwt_create failed with status " + std::to_string(hwt_create_status()));
    }
    ~Pricer() { hwt_destroy(ctx_); }
    Pricer(const Pricer &) = delete;
    Pricer &operator=(const Pricer &) = delete;

    hwt_ctx *handle() const { return ctx_; }

    void price(const Options &o, const Yield &y, std::vector<double> &results, const hwt_config &cfg,
               hwt_stats *stats = nullptr)
    {
        const hwt_options ov = o.view();
        const hwt_yield yv = y.view();
        results.resize(ov.n);
        const int rc = hwt_price_ex(ctx_, &ov, &yv, &cfg, results.data(), stats);
        if (rc == HWT_EINVAL) throw std::invalid_argument(hwt_last_error(ctx_));
        if (rc != HWT_OK) throw std::runtime_error(hwt_last_error(ctx_));
    }

  private:
    hwt_ctx *ctx_ = nullptr;
};

inline Pricer &default_pricer()
{
    static Pricer p(0);
    return p;
}

// seq::computeOptions(const Options&, const Yield&, std::vector<real>&)
// (seq/Seq.hpp:181-190), priced on the GPU in the chosen mode.
inline void computeOptions(const Options &options, const Yield &yield, std::vector<double> &results,
                           int mode = HWT_BATCHED_FP64)
{
    hwt_config cfg{};
    cfg.mode = mode;
    cfg.use_graph = 1;
    default_pricer().price(options, yield, results, cfg);
}

// KernelRunBase::run(options, yield, results, blockSize, sortType, isTest)
// (cuda-option/Kernel.cuh:303-314): runtime holds the last call's statistics.
class KernelRun {
  public:
    explicit KernelRun(int mode = HWT_BATCHED_FP64) : mode_(mode) {}
    hwt_stats runtime{};

    void run(const Options &options, const Yield &yield, std::vector<double> &results, const int blockSize = -1,
             const SortType sortType = SortType::NONE, const bool isTest = false)
    {
        hwt_config cfg{};
        cfg.mode = mode_;
        cfg.block_size = blockSize > 0 ? blockSize : 0;
        cfg.sort = static_cast<char>(sortType);
        cfg.use_graph = 1;
        default_pricer().price(options, yield, results, cfg, &runtime);
        if (isTest) {
            std::cout << "Priced " << results.size() << " options, block size " << runtime.block_size << ", "
                      << runtime.n_block_trees << " block trees, " << runtime.n_warp_tasks << " warp tasks"
                      << std::endl;
            std::cout << "Kernel executed in " << runtime.pricing_ms * 1000.0 << " microsec" << std::endl;
            std::cout << "Total execution time " << runtime.total_ms * 1000.0 << " microsec" << std::endl;
        }
    }

  private:
    int mode_;
};

}  // namespace hwtree
