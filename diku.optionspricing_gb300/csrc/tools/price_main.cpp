// hwt-price: command-line pricer with the reference drivers' flags
// (common/Args.hpp:38-45; seq/SeqMain.cpp, cuda-option/CudaOptionMain.cu):
//   -o|--options FILE   option records (.in)
//   -y|--yield FILE     yield curve (.in)
//   -v|--version M ...  pricing mode(s): 0 plain FP64, 1 batched FP64 (default),
//                       2 batched FP32, 3 batched mixed, 4 batched double-float
//   -b|--block B ...    threads per block-tree block (the reference's -b)
//   -s|--sort S ...     schedule order W w H h - i (results do not depend on it)
//   -r|--runs R         time R runs and print "mode,block,sort,kernel_us,total_us,bytes"
//   -d|--device D       CUDA device
//   -t|--test           human-readable timing instead of the price array
//   -w|--write-bin FILE write the options as a binary cache file (read back by -o) and exit
// Without -r the prices are printed as one "[p0, p1, ...]" array, the format
// test/Compare reads.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "hwtree.hpp"

namespace {

struct Args {
    std::string options, yield, write_bin;
    std::vector<int> modes, blocks;
    std::vector<char> sorts;
    int runs = 0, device = 0;
    bool test = false;
};

bool is_flag(const char *s) { return s[0] == '-' && s[1] != '\0' && !(s[1] >= '0' && s[1] <= '9') && s[1] != '.'; }

Args parse(int argc, char **argv)
{
    Args a;
    for (int i = 1; i < argc; ++i) {
        std::string f = argv[i];
        auto many = [&](auto push) {
            while (i + 1 < argc && (!is_flag(argv[i + 1]) || std::string(argv[i + 1]) == "-")) push(argv[++i]);
        };
        auto one = [&]() -> std::string {
            if (i + 1 >= argc) throw std::invalid_argument("missing value for " + f);
            return argv[++i];
        };
        if (f == "-o" || f == "--options") a.options = one();
        else if (f == "-y" || f == "--yield") a.yield = one();
        else if (f == "-v" || f == "--version") many([&](const char *v) { a.modes.push_back(std::atoi(v)); });
        else if (f == "-b" || f == "--block") many([&](const char *v) { a.blocks.push_back(std::atoi(v)); });
        else if (f == "-s" || f == "--sort") many([&](const char *v) {
            const char c = v[0];
            if (std::strlen(v) == 1 && (c == 'W' || c == 'w' || c == 'H' || c == 'h' || c == '-' || c == 'i')) a.sorts.push_back(c);
        });
        else if (f == "-r" || f == "--runs") a.runs = std::atoi(one().c_str());
        else if (f == "-d" || f == "--device") a.device = std::atoi(one().c_str());
        else if (f == "-t" || f == "--test") a.test = true;
        else if (f == "-w" || f == "--write-bin") a.write_bin = one();
        else throw std::invalid_argument("unknown flag " + f);
    }
    if (a.modes.empty()) a.modes.push_back(HWT_BATCHED_FP64);
    if (a.blocks.empty()) a.blocks.push_back(-1);
    if (a.sorts.empty()) a.sorts.push_back('-');
    return a;
}

}  // namespace

int main(int argc, char **argv)
{
    try {
        const Args args = parse(argc, argv);
        if (args.test) std::cout << "Loading options " << args.options << ", yield " << args.yield << std::endl;
        hwtree::Options options(args.options);
        if (!args.write_bin.empty()) {
            options.writeBinary(args.write_bin);
            return 0;
        }
        hwtree::Yield yield(args.yield);
        hwtree::Pricer pricer(args.device);
        for (int mode : args.modes) {
            for (int block : args.blocks) {
                for (char sort : args.sorts) {
                    hwt_config cfg{};
                    cfg.mode = mode;
                    cfg.block_size = block > 0 ? block : 0;
                    cfg.sort = sort;
                    cfg.use_graph = 1;
                    std::vector<double> results;
                    if (args.runs > 0) {
                        double best_k = 1e300, best_t = 1e300;
                        hwt_stats st{};
                        for (int r = 0; r < args.runs; ++r) {
                            pricer.price(options, yield, results, cfg, &st);
                            if (st.pricing_ms < best_k) best_k = st.pricing_ms;
                            if (st.total_ms < best_t) best_t = st.total_ms;
                        }
                        if (args.test)
                            std::cout << "Best times: kernel " << (long long)(best_k * 1000) << " microsec, total "
                                      << (long long)(best_t * 1000) << " microsec." << std::endl;
                        else
                            std::cout << mode << ',' << st.block_size << ',' << sort << ',' << (long long)(best_k * 1000)
                                      << ',' << (long long)(best_t * 1000) << ',' << st.device_bytes << std::endl;
                    } else {
                        hwt_stats st{};
                        pricer.price(options, yield, results, cfg, &st);
                        if (args.test)
                            std::cout << "Mode " << mode << ": kernel " << st.pricing_ms * 1000 << " microsec, total "
                                      << st.total_ms * 1000 << " microsec, " << st.n_block_trees << " block trees, "
                                      << st.n_warp_tasks << " warp tasks" << std::endl;
                        else
                            hwtree::Arrays::write_array(std::cout, results);
                    }
                }
            }
        }
    } catch (const std::exception &e) {
        std::cerr << "hwt-price: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}
