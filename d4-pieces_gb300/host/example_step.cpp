// example_step.cpp -- the reference's caller loop (Searcher::step,
// src/searcher.cpp:16-36) written against the C++ facade: build the frow
// tables once, then one CudaSearcher per board, search_GPU() until the
// height reaches 0.  Unlike the reference (which ends in std::terminate()),
// it prints the exact tiling count.
//
//   example_step <empty_area as decimal or 0x-hex> <min_m> <max_m> [C]
//
// Uses every free (or, with C, one-sided) polyomino of min_m..max_m cells
// once, like the reference's Naming over known_shapes.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "searcher_cuda.h"

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <empty_area> <min_m> <max_m> [C]\n", argv[0]);
        return 2;
    }
    const uint64_t empty_area = std::strtoull(argv[1], nullptr, 0);
    const unsigned min_m = (unsigned)std::atoi(argv[2]), max_m = (unsigned)std::atoi(argv[3]);
    const bool one_sided = argc > 4 && std::string(argv[4]) == "C";
    try {
        std::vector<uint64_t> shapes;
        for (unsigned m = min_m; m <= max_m; m++) {
            uint32_t n = 0;
            d4e_host::check(d4e_catalogue(m, one_sided, nullptr, 0, &n));
            std::vector<uint64_t> v(n);
            d4e_host::check(d4e_catalogue(m, one_sided, v.data(), n, &n));
            shapes.insert(shapes.end(), v.begin(), v.end());
        }
        d4e_host::set_piece_library(shapes, std::vector<uint32_t>(shapes.size(), 1u),
                                    one_sided ? 0b01101001u : 0xFFu);
        d4e_host::compute_frow_on_cpu(false);
        d4e_host::transfer_frow_to_gpu();
        d4e_host::CudaSearcher cs{ empty_area };
        while (cs.get_height()) {
            std::printf("height=%u size=%llu next=%llu\n", cs.get_height(),
                        (unsigned long long)cs.size(), (unsigned long long)cs.next_size());
            auto t1 = std::chrono::steady_clock::now();
            cs.search_GPU();
            auto t2 = std::chrono::steady_clock::now();
            std::printf("  => completed in %.3f ms\n",
                        std::chrono::duration<double, std::milli>(t2 - t1).count());
        }
        std::printf("count %llu\n", (unsigned long long)cs.count());
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
