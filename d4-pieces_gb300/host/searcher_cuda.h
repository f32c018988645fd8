// searcher_cuda.h -- C++ facade of the GB300 tiling engine with the
// reference's host API (b1f6c1c4/d4-pieces src/searcher_cuda.h:10-38 and
// src/frow.h:8-12), implemented over the C ABI in include/d4e.h.
//
// Differences a caller of the reference sees:
//  * the piece library is explicit (set_piece_library) instead of the
//    g_nme / g_sym globals read by compute_frow_on_cpu (src/frow.cpp:13-15);
//  * results are exact tiling counts with piece multiplicities
//    (count()), and boards may be taller than 8 rows (the rows constructor);
//  * size(i) counts states whose current row equals the 8-bit pattern i, the
//    reference's 256 `ea` buckets.
// Errors throw std::runtime_error, as the reference's THROW / C() do
// (src/util.hpp:73-74, src/util.cuh:23-40).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/d4e.h"

namespace d4e_host {

inline void check(int rc) {
    if (rc != D4E_OK)
        throw std::runtime_error(std::string("d4e: ") + d4e_last_error());
}

// Global piece library and tables, like the reference's g_nme / g_sym and
// h_frowInfoL/R / d_frowDataL/R globals.
struct FrowState {
    std::vector<uint64_t> shapes;
    std::vector<uint32_t> counts;
    unsigned sym = 0xFFu;
    d4e_frow *frow = nullptr;
};

inline FrowState &frow_state() {
    static FrowState s;
    return s;
}

inline void set_piece_library(std::vector<uint64_t> shapes, std::vector<uint32_t> counts,
                              unsigned sym = 0xFFu) {
    auto &s = frow_state();
    s.shapes = std::move(shapes);
    s.counts = std::move(counts);
    s.sym = sym;
}

// compute_frow_on_cpu(bool show_report) -- src/frow.h:10.
inline void compute_frow_on_cpu(bool show_report = true) {
    auto &s = frow_state();
    if (s.frow) {
        d4e_frow_destroy(s.frow);
        s.frow = nullptr;
    }
    check(d4e_frow_create(s.shapes.data(), s.counts.data(), (uint32_t)s.shapes.size(), s.sym, 8,
                          show_report ? 1 : 0, &s.frow));
}

// transfer_frow_to_gpu() -- src/frow.h:11.
inline void transfer_frow_to_gpu(int device = 0) {
    auto &s = frow_state();
    if (!s.frow)
        throw std::runtime_error("d4e: compute_frow_on_cpu() first");
    check(d4e_frow_transfer(s.frow, device));
}

// show_gpu_devices() -- src/frow.h:12.
inline void show_gpu_devices() { check(d4e_show_gpu_devices()); }

// struct CudaSearcher -- src/searcher_cuda.h:10-38.
class CudaSearcher {
public:
    explicit CudaSearcher(uint64_t empty_area) {
        check(d4e_searcher_create(frow(), empty_area, &s_));
    }
    CudaSearcher(const std::vector<uint8_t> &rows, bool keep_levels = false) {
        check(d4e_searcher_create_board(frow(), (uint32_t)rows.size(), rows.data(),
                                        keep_levels ? D4E_KEEP_LEVELS : 0u, &s_));
    }
    ~CudaSearcher() { d4e_searcher_destroy(s_); }
    CudaSearcher(const CudaSearcher &) = delete;
    CudaSearcher &operator=(const CudaSearcher &) = delete;

    [[nodiscard]] uint32_t get_height() const {
        uint32_t h = 0;
        check(d4e_searcher_get_height(s_, &h));
        return h;
    }
    [[nodiscard]] uint64_t size(unsigned i) const {
        uint64_t n = 0;
        check(d4e_searcher_bucket_size(s_, i, &n));
        return n;
    }
    [[nodiscard]] uint64_t size() const {
        uint64_t n = 0;
        check(d4e_searcher_size(s_, &n));
        return n;
    }
    [[nodiscard]] uint64_t next_size() const {
        uint64_t n = 0;
        check(d4e_searcher_next_size(s_, &n));
        return n;
    }
    void search_GPU() { check(d4e_searcher_search_GPU(s_)); }

    // Extensions over the reference's searcher.
    [[nodiscard]] uint64_t count() const {
        uint64_t n = 0;
        check(d4e_searcher_count(s_, &n));
        return n;
    }
    [[nodiscard]] d4e_stats stats() const {
        d4e_stats st{};
        check(d4e_searcher_stats(s_, &st));
        return st;
    }

private:
    static const d4e_frow *frow() {
        auto &s = frow_state();
        if (!s.frow)
            throw std::runtime_error("d4e: compute_frow_on_cpu() first");
        return s.frow;
    }
    d4e_searcher *s_ = nullptr;
};

}  // namespace d4e_host
