// The C++ board-family facade (host/board_family.h) run on the CPU, with
// the three engine calls it makes answered by the oracle: d4e_catalogue
// from a piece table, d4e_batch_sets by the oracle's solver over every
// multiset within the counts.  Checks the facade's host logic (ranking,
// ledgers, ledger files, resume); the GPU tests check the real engine.
//
//   family_file_sim <pieces file> <board file> <min_m> <max_m> <min_n> <max_n>
//                   ac | fb <file> [per_batch] [max_batches] | fB <file> ...
// pieces file: lines "m v" (a piece of m cells, Shape<8> value), in
// catalogue order.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <string>
#include <vector>

#include "board_family.h"
#include "../oracle/d4oracle.h"

static std::vector<std::vector<uint64_t>> g_pieces(64);

extern "C" const char *d4e_last_error(void) { return "oracle stub"; }

extern "C" int d4e_catalogue(uint32_t m, int32_t, uint64_t *out, uint32_t max, uint32_t *n) {
    const auto &v = g_pieces.at(m);
    *n = (uint32_t)v.size();
    for (uint32_t i = 0; out && i < v.size() && i < max; i++)
        out[i] = v[i];
    return D4E_OK;
}

extern "C" int d4e_batch_sets(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *,
                              d4e_result *results, uint64_t *offs, uint8_t *copies,
                              uint64_t *tilings, uint64_t max_sets, d4e_stats *) {
    std::vector<std::vector<uint8_t>> rows;
    std::vector<uint64_t> til;
    for (uint32_t k = 0; k < n; k++) {
        const d4e_instance &in = insts[k];
        offs[k] = rows.size();
        int cells = 0;
        std::vector<uint16_t> brows(in.height);
        for (uint32_t r = 0; r < in.height; r++) {
            brows[r] = in.rows[r];
            cells += __builtin_popcount(in.rows[r]);
        }
        std::vector<uint32_t> c(in.n_pieces, 0);
        std::function<void(uint32_t, int)> walk = [&](uint32_t p, int area) {
            if (p == in.n_pieces) {
                if (area != cells)
                    return;
                or_problem q{(int32_t)in.width, (int32_t)in.height, brows.data(),
                             (int32_t)in.n_pieces, in.shapes, c.data(), in.sym};
                const int64_t t = or_solve_count(&q);
                if (t > 0) {
                    rows.emplace_back(c.begin(), c.end());
                    til.push_back((uint64_t)t);
                }
                return;
            }
            for (uint32_t x = 0; x <= in.counts[p]; x++) {
                c[p] = x;
                walk(p + 1, area + (int)x * __builtin_popcountll(in.shapes[p]));
            }
            c[p] = 0;
        };
        walk(0, 0);
        results[k] = d4e_result{};
        results[k].status = D4E_OK;
        results[k].latency_ms = 1.0 + k;
    }
    offs[n] = rows.size();
    if (rows.size() > max_sets)
        return D4E_ERR_INVALID;
    for (size_t s = 0; s < rows.size(); s++) {
        std::fill(copies + s * D4E_SET_PIECES, copies + (s + 1) * D4E_SET_PIECES, 0);
        std::copy(rows[s].begin(), rows[s].end(), copies + s * D4E_SET_PIECES);
        tilings[s] = til[s];
    }
    return D4E_OK;
}

static void print_ledger(uint64_t names, const std::function<uint64_t(uint64_t)> &at) {
    uint64_t ranked = 0, total = 0, weighted = 0;
    for (uint64_t r = 0; r < names; r++)
        if (const uint64_t v = at(r)) {
            ranked++;
            total += v;
            weighted += (r + 1) * v;
        }
    std::printf("ledger %llu %llu %llu\n", (unsigned long long)ranked, (unsigned long long)total,
                (unsigned long long)weighted);
}

int main(int argc, char **argv) {
    if (argc < 8)
        return 2;
    std::ifstream pf(argv[1]);
    uint64_t m = 0, v = 0;
    while (pf >> m >> v)
        g_pieces.at(m).push_back(v);
    try {
        const auto board = d4e_host::Board<8>::from_file(argv[2]);
        const unsigned min_m = (unsigned)std::atoi(argv[3]), max_m = (unsigned)std::atoi(argv[4]);
        const unsigned min_n = (unsigned)std::atoi(argv[5]), max_n = (unsigned)std::atoi(argv[6]);
        const std::string mode = argv[7];
        std::vector<uint64_t> sizes;
        const auto pieces = d4e_host::pieces_by_size(min_m, max_m, false, &sizes);
        const d4e_host::Naming naming(min_m, max_m, min_n, max_n, board.left(), sizes);
        if (mode == "ac") {
            const auto run = d4e_host::family_ledger(board, naming, pieces, false);
            for (uint64_t b : run.unsolved)
                std::printf("ZERO-count board 0x%016llx\n", (unsigned long long)b);
            print_ledger(naming.size(), [&](uint64_t r) { return run.ledger[r]; });
            return 0;
        }
        if (argc < 9)
            return 2;
        const uint64_t per_batch = argc > 9 ? std::strtoull(argv[9], nullptr, 0) : 1024;
        const uint64_t max_batches = argc > 10 ? std::strtoull(argv[10], nullptr, 0) : 0;
        d4e_host::LedgerFile file(argv[8], board.count, naming.size(),
                                  mode == "fB" ? d4e_host::LedgerKind::Byte
                                               : d4e_host::LedgerKind::Bit);
        const auto run = d4e_host::family_ledger_file(board, naming, pieces, false, file,
                                                      per_batch, 0, 0, max_batches);
        std::printf("previously %llu now %llu batches %llu\n",
                    (unsigned long long)run.previously_solved,
                    (unsigned long long)run.solved_now, (unsigned long long)run.batches);
        for (uint64_t i : run.unsolved)
            std::printf("ZERO-count board 0x%016llx\n", (unsigned long long)file.config(i).shape);
        print_ledger(naming.size(), [&](uint64_t r) { return file.tiled(r); });
    } catch (const std::exception &e) {
        std::printf("error %s\n", e.what());
        return 3;
    }
    return 0;
}
