// example_family.cpp -- the reference's board-family search (search.cpp's
// main, src/search.cpp:245-330) written against the C++ facade: read a
// Board<8> file, rank the combinations of distinct pieces of min_m..max_m
// cells (min_n..max_n of them) with Naming, and find, for every
// configuration, the ranked combinations that tile it -- many
// configurations per d4e_batch_sets batch.
//
//   [S=v|ac|fb|fB] [C=1] example_family <board file> <min_m> <max_m> <min_n> <max_n> [ledger file]
//
// S=v: the Verify searcher (the number of (configuration, combination) pairs
// found, no ledger).
// S=ac (default): the AtomicCount ledger in memory (configurations per rank).
// S=fb / S=fB: the FileBit / FileByte ledger file, resumed if it exists.
// C=1: one-sided pieces and rotations only (the reference's env C).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>

#include "board_family.h"

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
    if (argc < 6) {
        std::fprintf(stderr,
                     "usage: [S=v|ac|fb|fB] [C=1] %s <board file> <min_m> <max_m> <min_n> <max_n>"
                     " [ledger file]\n",
                     argv[0]);
        return 2;
    }
    const char *env_s = std::getenv("S");
    const std::string mode = env_s && *env_s ? env_s : "ac";
    const char *env_c = std::getenv("C");
    const bool one_sided = env_c && *env_c;
    if (mode != "v" && mode != "ac" && mode != "fb" && mode != "fB") {
        std::fprintf(stderr, "set env S to v|ac|fb|fB\n");
        return 2;
    }
    if ((mode == "fb" || mode == "fB") && argc < 7) {
        std::fprintf(stderr, "S=%s needs a ledger file\n", mode.c_str());
        return 2;
    }
    try {
        const auto board = d4e_host::Board<8>::from_file(argv[1]);
        const unsigned min_m = (unsigned)std::atoi(argv[2]), max_m = (unsigned)std::atoi(argv[3]);
        const unsigned min_n = (unsigned)std::atoi(argv[4]), max_n = (unsigned)std::atoi(argv[5]);
        std::printf("working on a board of size=%d left=%zu count=%zu\n",
                    __builtin_popcountll(board.base), board.left(), board.count);
        std::vector<uint64_t> sizes;
        const auto pieces = d4e_host::pieces_by_size(min_m, max_m, one_sided, &sizes);
        const d4e_host::Naming naming(min_m, max_m, min_n, max_n, board.left(), sizes);
        std::printf("number of pieces combinations: %llu\n", (unsigned long long)naming.size());
        const auto t1 = std::chrono::steady_clock::now();
        if (mode == "v") {
            const auto run = d4e_host::family_ledger(board, naming, pieces, one_sided);
            uint64_t work = 0;
            for (uint64_t v : run.ledger)
                work += v;
            const auto t2 = std::chrono::steady_clock::now();
            std::printf("%llu/%llu configurations tiled, %llu work done in %.3f ms\n",
                        (unsigned long long)(run.configs - run.unsolved.size()),
                        (unsigned long long)run.configs, (unsigned long long)work,
                        std::chrono::duration<double, std::milli>(t2 - t1).count());
        } else if (mode == "ac") {
            const auto run = d4e_host::family_ledger(board, naming, pieces, one_sided);
            std::printf("configurations %llu, distinct boards %llu, sets %llu, tilings %llu\n",
                        (unsigned long long)run.configs, (unsigned long long)run.boards,
                        (unsigned long long)run.sets, (unsigned long long)run.tilings);
            for (uint64_t m : run.unsolved)
                std::printf("ZERO-count board 0x%016llx\n", (unsigned long long)m);
            const auto t2 = std::chrono::steady_clock::now();
            std::printf("completed in %.3f ms\n",
                        std::chrono::duration<double, std::milli>(t2 - t1).count());
            print_ledger(naming.size(), [&](uint64_t r) { return run.ledger[r]; });
        } else {
            d4e_host::LedgerFile file(argv[6], board.count, naming.size(),
                                      mode == "fB" ? d4e_host::LedgerKind::Byte
                                                   : d4e_host::LedgerKind::Bit);
            std::printf("file size: %llu B\n", (unsigned long long)file.bytes());
            const auto run = d4e_host::family_ledger_file(board, naming, pieces, one_sided, file);
            std::printf("%llu/%llu configs were previously solved; solved now %llu in %llu "
                        "batches\n",
                        (unsigned long long)run.previously_solved, (unsigned long long)run.configs,
                        (unsigned long long)run.solved_now, (unsigned long long)run.batches);
            for (uint64_t i : run.unsolved)
                std::printf("ZERO-count board 0x%016llx\n",
                            (unsigned long long)file.config(i).shape);
            const auto t2 = std::chrono::steady_clock::now();
            std::printf("completed in %.3f ms\n",
                        std::chrono::duration<double, std::milli>(t2 - t1).count());
            print_ledger(naming.size(), [&](uint64_t r) { return file.tiled(r); });
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
