// example_family.cpp -- the reference's board-family search (search.cpp's
// main with the AtomicCount searcher, src/search.cpp:36-53, 245-270) written
// against the C++ facade: read a Board<8> file, rank the combinations of
// distinct pieces of min_m..max_m cells (min_n..max_n of them) with Naming,
// and count, per rank, the configurations it tiles -- all configurations in
// one d4e_batch_sets batch.
//
//   example_family <board file> <min_m> <max_m> <min_n> <max_n> [C]
//
// C: one-sided pieces and rotations only (the reference's env C).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "board_family.h"

int main(int argc, char **argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s <board file> <min_m> <max_m> <min_n> <max_n> [C]\n",
                     argv[0]);
        return 2;
    }
    try {
        const auto board = d4e_host::Board<8>::from_file(argv[1]);
        const unsigned min_m = (unsigned)std::atoi(argv[2]), max_m = (unsigned)std::atoi(argv[3]);
        const unsigned min_n = (unsigned)std::atoi(argv[4]), max_n = (unsigned)std::atoi(argv[5]);
        const bool one_sided = argc > 6 && std::string(argv[6]) == "C";
        std::printf("working on a board of size=%d left=%zu count=%zu\n",
                    __builtin_popcountll(board.base), board.left(), board.count);
        std::vector<uint64_t> sizes;
        const auto pieces = d4e_host::pieces_by_size(min_m, max_m, one_sided, &sizes);
        const d4e_host::Naming naming(min_m, max_m, min_n, max_n, board.left(), sizes);
        std::printf("number of pieces combinations: %llu\n", (unsigned long long)naming.size());
        const auto t1 = std::chrono::steady_clock::now();
        const auto run = d4e_host::family_ledger(board, naming, pieces, one_sided);
        const auto t2 = std::chrono::steady_clock::now();
        uint64_t ranked = 0, total = 0, weighted = 0;
        for (uint64_t r = 0; r < run.ledger.size(); r++)
            if (run.ledger[r]) {
                ranked++;
                total += run.ledger[r];
                weighted += (r + 1) * run.ledger[r];
            }
        std::printf("configurations %llu, distinct boards %llu, sets %llu, tilings %llu\n",
                    (unsigned long long)run.configs, (unsigned long long)run.boards,
                    (unsigned long long)run.sets, (unsigned long long)run.tilings);
        for (uint64_t m : run.unsolved)
            std::printf("ZERO-count board 0x%016llx\n", (unsigned long long)m);
        std::printf("completed in %.3f ms\n",
                    std::chrono::duration<double, std::milli>(t2 - t1).count());
        std::printf("ledger %llu %llu %llu\n", (unsigned long long)ranked,
                    (unsigned long long)total, (unsigned long long)weighted);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
