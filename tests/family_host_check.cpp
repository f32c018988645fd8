// Host-only check of the C++ board-family facade (no GPU, no libd4e calls):
//   family_host_check board <file>
//     prints base, regions, count, left and every configuration (hex)
//   family_host_check naming <min_m> <max_m> <min_n> <max_n> <tgt> <size_min_m> ... <size_max_m>
//     prints the size, then every rank's pieces as m:i, checking name(resolve(r)) == r
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "board_family.h"

int main(int argc, char **argv) {
    if (argc >= 3 && std::string(argv[1]) == "board") {
        const auto b = d4e_host::Board<8>::from_file(argv[2]);
        std::printf("base %llx\n", (unsigned long long)b.base);
        for (uint64_t r : b.regions)
            std::printf("region %llx\n", (unsigned long long)r);
        std::printf("count %zu left %zu\n", b.count, b.left());
        b.foreach([](uint64_t m) { std::printf("config %llx\n", (unsigned long long)m); });
        return 0;
    }
    if (argc >= 7 && std::string(argv[1]) == "naming") {
        const uint64_t min_m = std::strtoull(argv[2], nullptr, 0), max_m = std::strtoull(argv[3], nullptr, 0);
        const uint64_t min_n = std::strtoull(argv[4], nullptr, 0), max_n = std::strtoull(argv[5], nullptr, 0);
        const uint64_t tgt = std::strtoull(argv[6], nullptr, 0);
        std::vector<uint64_t> sizes(max_m + 1, 0);
        for (uint64_t m = min_m; m <= max_m && (int)(7 + m - min_m) < argc; m++)
            sizes[m] = std::strtoull(argv[7 + m - min_m], nullptr, 0);
        const d4e_host::Naming nm(min_m, max_m, min_n, max_n, tgt, sizes);
        std::printf("size %llu\n", (unsigned long long)nm.size());
        for (uint64_t r = 0; r < nm.size(); r++) {
            std::vector<std::vector<char>> ch(max_m + 1);
            for (uint64_t m = 0; m <= max_m; m++)
                ch[m].assign(sizes[m], 0);
            std::printf("rank %llu:", (unsigned long long)r);
            nm.resolve(r, [&](uint64_t m, uint64_t i) {
                ch[m][i] = 1;
                std::printf(" %llu:%llu", (unsigned long long)m, (unsigned long long)i);
            });
            std::printf("\n");
            const auto back = nm.name([&](uint64_t m, uint64_t i) { return ch[m][i] != 0; });
            if (!back || *back != r) {
                std::printf("roundtrip failed at %llu\n", (unsigned long long)r);
                return 1;
            }
        }
        std::printf("roundtrip ok\n");
        return 0;
    }
    if (argc >= 6 && std::string(argv[1]) == "ledgerfile") {
        // ledgerfile <path> <configs> <names> <bit|byte>: opens (creating or
        // resuming) and, for every configuration not yet solved, logs the
        // ranks r with (r + i) % 3 == 0 and marks it solved; prints what it did
        // and the file's state.
        const uint64_t configs = std::strtoull(argv[3], nullptr, 0);
        const uint64_t names = std::strtoull(argv[4], nullptr, 0);
        const auto kind = std::string(argv[5]) == "byte" ? d4e_host::LedgerKind::Byte
                                                         : d4e_host::LedgerKind::Bit;
        try {
            d4e_host::LedgerFile f(argv[2], configs, names, kind);
            uint64_t skipped = 0;
            for (uint64_t i = 0; i < configs; i++) {
                auto &c = f.config(i);
                if (c.solved) {
                    skipped++;
                    continue;
                }
                c.shape = 0x1000 + i;
                uint64_t n = 0;
                for (uint64_t r = 0; r < names; r++)
                    if ((r + i) % 3 == 0)
                        n += f.log(r, i) ? 1u : 0u;
                // a second log of the same pair is not new
                if (names && f.log((3 - i % 3) % 3 < names ? (3 - i % 3) % 3 : 0, i))
                    n += 1000;
                c.count = n;
                c.solved = 1 + i;
                if (i == 1 && argc > 6 && std::string(argv[6]) == "stop")
                    break;
            }
            f.sync();
            std::printf("skipped %llu bytes %llu\n", (unsigned long long)skipped,
                        (unsigned long long)f.bytes());
            for (uint64_t r = 0; r < names; r++)
                std::printf("tiled %llu %llu\n", (unsigned long long)r,
                            (unsigned long long)f.tiled(r));
        } catch (const std::exception &e) {
            std::printf("error %s\n", e.what());
            return 3;
        }
        return 0;
    }
    std::fprintf(stderr, "usage: board <file> | naming <min_m> <max_m> <min_n> <max_n> <tgt> <sizes...>"
                         " | ledgerfile <path> <configs> <names> <bit|byte> [stop]\n");
    return 2;
}
