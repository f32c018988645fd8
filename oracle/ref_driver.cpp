// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Command-line driver around the reference's own CPU solver.  oracle/Makefile
// compiles it together with the reference sources where they lie
// (src/Piece.cpp, src/Shape.cpp, src/Group.cpp, src/known1.cpp,
// src/known2.cpp) into oracle/_ref/d4ref.  It is used only to generate and
// check the golden fixtures under tests/golden/.
//
// stdin:
//   W H sym mode            mode = count | all | one | catalogue
//   H row masks (decimal, bit c = column c must be covered)
//   n
//   n lines: shape count    (shape in Shape<8> layout, bit 8*r + c)
// stdout (count): "count N"
// stdout (all/one): "solutions N" then one line per solution with W*H type
//   ids followed by W*H step ids (row-major; -1 outside the board).
// stdout (catalogue): for m = 1..8: "free m v0 v1 ..." and "onesided m ...",
//   the reference's known_shapes / known_C_shapes tables.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "Piece.hpp"
#include "known.hpp"

template <size_t L>
static int run(int W, int H, unsigned sym, const std::string &mode,
               const std::vector<unsigned> &rows,
               const std::vector<std::pair<uint64_t, unsigned>> &pcs) {
    Shape<L> board{ 0u };
    for (int r = 0; r < H; r++)
        for (int c = 0; c < W; c++)
            if ((rows[r] >> c) & 1u)
                board = board.set(r, c);
    std::vector<Piece<L>> lib;
    for (auto [v, cnt] : pcs) {
        lib.emplace_back(Shape<8>{ v }.to<L>(), sym);
        lib.back().count = cnt;
    }
    if (mode == "count") {
        std::printf("count %zu\n", solve_count(lib, board));
        return 0;
    }
    auto sols = solve(lib, board, mode == "one");
    std::printf("solutions %zu\n", sols.size());
    for (auto &s : sols) {
        std::string line;
        for (int r = 0; r < H; r++)
            for (int c = 0; c < W; c++) {
                auto id = s.map[r][c];
                line += std::to_string(id < 0 ? -1 : (long)s.steps[id].piece_id) + " ";
            }
        for (int r = 0; r < H; r++)
            for (int c = 0; c < W; c++)
                line += std::to_string((long)s.map[r][c]) + " ";
        std::printf("%s\n", line.c_str());
    }
    return 0;
}

int main() {
    int W, H;
    unsigned sym;
    std::string mode;
    if (!(std::cin >> W >> H >> sym >> mode))
        return 2;
    if (mode == "catalogue") {
        for (int m = 1; m <= 8; m++) {
            std::printf("free %d", m);
            for (size_t i = 0; i < shapes_count[m]; i++)
                std::printf(" %llu", (unsigned long long)known_shapes[m][i]);
            std::printf("\nonesided %d", m);
            for (size_t i = 0; i < shapes_C_count[m]; i++)
                std::printf(" %llu", (unsigned long long)known_C_shapes[m][i]);
            std::printf("\n");
        }
        return 0;
    }
    std::vector<unsigned> rows(H);
    for (auto &r : rows)
        std::cin >> r;
    int n;
    std::cin >> n;
    std::vector<std::pair<uint64_t, unsigned>> pcs(n);
    for (auto &[v, c] : pcs)
        std::cin >> v >> c;
    if (W <= 8 && H <= 8)
        return run<8>(W, H, sym, mode, rows, pcs);
    if (W <= 11 && H <= 11)
        return run<11>(W, H, sym, mode, rows, pcs);
    std::fprintf(stderr, "board %dx%d does not fit Shape<11>\n", W, H);
    return 3;
}
