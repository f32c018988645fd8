// geometry.h -- host-side polyomino geometry and placement ("frow") tables.
//
// Shapes use the reference's Shape<8> layout: a uint64 with bit 8*r + c for
// cell (r, c) (src/Shape.hpp:20-24).  Transform index t follows
// Shape::transforms() (src/Shape.cpp:28-40): bit0 = flip X, bit1 = flip Y,
// bit2 = swap axes.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "d4e_types.h"

namespace d4e {

uint64_t shape_normalize(uint64_t v);
uint64_t shape_transform(uint64_t v, int t);           // normalized result
uint64_t shape_canonical(uint64_t v, unsigned forms);  // min over allowed transforms
bool shape_connected(uint64_t v);

// The reference's polyomino catalogues (src/known.hpp): free polyominoes
// (canonical under D4) and one-sided ones (canonical under C4), sorted by
// value, regenerated here by growing shapes cell by cell.
const std::vector<uint64_t> &catalogue_free(int m);      // m = 1..8
const std::vector<uint64_t> &catalogue_onesided(int m);  // m = 1..8

// A piece library with the placements of every piece anchored at every column
// of a board of the given width.  Restates compute_frow_on_cpu
// (src/frow.cpp:39-166) with whole-row fills enumerated on the device instead
// of precomputed L/R half-row combinations.
struct PieceLib {
    std::vector<uint64_t> shapes;   // Shape<8> values, one per type
    std::vector<uint32_t> counts;   // copies per type
    uint32_t sym = 0xFFu;
    uint32_t width = 8;
    uint32_t win_rows = 8;          // 64 / width
    uint32_t copies = 0;            // sum of counts
    uint32_t max_piece_rows = 0;
    uint32_t used_bits = 0;         // bits of the per-type binary copy counters
    uint32_t dyn_bits = 0;          // width * (max_piece_rows - 1)
    std::vector<TypeField> fields;       // copy counter per type
    std::vector<Plc> plc;                // grouped by anchor column
    std::vector<uint16_t> plc_type;      // type id per placement
    std::vector<uint32_t> plc_orient;    // transform index per placement
    uint16_t col_off[kMaxWidth] = {};
    uint16_t col_len[kMaxWidth] = {};
    // Candidate filters (see InstDesc): bitsets of `fwords` u64 words.
    uint32_t fwords = 1;
    uint32_t f0_off[kMaxWidth] = {};
    uint32_t f1_off[kMaxWidth] = {};
    uint32_t f2_off[kMaxWidth] = {};
    std::vector<uint64_t> filters;
};

// Builds the tables; returns an empty string on success, else the reason.
std::string build_piece_lib(const uint64_t *shapes, const uint32_t *counts, uint32_t n,
                            uint32_t sym, uint32_t width, PieceLib &out);

// Board symmetry-aware canonical D4 form of a solution grid (row-major, W x H
// type ids, -1 outside the board): lexicographic minimum over the transforms
// that map the board onto itself.
void canonical_grid(uint32_t width, uint32_t height, const uint8_t *rows,
                    const int8_t *grid, int8_t *out);

}  // namespace d4e
