// geometry.cpp -- host-side polyomino geometry and placement tables.
#include "geometry.h"

#include <algorithm>
#include <array>
#include <cstring>
#include <mutex>
#include <set>

namespace d4e {

uint64_t shape_normalize(uint64_t v) {
    if (!v)
        return 0;
    while (!(v & 0xFFull))
        v >>= 8;
    while (!(v & 0x0101010101010101ull))
        v >>= 1;
    return v;
}

uint64_t shape_transform(uint64_t v, int t) {
    const bool sw = (t >> 2) & 1, fx = t & 1, fy = (t >> 1) & 1;
    uint64_t out = 0;
    for (uint64_t bits = v; bits; bits &= bits - 1) {
        const int b = __builtin_ctzll(bits);
        const int r = b / 8, c = b % 8;
        // out(orow, ocol) = in(r, c) with in_row = Swap ? ocol : orow, etc.
        int orow = r, ocol = c;
        if (fy)
            orow = 7 - orow;
        if (fx)
            ocol = 7 - ocol;
        if (sw)
            std::swap(orow, ocol);
        out |= 1ull << (orow * 8 + ocol);
    }
    return shape_normalize(out);
}

uint64_t shape_canonical(uint64_t v, unsigned forms) {
    uint64_t best = ~0ull;
    for (int t = 0; t < 8; t++, forms >>= 1)
        if (forms & 1u)
            best = std::min(best, shape_transform(v, t));
    return best;
}

bool shape_connected(uint64_t v) {
    if (!v)
        return false;
    uint64_t seen = v & (~v + 1);
    for (;;) {
        uint64_t grow = seen | (seen << 8) | (seen >> 8) |
                        ((seen << 1) & ~0x0101010101010101ull) |
                        ((seen >> 1) & ~0x8080808080808080ull);
        grow &= v;
        if (grow == seen)
            return seen == v;
        seen = grow;
    }
}

namespace {

constexpr unsigned kFormsD4 = 0xFFu;
constexpr unsigned kFormsReflections = 0b10010110u;  // flip X, flip Y, flip primary, flip secondary

struct Catalogue {
    std::array<std::vector<uint64_t>, 9> free_, onesided;
    Catalogue() {
        // Grow free polyominoes one cell at a time inside the 8x8 frame.
        std::set<uint64_t> level{1ull};
        free_[1] = {1ull};
        for (int m = 2; m <= 8; m++) {
            std::set<uint64_t> next;
            for (uint64_t s : level) {
                // Cells are shifted by one row/column so that growth to the
                // top/left stays representable before re-normalizing.
                for (int dr = 0; dr <= 1; dr++)
                    for (int dc = 0; dc <= 1; dc++) {
                        uint64_t shifted = 0;
                        bool ok = true;
                        for (uint64_t bits = s; bits; bits &= bits - 1) {
                            int b = __builtin_ctzll(bits), r = b / 8 + dr, c = b % 8 + dc;
                            if (r > 7 || c > 7) {
                                ok = false;
                                break;
                            }
                            shifted |= 1ull << (r * 8 + c);
                        }
                        if (!ok)
                            continue;
                        for (int b = 0; b < 64; b++) {
                            if ((shifted >> b) & 1u)
                                continue;
                            uint64_t t = shifted | (1ull << b);
                            if (!shape_connected(t))
                                continue;
                            next.insert(shape_canonical(shape_normalize(t), kFormsD4));
                        }
                    }
            }
            level = next;
            free_[m].assign(next.begin(), next.end());
        }
        // One-sided: each free shape plus its mirror class when distinct
        // (the reference's catalogue generator, src/enum.cpp:46-54).
        for (int m = 1; m <= 8; m++) {
            std::set<uint64_t> s(free_[m].begin(), free_[m].end());
            for (uint64_t v : free_[m]) {
                uint64_t flip = shape_canonical(v, kFormsReflections);
                s.insert(flip);
            }
            onesided[m].assign(s.begin(), s.end());
        }
    }
};

const Catalogue &catalogue() {
    static Catalogue c;
    return c;
}

}  // namespace

const std::vector<uint64_t> &catalogue_free(int m) {
    static const std::vector<uint64_t> empty;
    if (m < 1 || m > 8)
        return empty;
    return catalogue().free_[m];
}

const std::vector<uint64_t> &catalogue_onesided(int m) {
    static const std::vector<uint64_t> empty;
    if (m < 1 || m > 8)
        return empty;
    return catalogue().onesided[m];
}

std::string build_piece_lib(const uint64_t *shapes, const uint32_t *counts, uint32_t n,
                            uint32_t sym, uint32_t width, PieceLib &out) {
    if (width < 1 || width > (uint32_t)kMaxWidth)
        return "board width must be 1..8";
    if ((sym & 0xFFu) == 0)
        return "symmetry mask allows no transform";
    out = PieceLib{};
    out.sym = sym & 0xFFu;
    out.width = width;
    out.win_rows = 64 / width;
    if (n > (uint32_t)kMaxTypes)
        return "more than 40 piece types";
    uint32_t base = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (!shapes[i])
            return "empty piece shape";
        if (!shape_connected(shape_normalize(shapes[i])))
            return "piece shape is not connected";
        out.shapes.push_back(shapes[i]);
        out.counts.push_back(counts[i]);
        const uint32_t c = counts[i];
        // binary counter of bit_length(c) bits (none for an absent type)
        uint32_t bits = 0;
        while (bits < 32 && (c >> bits))
            bits++;
        if (base + bits > (uint32_t)kMaxUsedBits)
            return "more than 40 bits of piece copy counters";
        TypeField tf{};
        if (bits) {
            tf.fm = ((1ull << bits) - 1) << base;
            tf.cap = (unsigned long long)c << base;
        }
        out.fields.push_back(tf);
        out.copies += c;
        base += bits;
    }
    out.used_bits = base;

    // Distinct allowed orientations per type, in Shape::transforms() order
    // (the enabled placements of Piece::Piece, src/Piece.cpp:12-22).
    struct Orient {
        uint32_t type, t;
        int ncells, h, w, cr[64], cc[64];
    };
    std::vector<Orient> orients;
    for (uint32_t i = 0; i < n; i++) {
        if (!counts[i])
            continue;
        std::vector<uint64_t> seen;
        unsigned s = out.sym;
        for (int t = 0; t < 8; t++, s >>= 1) {
            if (!(s & 1u))
                continue;
            uint64_t v = shape_transform(shapes[i], t);
            if (std::find(seen.begin(), seen.end(), v) != seen.end())
                continue;
            seen.push_back(v);
            Orient o{};
            o.type = i;
            o.t = (uint32_t)t;
            for (uint64_t bits = v; bits; bits &= bits - 1) {
                int b = __builtin_ctzll(bits);
                o.cr[o.ncells] = b / 8;
                o.cc[o.ncells] = b % 8;
                o.h = std::max(o.h, b / 8 + 1);
                o.w = std::max(o.w, b % 8 + 1);
                o.ncells++;
            }
            out.max_piece_rows = std::max(out.max_piece_rows, (uint32_t)o.h);
            orients.push_back(o);
        }
    }
    if (out.max_piece_rows > out.win_rows)
        return "piece taller than the row window of this board width";
    out.dyn_bits = out.max_piece_rows ? width * (out.max_piece_rows - 1) : 0;

    // Placements anchored at each column: the anchor is the piece's first
    // cell in row-major order (the lowest set bit), which the row-by-row
    // search always puts on the lowest empty cell.
    for (uint32_t col = 0; col < width; col++) {
        out.col_off[col] = (uint16_t)out.plc.size();
        for (const Orient &o : orients) {
            if (!out.counts[o.type])
                continue;
            int x = (int)col - o.cc[0];
            if (x < 0 || x + o.w > (int)width)
                continue;
            uint64_t m = 0;
            for (int k = 0; k < o.ncells; k++)
                m |= 1ull << (o.cr[k] * (int)width + o.cc[k] + x);
            Plc pl{};
            pl.mask = m;
            pl.type = (uint8_t)o.type;
            const TypeField &tf = out.fields[o.type];
            pl.off = (uint8_t)__builtin_ctzll(tf.fm);
            pl.bits = (uint8_t)__builtin_popcountll(tf.fm);
            pl.count = out.counts[o.type];
            out.plc.push_back(pl);
            out.plc_type.push_back((uint16_t)o.type);
            out.plc_orient.push_back(o.t);
        }
        const size_t len = out.plc.size() - out.col_off[col];
        if (len > (size_t)kMaxPlcPerCol)
            return "more than 255 placements anchored at one column";
        out.col_len[col] = (uint16_t)len;
        // A column's placements come grouped by type: each records where its
        // type's run ends, so a type without copies left is skipped at once.
        for (size_t i = len; i-- > 0;) {
            Plc &p = out.plc[out.col_off[col] + i];
            const bool last = i + 1 == len || out.plc[out.col_off[col] + i + 1].type != p.type;
            p.next_type = last ? (uint8_t)(i + 1) : out.plc[out.col_off[col] + i + 1].next_type;
        }
    }

    // Candidate filters: for column c, bitsets over its placements of those
    // whose row-0 cells fit a row-0 pattern (indexed by the bits right of c;
    // c itself is always empty at that point), and of those whose row-1
    // (row-2) cells fit a row-1 (row-2) pattern.
    uint32_t maxlen = 1;
    for (uint32_t col = 0; col < width; col++)
        maxlen = std::max<uint32_t>(maxlen, out.col_len[col]);
    out.fwords = (maxlen + 63) / 64;
    const uint32_t FW = out.fwords;
    const uint64_t rowmask = (1ull << width) - 1ull;
    // Fixed layout, so that the kernel computes offsets instead of loading
    // them: row-0 filters of column c at (c * 2^(W-1) + p) * FW, then the
    // row-1 filters at (W * 2^(W-1) + c * 2^W + q) * FW, then the row-2
    // filters W * 2^W * FW further on.
    const size_t n0 = (size_t)1 << (width - 1), n1 = (size_t)1 << width;
    out.filters.assign((width * n0 + 2 * width * n1) * FW, 0ull);
    for (uint32_t col = 0; col < width; col++) {
        out.f0_off[col] = (uint32_t)((col * n0) * FW);
        out.f1_off[col] = (uint32_t)((width * n0 + col * n1) * FW);
        out.f2_off[col] = (uint32_t)((width * n0 + width * n1 + col * n1) * FW);
        const uint32_t np = 1u << (width - 1 - col);
        for (uint32_t p = 0; p < np; p++) {
            const uint64_t row0 = ((uint64_t)p << (col + 1)) | (1ull << col);
            for (uint32_t i = 0; i < out.col_len[col]; i++) {
                const uint64_t m0 = out.plc[out.col_off[col] + i].mask & rowmask;
                if (!(m0 & ~row0))
                    out.filters[out.f0_off[col] + (size_t)p * FW + i / 64] |= 1ull << (i % 64);
            }
        }
        // Rows 1 and 2: placements whose cells in that row fit its pattern.
        for (uint32_t r = 1; r <= 2; r++) {
            const uint32_t off = r == 1 ? out.f1_off[col] : out.f2_off[col];
            for (uint32_t q = 0; q < (1u << width); q++)
                for (uint32_t i = 0; i < out.col_len[col]; i++) {
                    const uint64_t mr =
                        (out.plc[out.col_off[col] + i].mask >> (r * width)) & rowmask;
                    if (!(mr & ~(uint64_t)q))
                        out.filters[off + (size_t)q * FW + i / 64] |= 1ull << (i % 64);
                }
        }
    }
    return {};
}

void canonical_grid(uint32_t width, uint32_t height, const uint8_t *rows,
                    const int8_t *grid, int8_t *out) {
    const int W = (int)width, H = (int)height, cells = W * H;
    std::vector<int8_t> tmp((size_t)cells);
    bool have = false;
    for (int t = 0; t < 8; t++) {
        const bool sw = (t >> 2) & 1, fx = t & 1, fy = (t >> 1) & 1;
        if (sw && W != H)
            continue;
        bool ok = true;
        for (int r = 0; r < H && ok; r++)
            for (int c = 0; c < W; c++) {
                int ir = sw ? c : r, ic = sw ? r : c;
                if (fx)
                    ic = W - 1 - ic;
                if (fy)
                    ir = H - 1 - ir;
                if (((rows[r] >> c) & 1u) != ((rows[ir] >> ic) & 1u)) {
                    ok = false;
                    break;
                }
                tmp[(size_t)(r * W + c)] = grid[ir * W + ic];
            }
        if (!ok)
            continue;
        bool less = !have;
        for (int i = 0; have && i < cells; i++)
            if (tmp[(size_t)i] != out[i]) {
                less = tmp[(size_t)i] < out[i];
                break;
            }
        if (less)
            std::memcpy(out, tmp.data(), (size_t)cells);
        have = true;
    }
}

}  // namespace d4e
