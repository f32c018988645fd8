// board_family.h -- C++ facade of the reference's board-family search over
// the C ABI in include/d4e.h:
//  * Board<L>       -- src/board.hpp:9-57 (text rules of Shape<L>,
//                      src/Shape.hpp:49-77);
//  * Naming         -- src/naming.hpp:15-71, src/naming.cpp:34-90,
//                      src/naming.inl:6-72 (ranks of piece combinations);
//  * family_ledger  -- the AtomicCount searcher's ledger (src/search.cpp:36-53):
//                      for every combination rank, the number of
//                      configurations it tiles; all configurations run as one
//                      d4e_batch_sets batch.
//
// Differences a caller of the reference sees:
//  * regions are numbered in order of first appearance in the text (the
//    reference iterates an unordered_map, whose order is unspecified), so
//    configuration indices may differ; the configurations are the same;
//  * the piece library is explicit (min_m..max_m, one-sided or free) instead
//    of the g_nme / g_sym globals;
//  * configurations that no combination tiles are returned (the reference
//    prints them as ZERO-count boards, src/searcher.cpp:110-115).
#pragma once

#include <algorithm>
#include <cstdint>
#include <fstream>
#include <map>
#include <optional>
#include <sstream>
#include <string>
#include <string_view>
#include <vector>

#include "searcher_cuda.h"

namespace d4e_host {

// Shape<L>(std::string_view): bit L * row + column; a leading newline is
// skipped; '*', '1', '@', '#', 'X', '%' are cells, ' ', '0', '.', '-', '_'
// positions outside the shape, '\n' starts the next row, anything else is
// ignored.  A row longer than L runs on into the next row's bits; bits past
// 63 are dropped.
template <size_t L>
inline uint64_t shape_from_text(std::string_view sv) {
    if (!sv.empty() && sv.front() == '\n')
        sv.remove_prefix(1);
    uint64_t value = 0;
    unsigned row_start = 0, pos = 0;
    for (char ch : sv) {
        switch (ch) {
        case ' ': case '0': case '.': case '-': case '_':
            pos++;
            break;
        case '*': case '1': case '@': case '#': case 'X': case '%':
            if (row_start + pos < 64)
                value |= 1ull << (row_start + pos);
            pos++;
            break;
        case '\n':
            row_start += (unsigned)L;
            pos = 0;
            break;
        default:
            break;
        }
    }
    return value;
}

// Board<L>: letters and digits name regions (each also a base cell); the
// other cell marks belong to the base and, as in the reference, to every
// region.  A configuration clears one cell of every region.
template <size_t L>
struct Board {
    uint64_t base = 0;
    std::vector<uint64_t> regions;
    std::vector<char> names;
    size_t count = 1;

    explicit Board(std::string_view sv) {
        auto valid = [](char ch) {
            return (ch >= '0' && ch <= '9') || (ch >= 'A' && ch <= 'Z') || (ch >= 'a' && ch <= 'z');
        };
        for (char ch : sv)
            if (valid(ch) && std::find(names.begin(), names.end(), ch) == names.end())
                names.push_back(ch);
        std::string the_base;
        std::vector<std::string> texts(names.size());
        for (char ch : sv) {
            the_base.push_back(valid(ch) ? '#' : ch);
            for (size_t k = 0; k < names.size(); k++)
                texts[k].push_back(valid(ch) ? (ch == names[k] ? '#' : '.') : ch);
        }
        base = shape_from_text<L>(the_base);
        for (const auto &t : texts)
            regions.push_back(shape_from_text<L>(t));
        for (uint64_t r : regions)
            count *= (size_t)__builtin_popcountll(r);
    }

    static Board from_file(const std::string &path) {
        std::ifstream fin(path);
        if (!fin)
            throw std::runtime_error("d4e: cannot read " + path);
        std::stringstream buf;
        buf << fin.rdbuf();
        return Board(buf.str());
    }

    // Cells of every configuration.
    size_t left() const { return (size_t)__builtin_popcountll(base) - regions.size(); }

    // func(uint64_t board) for every configuration: the first region's cell
    // varies slowest, cells in increasing bit order.
    template <class F>
    void foreach(F &&func) const {
        std::vector<size_t> at(regions.size(), 0);
        std::vector<std::vector<unsigned>> cells(regions.size());
        for (size_t k = 0; k < regions.size(); k++)
            for (unsigned b = 0; b < 64; b++)
                if ((regions[k] >> b) & 1u)
                    cells[k].push_back(b);
        for (const auto &c : cells)
            if (c.empty())
                return;
        for (;;) {
            uint64_t m = base;
            for (size_t k = 0; k < regions.size(); k++)
                m &= ~(1ull << cells[k][at[k]]);
            func(m);
            size_t k = regions.size();
            while (k > 0 && ++at[k - 1] == cells[k - 1].size())
                at[--k] = 0;
            if (k == 0)
                return;
        }
    }
};

// Ranks of piece combinations: k_m distinct pieces of each size m in
// min_m..max_m (sizes[m] pieces of size m), min_n <= sum k_m <= max_n,
// sum m * k_m == tgt.  Ranks run over the size profiles (k_min_m, ...,
// k_max_m) in lexicographic order; within a profile the rank is mixed radix
// over the sizes, the smallest size the most significant digit, each digit
// the lexicographic rank of the chosen subset among C(sizes[m], k_m).  The
// ranks index the reference's ledgers, so this order is the reference's.
class Naming {
public:
    Naming(uint64_t min_m, uint64_t max_m, uint64_t min_n, uint64_t max_n, uint64_t tgt,
           std::vector<uint64_t> sizes)
        : min_m_(min_m), max_m_(max_m), min_n_(min_n), max_n_(max_n), sizes_(std::move(sizes)) {
        sizes_.resize(std::max<size_t>(sizes_.size(), max_m + 1), 0);
        std::vector<uint64_t> cur;
        walk(cur, tgt, 0);
        uint64_t total = 0;
        for (const auto &pr : profiles_) {
            std::vector<uint64_t> radix;
            uint64_t prod = 1;
            for (size_t d = 0; d < pr.size(); d++) {
                radix.push_back(binomial(sizes_[min_m + d], pr[d]));
                prod *= radix.back();
            }
            radix_.push_back(std::move(radix));
            starts_.push_back(total);
            total += prod;
        }
        size_ = total;
    }

    uint64_t size() const { return size_; }
    uint64_t size_pieces() const {
        uint64_t n = 0;
        for (uint64_t m = min_m_; m <= max_m_; m++)
            n += sizes_[m];
        return n;
    }
    // Piece (m, i) as one index over all sizes.
    uint64_t name_piece(uint64_t m, uint64_t i) const {
        uint64_t n = 0;
        for (uint64_t k = min_m_; k < m; k++)
            n += sizes_[k];
        return n + i;
    }

    // chosen(m, i): whether the i-th piece of size m is in the combination.
    template <class F>
    std::optional<uint64_t> name(F &&chosen) const {
        std::vector<uint64_t> profile;
        for (uint64_t m = min_m_; m <= max_m_; m++) {
            uint64_t k = 0;
            for (uint64_t i = 0; i < sizes_[m]; i++)
                k += chosen(m, i) ? 1u : 0u;
            profile.push_back(k);
        }
        auto it = std::lower_bound(profiles_.begin(), profiles_.end(), profile);
        if (it == profiles_.end() || *it != profile)
            return std::nullopt;
        const size_t p = (size_t)(it - profiles_.begin());
        uint64_t nm = 0;
        for (uint64_t m = min_m_; m <= max_m_; m++) {
            const size_t d = (size_t)(m - min_m_);
            uint64_t k = profile[d], r = 0, n = sizes_[m];
            for (uint64_t i = 0; k; i++, n--) {
                if (chosen(m, i))
                    k--;
                else
                    r += binomial(n - 1, k - 1);
            }
            nm = nm * radix_[p][d] + r;
        }
        return starts_[p] + nm;
    }

    // func(m, i) for every piece of the combination ranked nm; false when nm
    // is out of range.
    template <class F>
    bool resolve(uint64_t nm, F &&func) const {
        if (nm >= size_)
            return false;
        const size_t p =
            (size_t)(std::upper_bound(starts_.begin(), starts_.end(), nm) - starts_.begin()) - 1;
        nm -= starts_[p];
        std::vector<uint64_t> digit(radix_[p].size());
        for (size_t d = digit.size(); d-- > 0;) {
            digit[d] = nm % radix_[p][d];
            nm /= radix_[p][d];
        }
        for (size_t d = 0; d < digit.size(); d++) {
            const uint64_t m = min_m_ + d;
            uint64_t k = profiles_[p][d], x = digit[d], n = sizes_[m];
            for (uint64_t i = 0; k; i++, n--) {
                const uint64_t below = binomial(n - 1, k - 1);
                if (x < below) {
                    func(m, i);
                    k--;
                } else {
                    x -= below;
                }
            }
        }
        return true;
    }

    uint64_t min_m() const { return min_m_; }
    uint64_t max_m() const { return max_m_; }
    uint64_t min_n() const { return min_n_; }
    uint64_t max_n() const { return max_n_; }
    uint64_t pieces(uint64_t m) const { return m < sizes_.size() ? sizes_[m] : 0; }

    static uint64_t binomial(uint64_t n, uint64_t k) {
        if (k > n)
            return 0;
        k = std::min(k, n - k);
        unsigned __int128 r = 1;
        for (uint64_t j = 1; j <= k; j++)
            r = r * (n - k + j) / j;   // exact: C(n-k+j, j) * j = C(n-k+j-1, j-1) * (n-k+j)
        return (uint64_t)r;
    }

private:
    void walk(std::vector<uint64_t> &cur, uint64_t left, uint64_t n) {
        const uint64_t m = min_m_ + cur.size();
        if (left == 0) {
            if (n >= min_n_) {
                std::vector<uint64_t> pr = cur;
                pr.resize(max_m_ - min_m_ + 1, 0);
                profiles_.push_back(std::move(pr));
            }
            return;
        }
        if (m > max_m_)
            return;
        for (uint64_t k = 0; k * m <= left && n + k <= max_n_ && k <= sizes_[m]; k++) {
            cur.push_back(k);
            walk(cur, left - k * m, n + k);
            cur.pop_back();
        }
    }

    uint64_t min_m_, max_m_, min_n_, max_n_;
    std::vector<uint64_t> sizes_;
    std::vector<std::vector<uint64_t>> profiles_;
    std::vector<std::vector<uint64_t>> radix_;
    std::vector<uint64_t> starts_;
    uint64_t size_ = 0;
};

// The catalogue's pieces of min_m..max_m cells, free or one-sided, in the
// reference's known_shapes / known_C_shapes order.
inline std::vector<uint64_t> pieces_by_size(unsigned min_m, unsigned max_m, bool one_sided,
                                            std::vector<uint64_t> *sizes = nullptr) {
    std::vector<uint64_t> out;
    if (sizes)
        sizes->assign(max_m + 1, 0);
    for (unsigned m = min_m; m <= max_m; m++) {
        uint32_t n = 0;
        check(d4e_catalogue(m, one_sided ? 1 : 0, nullptr, 0, &n));
        std::vector<uint64_t> v(n);
        check(d4e_catalogue(m, one_sided ? 1 : 0, v.data(), n, &n));
        out.insert(out.end(), v.begin(), v.end());
        if (sizes)
            (*sizes)[m] = n;
    }
    return out;
}

struct FamilyLedger {
    std::vector<uint64_t> ledger;     // [Naming rank] -> configurations it tiles
    std::vector<uint64_t> unsolved;   // configurations no ranked combination tiles
    uint64_t configs = 0;             // configurations visited (Board::count)
    uint64_t boards = 0;              // distinct boards solved
    uint64_t sets = 0;                // (distinct board, ranked combination) pairs
    uint64_t tilings = 0;             // tilings of those pairs
};

// The AtomicCount run over a whole family: every distinct configuration is
// one instance of a d4e_batch_sets batch over the pieces of min_m..max_m
// cells (each at most once); a set is ranked when it has min_n..max_n
// pieces covering the configuration's `left` cells.
inline FamilyLedger family_ledger(const Board<8> &board, const Naming &naming,
                                  const std::vector<uint64_t> &pieces, bool one_sided,
                                  int device = 0, uint64_t max_states = 0) {
    FamilyLedger out;
    std::map<uint64_t, uint64_t> mult;   // distinct board -> configurations
    std::vector<uint64_t> order;
    board.foreach([&](uint64_t m) {
        out.configs++;
        if (mult[m]++ == 0)
            order.push_back(m);
    });
    std::vector<uint64_t> uniq(order);
    std::sort(uniq.begin(), uniq.end());
    out.boards = uniq.size();

    const std::vector<uint32_t> counts(pieces.size(), 1u);
    std::vector<std::vector<uint8_t>> rows(uniq.size());
    std::vector<d4e_instance> insts(uniq.size());
    for (size_t k = 0; k < uniq.size(); k++) {
        for (unsigned r = 0; r < 8; r++)
            rows[k].push_back((uint8_t)(uniq[k] >> (8 * r)));
        while (rows[k].size() > 1 && rows[k].back() == 0)
            rows[k].pop_back();
        insts[k] = d4e_instance{8u, (uint32_t)rows[k].size(), rows[k].data(),
                                (uint32_t)pieces.size(), pieces.data(), counts.data(),
                                one_sided ? 0b01101001u : 0xFFu};
    }
    d4e_batch_opts o{};
    o.mode = D4E_MODE_SETS;
    o.device = device;
    o.max_states = max_states;
    std::vector<d4e_result> res(uniq.size());
    std::vector<uint64_t> offs(uniq.size() + 1);
    uint64_t max_sets = 1u << 16;
    std::vector<uint8_t> copies;
    std::vector<uint64_t> til;
    for (;;) {
        copies.resize(max_sets * D4E_SET_PIECES);
        til.resize(max_sets);
        const int rc = d4e_batch_sets(insts.data(), (uint32_t)insts.size(), &o, res.data(),
                                      offs.data(), copies.data(), til.data(), max_sets, nullptr);
        if (rc == D4E_ERR_INVALID && offs.back() > max_sets) {
            max_sets = offs.back();
            continue;
        }
        check(rc);
        break;
    }
    for (size_t k = 0; k < uniq.size(); k++)
        if (res[k].status != D4E_OK)
            throw std::runtime_error("d4e: configuration failed with status " +
                                     std::to_string(res[k].status));

    // piece index -> (size, index within the size)
    std::vector<std::pair<uint64_t, uint64_t>> who;
    for (uint64_t m = naming.min_m(); m <= naming.max_m(); m++)
        for (uint64_t i = 0; i < naming.pieces(m); i++)
            who.emplace_back(m, i);
    if (who.size() != pieces.size())
        throw std::runtime_error("d4e: the piece list does not match the Naming sizes");
    std::vector<std::vector<uint8_t>> chosen(naming.max_m() + 1);
    for (uint64_t m = naming.min_m(); m <= naming.max_m(); m++)
        chosen[m].assign(naming.pieces(m), 0);

    out.ledger.assign(naming.size(), 0);
    const uint64_t left = board.left();
    std::map<uint64_t, bool> solved;
    for (size_t k = 0; k < uniq.size(); k++) {
        bool any = false;
        for (uint64_t s = offs[k]; s < offs[k + 1]; s++) {
            const uint8_t *c = copies.data() + s * D4E_SET_PIECES;
            uint64_t n = 0, area = 0;
            for (size_t p = 0; p < pieces.size(); p++) {
                n += c[p];
                area += c[p] * (uint64_t)__builtin_popcountll(pieces[p]);
                chosen[who[p].first][who[p].second] = c[p];
            }
            if (n < naming.min_n() || n > naming.max_n() || area != left)
                continue;
            const auto rank = naming.name([&](uint64_t m, uint64_t i) { return chosen[m][i] != 0; });
            if (!rank)
                throw std::runtime_error("d4e: a tiling combination has no Naming rank");
            out.ledger[*rank] += mult[uniq[k]];
            out.sets++;
            out.tilings += til[s];
            any = true;
        }
        solved[uniq[k]] = any;
    }
    board.foreach([&](uint64_t m) {
        if (!solved[m])
            out.unsolved.push_back(m);
    });
    return out;
}

}  // namespace d4e_host
