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
//  * LedgerFile / family_ledger_file -- the FileBit / FileByte searchers'
//                      mmap'ed ledger with resume (src/search.cpp:56-226), same
//                      file layout.
//
// Differences a caller of the reference sees:
//  * the piece library is explicit (min_m..max_m, one-sided or free) instead
//    of the g_nme / g_sym globals;
//  * configurations that no combination tiles are returned (the reference
//    prints them as ZERO-count boards, src/searcher.cpp:110-115).
#pragma once

#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <optional>
#include <sstream>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

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
// region.  A configuration clears one cell of every region.  Regions are
// kept in the iteration order of a std::unordered_map<char, std::string>
// filled in text order, as the reference keeps them: configuration i is the
// same board here and there (with the same C++ standard library), which the
// ledger files index by.
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
        std::unordered_map<char, std::string> texts;
        for (char ch : sv)
            if (valid(ch))
                texts.emplace(ch, "");
        std::string the_base;
        for (char ch : sv) {
            the_base.push_back(valid(ch) ? '#' : ch);
            for (auto &[k, t] : texts)
                t.push_back(valid(ch) ? (ch == k ? '#' : '.') : ch);
        }
        base = shape_from_text<L>(the_base);
        for (const auto &[k, t] : texts) {
            names.push_back(k);
            regions.push_back(shape_from_text<L>(t));
        }
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

// Ranked combinations of each board: one d4e_batch_sets batch over the
// pieces (each at most once); a tiling piece set is ranked when it has
// naming.min_n()..max_n() pieces covering `left` cells.
struct BoardRanks {
    std::vector<std::vector<uint64_t>> ranks;   // per board, in the sets' order
    std::vector<uint64_t> tilings;              // per board: tilings of its ranked sets
    std::vector<uint64_t> sets;                 // per board: ranked sets
    std::vector<double> ms;                     // per board: batch start to its completion
};

inline BoardRanks rank_boards(const std::vector<uint64_t> &boards, uint64_t left,
                              const Naming &naming, const std::vector<uint64_t> &pieces,
                              bool one_sided, int device = 0, uint64_t max_states = 0) {
    BoardRanks out;
    const size_t nb = boards.size();
    out.ranks.resize(nb);
    out.tilings.assign(nb, 0);
    out.sets.assign(nb, 0);
    out.ms.assign(nb, 0.0);
    if (!nb)
        return out;
    const std::vector<uint32_t> counts(pieces.size(), 1u);
    std::vector<std::vector<uint8_t>> rows(nb);
    std::vector<d4e_instance> insts(nb);
    for (size_t k = 0; k < nb; k++) {
        for (unsigned r = 0; r < 8; r++)
            rows[k].push_back((uint8_t)(boards[k] >> (8 * r)));
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
    std::vector<d4e_result> res(nb);
    std::vector<uint64_t> offs(nb + 1);
    uint64_t max_sets = 1u << 16;
    std::vector<uint8_t> copies;
    std::vector<uint64_t> til;
    for (;;) {
        copies.resize(max_sets * D4E_SET_PIECES);
        til.resize(max_sets);
        const int rc = d4e_batch_sets(insts.data(), (uint32_t)nb, &o, res.data(), offs.data(),
                                      copies.data(), til.data(), max_sets, nullptr);
        if (rc == D4E_ERR_INVALID && offs.back() > max_sets) {
            max_sets = offs.back();
            continue;
        }
        check(rc);
        break;
    }
    for (size_t k = 0; k < nb; k++)
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

    for (size_t k = 0; k < nb; k++) {
        out.ms[k] = res[k].latency_ms;
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
            out.ranks[k].push_back(*rank);
            out.sets[k]++;
            out.tilings[k] += til[s];
        }
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
// one instance of one d4e_batch_sets batch.
inline FamilyLedger family_ledger(const Board<8> &board, const Naming &naming,
                                  const std::vector<uint64_t> &pieces, bool one_sided,
                                  int device = 0, uint64_t max_states = 0) {
    FamilyLedger out;
    std::map<uint64_t, uint64_t> mult;   // distinct board -> configurations
    board.foreach([&](uint64_t m) {
        out.configs++;
        mult[m]++;
    });
    std::vector<uint64_t> uniq;
    for (const auto &e : mult)
        uniq.push_back(e.first);
    out.boards = uniq.size();
    const BoardRanks br = rank_boards(uniq, board.left(), naming, pieces, one_sided, device,
                                      max_states);
    out.ledger.assign(naming.size(), 0);
    std::map<uint64_t, bool> solved;
    for (size_t k = 0; k < uniq.size(); k++) {
        for (uint64_t r : br.ranks[k])
            out.ledger[r] += mult[uniq[k]];
        out.sets += br.sets[k];
        out.tilings += br.tilings[k];
        solved[uniq[k]] = !br.ranks[k].empty();
    }
    board.foreach([&](uint64_t m) {
        if (!solved[m])
            out.unsolved.push_back(m);
    });
    return out;
}

// The FileBit / FileByte ledger file (src/search.cpp:56-226), mapped shared:
//   configs x {shape, count, solved, padding}   (u64 each; solved = ms, 0 = not yet)
//   names   x u64                               (configurations each rank tiles)
//   names   x w bytes                           (Byte: w = configs, one 0xff byte per
//                                                (rank, configuration) tiled;
//                                                Bit: w = ceil(configs / 8), bit i % 8 of
//                                                byte i / 8 for configuration i)
// A new (empty) file is sized to fit; an existing one must have exactly
// that size, and its solved configurations are skipped (resume).
enum class LedgerKind { Bit, Byte };

struct ConfigDescriptor {
    uint64_t shape;
    uint64_t count;     // ranked combinations that tile the configuration
    uint64_t solved;    // 0: not yet; else milliseconds spent on it (at least 1)
    uint64_t padding;
};
static_assert(sizeof(ConfigDescriptor) == 32, "the reference's config_descriptor is 32 B");

class LedgerFile {
public:
    LedgerFile(const std::string &path, uint64_t configs, uint64_t names, LedgerKind kind)
        : configs_(configs), names_(names), kind_(kind),
          width_(kind == LedgerKind::Byte ? configs : (configs + 7) / 8) {
        size_ = configs_ * sizeof(ConfigDescriptor) + names_ * sizeof(uint64_t) + names_ * width_;
        fd_ = ::open(path.c_str(), O_RDWR | O_CREAT, 0666);
        if (fd_ < 0)
            throw std::runtime_error("d4e: open " + path + ": " + std::strerror(errno));
        struct stat st {};
        if (::fstat(fd_, &st) != 0)
            fail("fstat");
        if (st.st_size == 0) {
            if (::ftruncate(fd_, (off_t)size_) != 0)
                fail("ftruncate");
        } else if ((uint64_t)st.st_size > size_) {
            fail("file too long for this board family and Naming", false);
        } else if ((uint64_t)st.st_size < size_) {
            fail("file too short for this board family and Naming", false);
        }
        void *m = size_ ? ::mmap(nullptr, size_, PROT_READ | PROT_WRITE, MAP_SHARED, fd_, 0)
                        : nullptr;
        if (size_ && m == MAP_FAILED)
            fail("mmap");
        base_ = static_cast<uint8_t *>(m);
    }
    LedgerFile(const LedgerFile &) = delete;
    LedgerFile &operator=(const LedgerFile &) = delete;
    ~LedgerFile() {
        if (base_)
            ::munmap(base_, size_);
        if (fd_ >= 0)
            ::close(fd_);
    }

    uint64_t configs() const { return configs_; }
    uint64_t names() const { return names_; }
    LedgerKind kind() const { return kind_; }
    uint64_t bytes() const { return size_; }

    ConfigDescriptor &config(uint64_t i) {
        return reinterpret_cast<ConfigDescriptor *>(base_)[i];
    }
    uint64_t &tiled(uint64_t v) {
        return reinterpret_cast<uint64_t *>(base_ + configs_ * sizeof(ConfigDescriptor))[v];
    }
    bool logged(uint64_t v, uint64_t i) const {
        const uint8_t *l = ledger() + v * width_;
        return kind_ == LedgerKind::Byte ? l[i] != 0 : ((l[i / 8] >> (i % 8)) & 1u) != 0;
    }
    // Marks rank v as tiling configuration i; true (and the rank's count
    // raised) the first time.
    bool log(uint64_t v, uint64_t i) {
        if (v >= names_ || i >= configs_)
            throw std::runtime_error("d4e: ledger index out of range");
        if (logged(v, i))
            return false;
        uint8_t *l = const_cast<uint8_t *>(ledger()) + v * width_;
        if (kind_ == LedgerKind::Byte)
            l[i] = 0xFF;
        else
            l[i / 8] |= (uint8_t)(1u << (i % 8));
        tiled(v)++;
        return true;
    }
    void sync() {
        if (base_ && ::msync(base_, size_, MS_SYNC) != 0)
            fail("msync");
    }

private:
    const uint8_t *ledger() const {
        return base_ + configs_ * sizeof(ConfigDescriptor) + names_ * sizeof(uint64_t);
    }
    [[noreturn]] void fail(const char *what, bool with_errno = true) {
        const std::string msg = std::string("d4e: ledger file: ") + what +
                                (with_errno ? std::string(": ") + std::strerror(errno) : "");
        if (base_)
            ::munmap(base_, size_);
        base_ = nullptr;
        if (fd_ >= 0)
            ::close(fd_);
        fd_ = -1;
        throw std::runtime_error(msg);
    }

    uint64_t configs_, names_;
    LedgerKind kind_;
    uint64_t width_, size_ = 0;
    int fd_ = -1;
    uint8_t *base_ = nullptr;
};

struct FileRun {
    uint64_t configs = 0;            // configurations of the family
    uint64_t previously_solved = 0;  // skipped: solved in an earlier run
    uint64_t solved_now = 0;
    uint64_t batches = 0;
    std::vector<uint64_t> unsolved;  // configurations (indices) no ranked combination tiles
};

// Fills a ledger file like the reference's FileBit / FileByte run: every
// configuration not yet solved in the file, `per_batch` configurations per
// d4e_batch_sets batch; each batch's results are written and synced before
// the next starts, so an interrupted run resumes after its last batch.
// max_batches > 0 stops after that many batches (a time-sliced run).
inline FileRun family_ledger_file(const Board<8> &board, const Naming &naming,
                                  const std::vector<uint64_t> &pieces, bool one_sided,
                                  LedgerFile &file, uint64_t per_batch = 1024, int device = 0,
                                  uint64_t max_states = 0, uint64_t max_batches = 0) {
    if (file.configs() != board.count || file.names() != naming.size())
        throw std::runtime_error("d4e: the ledger file does not match the family and Naming");
    FileRun out;
    std::vector<std::pair<uint64_t, uint64_t>> todo;   // (configuration index, board)
    uint64_t i = 0;
    board.foreach([&](uint64_t m) {
        ConfigDescriptor &c = file.config(i);
        c.shape = m;
        if (c.solved)
            out.previously_solved++;
        else
            todo.emplace_back(i, m);
        i++;
    });
    out.configs = i;
    per_batch = std::max<uint64_t>(per_batch, 1);
    for (size_t at = 0; at < todo.size() && (!max_batches || out.batches < max_batches);
         at += per_batch) {
        const size_t end = std::min<size_t>(todo.size(), at + per_batch);
        std::vector<uint64_t> uniq;
        for (size_t k = at; k < end; k++)
            uniq.push_back(todo[k].second);
        std::sort(uniq.begin(), uniq.end());
        uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
        const BoardRanks br = rank_boards(uniq, board.left(), naming, pieces, one_sided, device,
                                          max_states);
        for (size_t k = at; k < end; k++) {
            const size_t b = (size_t)(std::lower_bound(uniq.begin(), uniq.end(), todo[k].second) -
                                      uniq.begin());
            ConfigDescriptor &c = file.config(todo[k].first);
            uint64_t n = 0;
            for (uint64_t r : br.ranks[b])
                n += file.log(r, todo[k].first) ? 1u : 0u;
            c.count = n;
            c.solved = std::max<uint64_t>(1, (uint64_t)(br.ms[b] + 0.5));
            if (!n)
                out.unsolved.push_back(todo[k].first);
            out.solved_now++;
        }
        file.sync();
        out.batches++;
    }
    return out;
}

}  // namespace d4e_host
