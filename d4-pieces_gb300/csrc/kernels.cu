// kernels.cu -- sm_103a kernels of the row-by-row polyomino tiling engine.
//
// Hot path (one launch pair per board row):
//   k_expand  : replaces the reference's tiled_row_search / linear_row_search
//               + impl<H> (src/kernel.cuh:12-227).  Each state is expanded by
//               every whole-row fill -- a depth-first walk over placements
//               anchored at the lowest empty cell of the current row.  A
//               single-instance launch first stages the instance's placement
//               table and descriptor in shared memory; the candidate filters
//               (and, in batches, every table) are read through L1.  Each
//               child is inserted straight into an HBM-resident
//               open-addressing table (key CAS + 64-bit count add), which
//               replaces the reference's ring buffer + host hash-set Sorter
//               (src/device.cu:14-309, src/sorter.cpp:72-214).
//   k_compact : streams the table through shared memory (1-D bulk copies)
//               into the next frontier, instance by instance, clearing it
//               for the next row.
// Both are templated on the key encoding (K64 packed / K128 general, see
// d4e_types.h).
#include "kernels.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <cstdlib>
#include <cstring>

#include "state_hash.cuh"

namespace d4e {

namespace {

constexpr int kExpandBlock = kExpandWarps * 32;
constexpr int kCompactBlock = 256;


// Home slot in a table of `cap` slots (any capacity): the high half of
// hash * cap maps the 64-bit hash uniformly onto [0, cap).
__device__ __forceinline__ unsigned long long home64(unsigned long long key, unsigned long long cap) {
    return __umul64hi(mix64(key), cap);
}
__device__ __forceinline__ unsigned long long home128(unsigned long long k0, unsigned long long k1,
                                                      unsigned long long cap) {
    return __umul64hi(mix64(k0 ^ mix64(k1 ^ 0x9e3779b97f4a7c15ull)), cap);
}

__device__ __forceinline__ unsigned long long next_slot(unsigned long long h, unsigned long long cap) {
    return h + 1 == cap ? 0ull : h + 1;
}

// 128-bit compare-and-swap on a 16-byte aligned global address (sm_90+).
__device__ __forceinline__ void cas128(unsigned long long *addr,
                                       unsigned long long cmp0, unsigned long long cmp1,
                                       unsigned long long new0, unsigned long long new1,
                                       unsigned long long &old0, unsigned long long &old1) {
    asm volatile(
        "{\n\t.reg .b128 c, n, d;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 n, {%4, %5};\n\t"
        "atom.relaxed.gpu.global.cas.b128 d, [%6], c, n;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(old0), "=l"(old1)
        : "l"(cmp0), "l"(cmp1), "l"(new0), "l"(new1), "l"(addr)
        : "memory");
}

// Insert with multiplicity cnt (linear probing).  Returns 1 for a newly
// claimed key, 0 for an existing one, -1 when the probe limit was reached.
// The value field of a slot: counts are summed; witnesses (solve-one
// instances) keep the largest.
__device__ __forceinline__ void merge_value(unsigned long long *v, unsigned long long x, bool wmax) {
    if (wmax)
        atomicMax(v, x);
    else
        atomicAdd(v, x);
}

// Insert with multiplicity cnt (linear probing from slot h).  Returns 1
// for a newly claimed key, 0 for an existing one, -1 when the probe limit
// was reached.
__device__ __forceinline__ int insert64_at(Slot16 *__restrict__ T, unsigned long long cap,
                                           unsigned long long h, unsigned long long key,
                                           unsigned long long cnt, unsigned int max_probe,
                                           bool wmax) {
    for (unsigned int p = 0; p < max_probe; ++p) {
        // A naturally aligned 8-byte load is single-copy atomic: a key seen
        // here is final.  Only an empty slot needs the CAS.
        unsigned long long k = __ldcg(&T[h].key);
        if (k == 0ull) {
            k = atomicCAS(&T[h].key, 0ull, key);
            if (k == 0ull) {
                merge_value(&T[h].cnt, cnt, wmax);
                return 1;
            }
        }
        if (k == key) {
            merge_value(&T[h].cnt, cnt, wmax);
            return 0;
        }
        h = next_slot(h, cap);
    }
    return -1;
}

__device__ __forceinline__ int insert64(Slot16 *__restrict__ T, unsigned long long cap,
                                        unsigned long long key, unsigned long long cnt,
                                        unsigned int max_probe, bool wmax = false) {
    return insert64_at(T, cap, home64(key, cap), key, cnt, max_probe, wmax);
}

__device__ __forceinline__ int insert128_at(Slot32 *__restrict__ T, unsigned long long cap,
                                            unsigned long long h, unsigned long long k0,
                                            unsigned long long k1, unsigned long long cnt,
                                            unsigned int max_probe, bool wmax) {
    for (unsigned int p = 0; p < max_probe; ++p) {
        unsigned long long o0, o1;
        cas128(&T[h].k0, 0ull, 0ull, k0, k1, o0, o1);
        const bool claimed = (o0 | o1) == 0ull;
        if (claimed || (o0 == k0 && o1 == k1)) {
            merge_value(&T[h].cnt, cnt, wmax);
            return claimed ? 1 : 0;
        }
        h = next_slot(h, cap);
    }
    return -1;
}

__device__ __forceinline__ int insert128(Slot32 *__restrict__ T, unsigned long long cap,
                                         unsigned long long k0, unsigned long long k1,
                                         unsigned long long cnt, unsigned int max_probe,
                                         bool wmax = false) {
    return insert128_at(T, cap, home128(k0, k1, cap), k0, k1, cnt, max_probe, wmax);
}



// Membership lookups (the table is read-only while they run).
__device__ __forceinline__ bool find64(const Slot16 *__restrict__ T, unsigned long long cap,
                                       unsigned long long key, unsigned int max_probe) {
    unsigned long long h = home64(key, cap);
    for (unsigned int p = 0; p < max_probe; ++p) {
        const unsigned long long k = T[h].key;
        if (k == key)
            return true;
        if (k == 0ull)
            return false;
        h = next_slot(h, cap);
    }
    return false;
}

__device__ __forceinline__ bool find128(const Slot32 *__restrict__ T, unsigned long long cap,
                                        unsigned long long k0, unsigned long long k1,
                                        unsigned int max_probe) {
    unsigned long long h = home128(k0, k1, cap);
    for (unsigned int p = 0; p < max_probe; ++p) {
        const ulonglong2 k = *reinterpret_cast<const ulonglong2 *>(&T[h].k0);
        if (k.x == k0 && k.y == k1)
            return true;
        if ((k.x | k.y) == 0ull)
            return false;
        h = next_slot(h, cap);
    }
    return false;
}

// Shared-memory copy of one instance's placement table.
struct SmemTable {
    unsigned long long mask[kMaxPlc];
    uint8_t type[kMaxPlc];
    TypeField field[kMaxTypes];
    uint16_t off[kMaxWidth];
    uint16_t len[kMaxWidth];
    uint32_t width;
    uint32_t dyn_bits;
    uint32_t used_bits;
};

__device__ __forceinline__ void load_table(SmemTable &st, const InstDesc *__restrict__ d,
                                           const Plc *__restrict__ plc_all) {
    const uint32_t np = d->n_plc;
    const Plc *src = plc_all + d->plc_off;
    for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) {
        const Plc p = src[i];
        st.mask[i] = p.mask;
        st.type[i] = (uint8_t)p.type;
    }
    for (uint32_t i = threadIdx.x; i < d->n_types; i += blockDim.x)
        st.field[i] = d->types[i];
    if (threadIdx.x < kMaxWidth) {
        st.off[threadIdx.x] = d->col_off[threadIdx.x];
        st.len[threadIdx.x] = d->col_len[threadIdx.x];
    }
    if (threadIdx.x == 0) {
        st.width = d->width;
        st.dyn_bits = d->dyn_bits;
        st.used_bits = d->used_bits;
    }
}

// Copy counter tests straight from a placement record, on the counters in
// 64-bit words or, when every counter of the launch fits 32 bits, in 32-bit
// words (fewer instructions per walk step).
template <class UT>
__device__ __forceinline__ bool plc_free(const Plc &p, UT u) {
    const UT fmask = ~(UT)0 >> (8u * sizeof(UT) - p.bits);
    return ((u >> p.off) & fmask) < (UT)p.count;
}
template <class UT>
__device__ __forceinline__ UT plc_inc(const Plc &p) { return (UT)1 << p.off; }

// Depth-first enumeration of the whole-row fills of one state (window w,
// copy counters u).  The fill stack lives in two registers: 8-bit placement
// index and 4-bit anchor column per depth (a row of <= 8 cells takes <= 8
// placements).  A placement is undone by restoring its cells and decrementing
// its type's counter.  `emit(window, used, sidx, scol, depth)` is called at
// every completed row with the window before the shift; returning true stops
// the walk.
template <class Emit>
__device__ __forceinline__ void row_fills(const SmemTable &st, unsigned long long w,
                                          unsigned long long u, Emit &&emit) {
    const uint32_t W = st.width;
    const uint32_t rowmask = (1u << W) - 1u;
    unsigned long long sidx = 0;
    uint32_t scol = 0, depth = 0, idx = 0;
    for (;;) {
        const uint32_t row = (uint32_t)w & rowmask;
        bool down = false;
        if (row == 0) {
            if (emit(w, u, sidx, scol, depth))
                return;
        } else {
            const uint32_t c = __ffs(row) - 1;
            const uint32_t off = st.off[c], len = st.len[c];
            for (; idx < len; ++idx) {
                const unsigned long long m = st.mask[off + idx];
                if (m & ~w)
                    continue;
                const TypeField f = st.field[st.type[off + idx]];
                if ((u & f.fm) >= f.cap)
                    continue;
                sidx |= (unsigned long long)idx << (8 * depth);
                scol |= c << (4 * depth);
                ++depth;
                w &= ~m;
                u += f.fm & (0ull - f.fm);
                idx = 0;
                down = true;
                break;
            }
        }
        if (down)
            continue;
        if (depth == 0)
            return;
        --depth;
        idx = (uint32_t)(sidx >> (8 * depth)) & 0xFFu;
        sidx &= ~(0xFFull << (8 * depth));
        const uint32_t c = (scol >> (4 * depth)) & 0xFu;
        scol &= ~(0xFu << (4 * depth));
        const uint32_t pi = st.off[c] + idx;
        w |= st.mask[pi];
        const unsigned long long fm = st.field[st.type[pi]].fm;
        u -= fm & (0ull - fm);
        ++idx;
    }
}

// Key codec -----------------------------------------------------------------
struct Codec {
    unsigned long long dynmask, usedmask, hi_board, in_shift, tag;
    uint32_t W, dyn_bits;

    // K64: window = kept rows | board rows below them; used above the window.
    __device__ __forceinline__ void parse64(unsigned long long key, unsigned long long &w,
                                            unsigned long long &u) const {
        w = (key & dynmask) | hi_board;
        u = (key >> dyn_bits) & usedmask;
    }
    __device__ __forceinline__ unsigned long long child64(unsigned long long w,
                                                          unsigned long long u) const {
        return ((w >> W) & dynmask) | (u << dyn_bits) | tag;
    }
};

__device__ __forceinline__ Codec make_codec(const SmemTable &st, unsigned long long hi_board,
                                            unsigned long long in_shift, unsigned long long tag) {
    Codec c;
    c.W = st.width;
    c.dyn_bits = st.dyn_bits;
    c.dynmask = (1ull << st.dyn_bits) - 1ull;
    c.usedmask = (1ull << st.used_bits) - 1ull;
    c.hi_board = hi_board;
    c.in_shift = in_shift;
    c.tag = tag;
    return c;
}

template <bool K64>
__device__ __forceinline__ void parse_key(const Codec &cd, unsigned long long k0,
                                          unsigned long long k1, unsigned long long &w,
                                          unsigned long long &u) {
    if constexpr (K64) {
        cd.parse64(k0, w, u);
    } else {
        w = k0;
        u = k1 & kUsedMask128;
    }
}

// Children staged per warp before the warp inserts them together.
constexpr int kWarps = kExpandBlock / 32;
constexpr int kStage = 64;
struct WarpStage {
    unsigned long long k0[kStage];
    unsigned long long k1[kStage];
    unsigned long long cnt[kStage];
    unsigned long long home[kStage];   // home slot within the instance's region
    uint32_t seg[kStage];   // producing segment | witness flag (bit 31)
};

// Inserts staged children into their instances' table regions.  An insert
// that reaches the probe limit marks its instance (kUniqueOverflow: the
// instance's row is redone with a larger region) and the status word.
// Returns, per lane, the instance id of the child it failed to insert
// (0xFFFFFFFF when none), so that lanes walking that instance can stop.
template <bool K64>
__device__ __forceinline__ uint32_t flush_children(const ExpandArgs &a, const WarpStage &ws,
                                                   int base, int n, unsigned lane) {
    // Lane i inserts child base + i: up to 32 independent inserts in flight.
    int r = 2;
    uint32_t inst = 0xFFFFFFFFu;
    if constexpr (K64) {
        if (a.append) {
            // Partitioned dedup: append to the child's bucket (the bucket
            // counters are few enough to stay in L2).
            if ((int)lane < n) {
                const int j = base + (int)lane;
                const unsigned long long key = ws.k0[j];
                const unsigned long long b = __umul64hi(mix64(key), a.n_bkt);
                const unsigned int pos = atomicAdd(a.bkt_cnt + b, 1u);
                if (pos < a.bkt_cap)
                    a.bkt_recs[b * a.bkt_cap + pos] = make_ulonglong2(key, ws.cnt[j]);
                else
                    atomicOr(a.status, kStatusBucketOverflow);
            }
            return 0xFFFFFFFFu;
        }
    }
    if ((int)lane < n) {
        const int j = base + (int)lane;
        const uint32_t si = ws.seg[j];
        const bool wmax = (si >> 31) != 0u;   // solve-one instance: value = witness
        const Seg &s = a.segs[si & 0x7FFFFFFFu];
        inst = s.inst;
        if constexpr (K64) {
            const unsigned long long h = a.prefetch ? ws.home[j] : home64(ws.k0[j], s.tcap);
            r = insert64_at(static_cast<Slot16 *>(a.table) + s.tbase, s.tcap, h, ws.k0[j],
                            ws.cnt[j], a.max_probe, wmax);
        } else {
            const unsigned long long h =
                a.prefetch ? ws.home[j] : home128(ws.k0[j], ws.k1[j], s.tcap);
            r = insert128_at(static_cast<Slot32 *>(a.table) + s.tbase, s.tcap, h, ws.k0[j],
                             ws.k1[j], ws.cnt[j], a.max_probe, wmax);
        }
    }
    if (r < 0)
        atomicOr(&a.inst_unique[inst], kUniqueOverflow);
    const bool over = __any_sync(0xffffffffu, r < 0);
    if (over && lane == 0)
        atomicOr(a.status, kStatusTableOverflow);
    // New keys per instance, aggregated over the lanes sharing an instance.
    const bool fresh = r == 1;
    const unsigned peers = __match_any_sync(0xffffffffu, fresh ? inst : 0xFFFFFFFFu);
    if (fresh && lane == (unsigned)(__ffs(peers) - 1))
        atomicAdd(&a.inst_unique[inst], (unsigned)__popc(peers));
    return r < 0 ? inst : 0xFFFFFFFFu;
}

// Expansion.  Warps work independently (no block barrier): each warp takes
// a chunk of work items from a global counter, and its lanes take items from
// that chunk as they become free.  A work item is one state with its first
// placement fixed (the state's walk split `fan` ways), so a state with
// thousands of row fills spreads over many lanes.  Every iteration of the
// warp loop performs exactly one step of each lane's depth-first walk --
// test one candidate placement and descend, or backtrack; a placement that
// completes the row emits its child in the same step and the walk stays at
// its node -- so the lanes do uniform work.  A launch over one instance reads its
// placement table and descriptor from shared memory (staged at block start);
// batched launches read every instance's tables through L1, and each lane
// keeps its own instance, so a warp may move to a chunk of another instance
// while some lanes finish earlier items.
// Completed rows are staged in shared memory and inserted by the whole
// warp, 32 at a time.
template <bool K64, bool U32, bool MW, bool PARTS>
__global__ void __launch_bounds__(kExpandBlock, 4)
k_expand(ExpandArgs a) {
    using UT = std::conditional_t<U32, uint32_t, unsigned long long>;
    __shared__ WarpStage stage[kWarps];
    const unsigned lane = threadIdx.x & 31u;
    // Partition claims: where each warp last found work (kept in shared
    // memory, off the walk's registers).
    __shared__ uint32_t s_part[kWarps];
    if (PARTS && lane == 0) {
        uint32_t smid;
        asm("mov.u32 %0, %%smid;" : "=r"(smid));
        s_part[threadIdx.x >> 5] = smid % a.parts;
    }
    // Single-instance launch: the instance's descriptor and placement table
    // staged in shared memory (dynamic), read there by every walk step.
    const InstDesc *st_d = nullptr;
    const Plc *st_plc = nullptr;
    if (a.stage_plc) {
        extern __shared__ __align__(16) unsigned char x_stage[];
        const InstDesc *gd = a.insts + a.segs[0].inst;
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(gd);
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(x_stage);
        for (uint32_t i = threadIdx.x; i < sizeof(InstDesc) / 8; i += blockDim.x)
            dst[i] = src[i];
        const ulonglong2 *ps = reinterpret_cast<const ulonglong2 *>(a.plc + gd->plc_off);
        ulonglong2 *pd = reinterpret_cast<ulonglong2 *>(x_stage + kStageDescBytes);
        const uint32_t np = gd->n_plc;
        for (uint32_t i = threadIdx.x; i < np; i += blockDim.x)
            pd[i] = ps[i];
        __syncthreads();
        st_d = reinterpret_cast<const InstDesc *>(x_stage);
        st_plc = reinterpret_cast<const Plc *>(x_stage + kStageDescBytes);
    }
    WarpStage &ws = stage[threadIdx.x >> 5];
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned long long raw = 0;

    // Warp-uniform chunk cursor.
    unsigned long long c_next = 0, c_end = 0;   // items of the current chunk not yet taken
    uint32_t c_seg = 0;
    bool no_more = false;

    // Lane walk state and context.
    bool active = false;
    const Seg *sg = nullptr;
    const InstDesc *d = nullptr;
    const Plc *plc = nullptr;
    uint32_t W = 0, rowmask = 0, dyn_bits = 0;
    unsigned long long usedmask = 0, dynmask = 0;
    unsigned long long w = 0, cnt = 0, sidx = 0;
    UT u = 0;
    bool wit = false;   // solve-one instance: cnt holds the parent's witness
    uint32_t scol = 0, depth = 0, idx = 0, min_depth = 0;
    unsigned long long rw = 0;   // walk state at the root of the lane's subtree
    UT ru = 0;
    int nbuf = 0;   // warp-uniform: staged children

    for (;;) {
        // ---- hand out items to idle lanes ----------------------------------
        unsigned need = __ballot_sync(0xffffffffu, !active);
        while (need && !no_more) {
            if (c_next >= c_end) {
                unsigned long long ci = ~0ull;
                if (lane == 0) {
                    if constexpr (PARTS) {
                        // Own partition first, then the following ones; a
                        // claim past a partition's end takes nothing.
                        const uint32_t cur_part = s_part[threadIdx.x >> 5];
                        for (uint32_t t = 0; t < a.parts; ++t) {
                            const uint32_t q = cur_part + t < a.parts ? cur_part + t
                                                                      : cur_part + t - a.parts;
                            const unsigned long long lo0 = a.part_step * q;
                            const unsigned long long lo = lo0 < a.n_chunks ? lo0 : a.n_chunks;
                            const unsigned long long hi0 = lo + a.part_step;
                            const unsigned long long hi = hi0 < a.n_chunks ? hi0 : a.n_chunks;
                            if (lo >= hi)
                                continue;
                            const unsigned long long o = atomicAdd(a.part_ctr + q, 1ull);
                            if (lo + o < hi) {
                                ci = lo + o;
                                s_part[threadIdx.x >> 5] = q;
                                break;
                            }
                        }
                    } else {
                        if (!(a.preempt && *(const volatile unsigned int *)a.preempt))
                            ci = atomicAdd(a.work, 1ull);
                    }
                }
                ci = __shfl_sync(0xffffffffu, ci, 0);
                if (ci >= a.n_chunks) {
                    no_more = true;
                    break;
                }
                // Segment holding chunk ci: last seg with chunk_base <= ci.
                uint32_t lo = 0, hi = a.n_segs - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (a.segs[mid].chunk_base <= ci)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                c_seg = lo;
                const Seg &s = a.segs[lo];
                c_next = s.begin + (ci - s.chunk_base) * a.chunk_states;
                const unsigned long long se = s.begin + s.len;
                c_end = c_next + a.chunk_states < se ? c_next + a.chunk_states : se;
                // An instance past its frontier limit fails anyway, and one
                // whose table region overflowed is redone: skip its work.
                // The counter changes under other warps, so one lane reads
                // it and the decision stays warp-uniform.
                const uint32_t lim = a.insts[s.inst].limit;
                uint32_t un = 0;
                if (lane == 0)
                    un = __ldcg(a.inst_unique + s.inst);
                un = __shfl_sync(0xffffffffu, un, 0);
                if ((un & kUniqueOverflow) || (lim && un > lim))
                    c_next = c_end;
            }
            const unsigned long long avail = c_end - c_next;
            const unsigned take = (unsigned)(avail < (unsigned long long)__popc(need)
                                                 ? avail
                                                 : (unsigned long long)__popc(need));
            // The first `take` needing lanes (in lane order) get items.
            const unsigned rank = __popc(need & lt_mask);
            if (((need >> lane) & 1u) && rank < take) {
                const unsigned long long item = c_next + rank;
                sg = a.segs + c_seg;
                d = st_d ? st_d : a.insts + sg->inst;
                plc = st_plc ? st_plc : a.plc + d->plc_off;
                W = d->width;
                rowmask = (1u << W) - 1u;
                dyn_bits = d->dyn_bits;
                dynmask = (1ull << dyn_bits) - 1ull;
                usedmask = (1ull << d->used_bits) - 1ull;
                // The item's state, and (a split segment) which first
                // placements it fixes: item - begin = (state * fan + second)
                // * fan + first.
                const uint32_t lvs = sg->levels;
                const uint32_t fs = lvs ? sg->fan : 1u;
                const uint32_t per = lvs == 2 ? fs * fs : fs;
                const unsigned long long rel = item - sg->begin;
                const unsigned long long si = sg->rec + (lvs ? rel / per : rel);
                const ulonglong2 rec = a.recs[si];
                wit = (d->flags & kInstWitness) != 0u;
                if constexpr (K64) {
                    w = (rec.x & dynmask) | sg->hi_board;
                    u = (UT)((rec.x >> dyn_bits) & usedmask);
                    cnt = wit ? witness64(rec.x, sg->tag) : rec.y;
                } else {
                    w = rec.x;
                    u = (UT)(rec.y & kUsedMask128);
                    cnt = wit ? witness128(rec.x, rec.y) : a.cnts[si];
                }
                sidx = 0;
                scol = 0;
                depth = 0;
                idx = 0;
                min_depth = 0;
                active = true;
                if (lvs) {
                    // Place this item's first choice (and, split two ways,
                    // its second) and walk only beneath them: min_depth =
                    // the placements fixed.  Items whose choices do not fit
                    // are empty; a row completed early is emitted by the one
                    // item whose remaining choices are 0.
                    const uint32_t rem = (uint32_t)(rel % per);   // per <= 2^16
                    uint32_t choice = rem % fs;
                    uint32_t later = rem / fs;   // choices below the current level
                    active = true;
                    for (uint32_t lv = 0; active && lv < lvs; ++lv) {
                        const uint32_t row = (uint32_t)w & rowmask;
                        if (row == 0) {
                            active = choice == 0 && later == 0;
                            break;
                        }
                        const uint32_t c = __ffs(row) - 1;
                        active = false;
                        if (choice < d->col_len[c]) {
                            const Plc p = plc[d->col_off[c] + choice];
                            if (!(p.mask & ~w)) {
                                if (plc_free<UT>(p, u)) {
                                    sidx |= (unsigned long long)choice << (8 * depth);
                                    scol |= c << (4 * depth);
                                    ++depth;
                                    w &= ~p.mask;
                                    u += plc_inc<UT>(p);
                                    active = true;
                                    min_depth = depth;
                                }
                            }
                        }
                        choice = later;
                        later = 0;
                    }
                }
                rw = w;
                ru = u;
            }
            c_next += take;
            need = __ballot_sync(0xffffffffu, !active);
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (no_more)
                break;
            continue;   // every item handed out was empty: hand out more
        }
        // ---- work donation: no items left, some lanes idle ------------------
        // A lane that has descended below its subtree root gives the rest of
        // the root node (candidates after its current root choice) to an
        // idle lane and keeps only the subtree of that choice.
        if (no_more) {
            const unsigned idle = __ballot_sync(0xffffffffu, !active);
            const unsigned donors = __ballot_sync(0xffffffffu, active && depth > min_depth);
            if (idle && donors) {
                const unsigned pairs = min(__popc(idle), __popc(donors));
                const unsigned irank = __popc(idle & lt_mask);
                const unsigned drank = __popc(donors & lt_mask);
                const bool recv = !active && irank < pairs;
                const bool give = active && depth > min_depth && drank < pairs;
                const int src = recv ? (int)__fns(donors, 0, (int)irank + 1) : (int)lane;
                // Donor's root choice and the start of the donated range.
                uint32_t ci = 0, cc = 0;
                if (give) {
                    ci = (uint32_t)(sidx >> (8 * min_depth)) & 0xFFu;
                    cc = (scol >> (4 * min_depth)) & 0xFu;
                }
                const unsigned long long d_rw = __shfl_sync(0xffffffffu, rw, src);
                const UT d_ru = __shfl_sync(0xffffffffu, ru, src);
                const unsigned long long d_cnt = __shfl_sync(0xffffffffu, cnt, src);
                const uint32_t d_idx = __shfl_sync(0xffffffffu, ci + 1, src);
                const unsigned long long d_sg =
                    __shfl_sync(0xffffffffu, (unsigned long long)sg, src);
                if (recv) {
                    sg = reinterpret_cast<const Seg *>(d_sg);
                    d = st_d ? st_d : a.insts + sg->inst;
                    wit = (d->flags & kInstWitness) != 0u;
                    plc = st_plc ? st_plc : a.plc + d->plc_off;
                    W = d->width;
                    rowmask = (1u << W) - 1u;
                    dyn_bits = d->dyn_bits;
                    dynmask = (1ull << dyn_bits) - 1ull;
                    usedmask = (1ull << d->used_bits) - 1ull;
                    w = rw = d_rw;
                    u = ru = d_ru;
                    cnt = d_cnt;
                    sidx = 0;
                    scol = 0;
                    depth = 0;
                    min_depth = 0;
                    idx = d_idx;
                    active = true;
                }
                if (give) {
                    // New subtree root: the old root with its choice placed.
                    const Plc p = plc[d->col_off[cc] + ci];
                    rw &= ~p.mask;
                    ru += plc_inc<UT>(p);
                    ++min_depth;
                }
            }
        }

        // ---- one walk step per lane -----------------------------------------
        bool emit = false, pop = false;
        unsigned long long ck0 = 0, ck1 = 0;
        if (active) {
            const uint32_t row = (uint32_t)w & rowmask;
            bool found = false;
            uint32_t c = 0;
            if (row == 0) {
                // Row complete at a work item's root: the child, then back up.
                emit = true;
                if constexpr (K64) {
                    ck0 = ((w >> W) & dynmask) | ((unsigned long long)u << dyn_bits) | sg->tag;
                } else {
                    ck0 = (w >> W) | sg->in_shift;
                    ck1 = (unsigned long long)u | sg->tag;
                }
                pop = true;
            } else {
                c = __ffs(row) - 1;
                // Next candidate >= idx whose row-0, row-1 and row-2 cells
                // fit: AND of the column's three filter bitsets.
                // Fixed filter layout (see build_piece_lib): offsets from
                // the column and the row patterns, no per-column loads.
                const uint32_t fw = d->fwords;
                const unsigned long long *fb = a.filt + d->filt_off;
                const uint32_t n0 = 1u << (W - 1);
                const unsigned long long *f0 =
                    fb + (unsigned long long)((c << (W - 1)) + (row >> (c + 1))) * fw;
                const unsigned long long *f1 =
                    fb + (unsigned long long)(W * n0 + (c << W) + ((uint32_t)(w >> W) & rowmask)) * fw;
                const unsigned long long *f2 =
                    fb + (unsigned long long)(W * n0 + (W << W) + (c << W) +
                                              ((uint32_t)(w >> (2 * W)) & rowmask)) * fw;
                // Words of this column's bitsets that can hold candidates: one
                // when every instance of the launch has single-word filters,
                // else as many as this column's placements need.
                const uint32_t cfw = MW ? (((uint32_t)d->col_len[c] + 63u) >> 6) : 1u;
                for (uint32_t k = idx >> 6; k < cfw; ++k) {
                    unsigned long long m = __ldg(f0 + k) & __ldg(f1 + k) & __ldg(f2 + k);
                    if (k == (idx >> 6))
                        m &= ~0ull << (idx & 63u);
                    if (m) {
                        idx = k * 64 + (uint32_t)(__ffsll((long long)m) - 1);
                        found = true;
                        break;
                    }
                }
                pop = !found;
            }
            // One placement load per step: the candidate to test, or, backing
            // up, the placement to undo (the column and index it was taken
            // at come off the fill stack).
            const bool up = pop && depth > min_depth;
            if (pop && !up)
                active = false;
            uint32_t pc = c, pi = idx;
            if (up) {
                --depth;
                pi = (uint32_t)(sidx >> (8 * depth)) & 0xFFu;
                sidx &= ~(0xFFull << (8 * depth));
                pc = (scol >> (4 * depth)) & 0xFu;
                scol &= ~(0xFu << (4 * depth));
            }
            if (found || up) {
                const Plc p = plc[d->col_off[pc] + pi];
                if (up) {
                    w |= p.mask;
                    u -= plc_inc<UT>(p);
                    idx = pi + 1;
                } else if (!(p.mask & ~w)) {
                    if (plc_free<UT>(p, u)) {
                        const unsigned long long nw = w & ~p.mask;
                        if (((uint32_t)nw & rowmask) == 0u) {
                            // The placement completes the row: the child is
                            // emitted here and the walk stays at this node.
                            emit = true;
                            const UT nu = u + plc_inc<UT>(p);
                            if constexpr (K64) {
                                ck0 = ((nw >> W) & dynmask) | ((unsigned long long)nu << dyn_bits) | sg->tag;
                            } else {
                                ck0 = (nw >> W) | sg->in_shift;
                                ck1 = (unsigned long long)nu | sg->tag;
                            }
                            ++idx;
                        } else {
                            sidx |= (unsigned long long)idx << (8 * depth);
                            scol |= c << (4 * depth);
                            ++depth;
                            w = nw;
                            u += plc_inc<UT>(p);
                            idx = 0;
                        }
                    } else {
                        idx = p.next_type;   // no copies left: skip the type's run
                    }
                } else {
                    ++idx;
                }
            }
        }
        // ---- stage this iteration's children (<= 32) after the staged ones --
        const unsigned em = __ballot_sync(0xffffffffu, emit);
        if (emit) {
            const int pos = nbuf + __popc(em & lt_mask);
            ws.k0[pos] = ck0;
            if constexpr (!K64)
                ws.k1[pos] = ck1;
            ws.cnt[pos] = cnt;
            ws.seg[pos] = (uint32_t)(sg - a.segs) | (wit ? 0x80000000u : 0u);
            // The child's home slot; for moderate tables its line is also
            // requested into L2 now, so the insert at the next flush finds it
            // there (on tables of many GB the extra line fills cost more
            // HBM bandwidth than the latency they hide: the host turns it
            // off).
            if (a.prefetch) {
                // (Only then: hashing here, on the few lanes that emit, costs
                // more issue slots than hashing in the converged flush.)
                const unsigned long long hr =
                    K64 ? home64(ck0, sg->tcap) : home128(ck0, ck1, sg->tcap);
                ws.home[pos] = hr;
                const void *line = K64 ? (const void *)(static_cast<const Slot16 *>(a.table) +
                                                        sg->tbase + hr)
                                       : (const void *)(static_cast<const Slot32 *>(a.table) +
                                                        sg->tbase + hr);
                asm volatile("prefetch.global.L2 [%0];" ::"l"(line));
            }
            ++raw;
        }
        nbuf += __popc(em);
        if (nbuf >= 32) {
            __syncwarp();
            const uint32_t failed = flush_children<K64>(a, ws, nbuf - 32, 32, lane);
            nbuf -= 32;
            __syncwarp();
            // Lanes walking an instance whose region just overflowed stop
            // (its row is redone); rare, so the 32-way compare is cheap.
            if (__any_sync(0xffffffffu, failed != 0xFFFFFFFFu)) {
                const uint32_t mine = active ? sg->inst : 0xFFFFFFFEu;
                bool hit = false;
                for (int q = 0; q < 32; q++)
                    hit |= __shfl_sync(0xffffffffu, failed, q) == mine;
                if (hit)
                    active = false;
            }
        }
    }
    if (nbuf > 0) {
        __syncwarp();
        flush_children<K64>(a, ws, 0, nbuf, lane);
        __syncwarp();
    }
    // One atomic per warp for the raw-children counter.
    unsigned long long tot = raw;
    for (int o = 16; o > 0; o >>= 1)
        tot += __shfl_down_sync(0xffffffffu, tot, o);
    if (lane == 0 && tot)
        atomicAdd(a.n_raw, tot);
}

// Compaction streams the table in tiles of kCompactTileBytes (2048 K64 or
// 1024 K128 slots; slot tile_base + j * kCompactBlock + thread for round j).
// The tiles come into shared memory by 1-D bulk copies (cp.async.bulk, the
// async copy engine), CompactArgs::stages deep per block (3 by default, two
// blocks per SM: ~64 KB of the table in flight per block while it works on
// the tile it holds; the launch plan can trade blocks for stages).  When
// every occupied slot of a tile belongs to one instance -- always for a
// single puzzle, and for every tile of a batch, whose instances own whole
// tiles -- the block computes output positions with ballots and one shared
// prefix and reserves them with ONE cursor atomic per tile, writing
// coalesced runs.  Tiles holding several instances reserve per round and warp
// with __match_any_sync aggregation instead.  Occupied slots are cleared in
// the table as they are taken.
constexpr int kCompactTileBytes = 32768;
constexpr int kCompactMaxStages = 6;
constexpr int kCompactWarps = kCompactBlock / 32;
// A staged tile that has not arrived after this long (never expected: the
// copy engine reads device memory the kernel owns) ends the launch with
// kStatusCompactStall instead of waiting on.
constexpr unsigned long long kCompactWaitNs = 2000000000ull;

template <bool K64>
__host__ __device__ constexpr int compact_per() {
    return kCompactTileBytes / (K64 ? 16 : 32) / kCompactBlock;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

// Arms the barrier for `bytes` of transfer (and the issuing thread's arrival).
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

// Waits for phase `parity` of the barrier for at most kCompactWaitNs;
// false on a timeout.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity))
        return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity))
            return true;
        if (global_ns() - t0 > kCompactWaitNs)
            return false;
    }
}

// Global -> shared bulk copy completing on `bar` (both addresses 16-byte
// aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes,
                                          unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Orders this thread's earlier shared-memory accesses before later
// async-proxy (bulk copy) accesses of the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Shared bookkeeping of one k_compact block.
template <int PER>
struct CompactShared {
    unsigned int cnt[PER][kCompactWarps];   // stored slots per round, warp
    uint32_t min[kCompactWarps], max[kCompactWarps];
    unsigned long long base, fin_sum;
    unsigned int fin_n;
};

// Moves one tile's occupied slots (already in registers: key words, value,
// instance id or 0xFFFFFFFF for an empty slot) to their instances' next
// frontier segments or final results.  Every thread of the block calls it.
template <bool K64, int PER>
__device__ __forceinline__ void compact_tile(const CompactArgs &a, CompactShared<PER> &sh,
                                             const unsigned long long (&k0)[PER],
                                             const unsigned long long (&k1)[PER],
                                             const unsigned long long (&cnt)[PER],
                                             const uint32_t (&inst)[PER]) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    uint32_t tmin = 0xFFFFFFFFu, tmax = 0u;
#pragma unroll
    for (int j = 0; j < PER; j++)
        if (inst[j] != 0xFFFFFFFFu) {
            tmin = min(tmin, inst[j]);
            tmax = max(tmax, inst[j]);
        }
    // Is the tile single-instance?
    for (int o = 16; o > 0; o >>= 1) {
        tmin = min(tmin, __shfl_xor_sync(0xffffffffu, tmin, o));
        tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
    }
    if (lane == 0) {
        sh.min[warp] = tmin;
        sh.max[warp] = tmax;
    }
    __syncthreads();
    uint32_t bmin = 0xFFFFFFFFu, bmax = 0u;
#pragma unroll
    for (int w = 0; w < kCompactWarps; w++) {
        bmin = min(bmin, sh.min[w]);
        bmax = max(bmax, sh.max[w]);
    }
    if (bmin == 0xFFFFFFFFu) {   // empty tile
        __syncthreads();
        return;
    }
    if (bmin == bmax) {
        // ---- single instance: one reservation for the tile -----------------
        const uint32_t in0 = bmin;
        const unsigned long long cur = a.cursor[in0];
        const bool fin = cur == kCursorFinal;
        const bool drop = cur == kCursorDrop;
        const unsigned long long km = a.keep_max ? a.keep_max[in0] : ~0ull;
        bool st[PER];
        unsigned long long fsum = 0;
        unsigned int fn = 0;
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const bool occ = inst[j] != 0xFFFFFFFFu;
            st[j] = occ && !fin && !drop;
            if (st[j] && km != ~0ull) {
                const unsigned long long wid =
                    K64 ? (k0[j] & ((1ull << a.inst_off) - 1ull)) : witness128(k0[j], k1[j]);
                st[j] = sample_hash(wid) <= km;
            }
            if (occ && fin) {
                fsum += cnt[j];
                fn++;
            }
            const unsigned b = __ballot_sync(0xffffffffu, st[j]);
            if (lane == 0)
                sh.cnt[j][warp] = __popc(b);
        }
        if (fin) {
            for (int o = 16; o > 0; o >>= 1) {
                fsum += __shfl_xor_sync(0xffffffffu, fsum, o);
                fn += __shfl_xor_sync(0xffffffffu, fn, o);
            }
            if (threadIdx.x == 0) {
                sh.fin_sum = 0;
                sh.fin_n = 0;
            }
        }
        __syncthreads();
        if (fin) {
            if (lane == 0 && fn) {
                atomicAdd(&sh.fin_sum, fsum);
                atomicAdd(&sh.fin_n, fn);
            }
            __syncthreads();
            if (threadIdx.x == 0 && sh.fin_n) {
                atomicAdd(&a.results[in0], sh.fin_sum);
                atomicAdd(&a.final_states[in0], sh.fin_n);
            }
            __syncthreads();
            return;
        }
        if (threadIdx.x == 0) {
            unsigned int total = 0;
            for (int j = 0; j < PER; j++)
                for (int w = 0; w < kCompactWarps; w++)
                    total += sh.cnt[j][w];
            sh.base = total ? atomicAdd(&a.cursor[in0], (unsigned long long)total) : 0ull;
        }
        __syncthreads();
        // Position = base + stored slots before (round j, warp, lane).
        unsigned long long pos = sh.base;
#pragma unroll
        for (int j = 0; j < PER; j++) {
            unsigned int before = 0, round_total = 0;
#pragma unroll
            for (int w = 0; w < kCompactWarps; w++) {
                before += w < (int)warp ? sh.cnt[j][w] : 0u;
                round_total += sh.cnt[j][w];
            }
            const unsigned b = __ballot_sync(0xffffffffu, st[j]);
            if (st[j]) {
                const unsigned long long p = pos + before + __popc(b & lt);
                if constexpr (K64) {
                    a.out_recs[p] = make_ulonglong2(k0[j], cnt[j]);
                } else {
                    a.out_recs[p] = make_ulonglong2(k0[j], k1[j]);
                    a.out_cnts[p] = cnt[j];
                }
            }
            pos += round_total;
        }
        __syncthreads();
        return;
    }
    // ---- several instances: warp-aggregated reservation per round ----------
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const bool occ = inst[j] != 0xFFFFFFFFu;
        const unsigned long long cur = occ ? a.cursor[inst[j]] : 0ull;
        const bool fin = occ && cur == kCursorFinal;
        bool store = occ && !fin && cur != kCursorDrop;
        if (store && a.keep_max) {
            const unsigned long long km = a.keep_max[inst[j]];
            if (km != ~0ull) {
                const unsigned long long wid =
                    K64 ? (k0[j] & ((1ull << a.inst_off) - 1ull)) : witness128(k0[j], k1[j]);
                store = sample_hash(wid) <= km;
            }
        }
        const unsigned peers = __match_any_sync(0xffffffffu, store ? inst[j] : 0xFFFFFFFFu);
        if (store) {
            const unsigned leader = __ffs(peers) - 1;
            unsigned long long basepos = 0;
            if (lane == leader)
                basepos = atomicAdd(&a.cursor[inst[j]], (unsigned long long)__popc(peers));
            basepos = __shfl_sync(peers, basepos, leader);
            const unsigned long long p = basepos + __popc(peers & lt);
            if constexpr (K64) {
                a.out_recs[p] = make_ulonglong2(k0[j], cnt[j]);
            } else {
                a.out_recs[p] = make_ulonglong2(k0[j], k1[j]);
                a.out_cnts[p] = cnt[j];
            }
        }
        if (fin) {
            atomicAdd(&a.results[inst[j]], cnt[j]);
            atomicAdd(&a.final_states[inst[j]], 1u);
        }
    }
    __syncthreads();
}

// Reads slot i of a staged tile (shared memory) into registers; returns the
// instance id, or 0xFFFFFFFF for an empty slot.
template <bool K64>
__device__ __forceinline__ uint32_t read_slot(const CompactArgs &a, const unsigned char *tile,
                                              uint32_t i, unsigned long long &k0,
                                              unsigned long long &k1, unsigned long long &cnt) {
    if constexpr (K64) {
        const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(tile)[i];
        k0 = v.x;
        k1 = 0;
        cnt = v.y;
        return v.x ? (uint32_t)((v.x >> a.inst_off) & a.inst_mask) : 0xFFFFFFFFu;
    } else {
        const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(tile)[2 * i];
        k0 = v.x;
        k1 = v.y;
        cnt = reinterpret_cast<const unsigned long long *>(tile)[4 * i + 2];
        return v.y ? (uint32_t)((v.y & ~kMarker) >> kInstShift128) : 0xFFFFFFFFu;
    }
}

template <bool K64>
__global__ void __launch_bounds__(kCompactBlock, 2)
k_compact(CompactArgs a) {
    constexpr int PER = compact_per<K64>();
    constexpr uint32_t kSlotBytes = K64 ? 16u : 32u;
    constexpr unsigned long long kTile = (unsigned long long)PER * kCompactBlock;   // slots
    extern __shared__ __align__(128) unsigned char c_stage[];
    __shared__ __align__(8) unsigned long long bars[kCompactMaxStages];
    const uint32_t S = a.stages;
    __shared__ CompactShared<PER> sh;
    const unsigned long long n_tiles = (a.cap + kTile - 1) / kTile;
    const unsigned long long mine =
        blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0ull;
    // Thread 0 issues the bulk copy of this block's k-th tile into stage k % S.
    auto issue = [&](unsigned long long k) {
        const unsigned long long first = (blockIdx.x + k * gridDim.x) * kTile;
        const unsigned long long n = a.cap - first < kTile ? a.cap - first : kTile;
        unsigned long long *bar = &bars[k % S];
        const uint32_t bytes = (uint32_t)n * kSlotBytes;
        mbar_expect_tx(bar, bytes);
        bulk_load(c_stage + (k % S) * kCompactTileBytes,
                  static_cast<const unsigned char *>(a.table) + first * kSlotBytes, bytes, bar);
    };
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; s++)
            mbar_init(&bars[s], 1);
        fence_mbar_init();
        fence_proxy_async_smem();
        for (unsigned long long k = 0; k < mine && k < (unsigned long long)S; k++)
            issue(k);
    }
    __syncthreads();
    unsigned long long k = 0;
    for (; k < mine; k++) {
        const int s = (int)(k % S);
        const uint32_t parity = (uint32_t)((k / S) & 1ull);
        const bool ok = mbar_wait_bounded(&bars[s], parity);
        if (__syncthreads_or(!ok))
            break;
        const unsigned long long tb = (blockIdx.x + k * gridDim.x) * kTile;
        const unsigned char *tile = c_stage + s * kCompactTileBytes;
        unsigned long long k0[PER], k1[PER], cnt[PER];
        uint32_t inst[PER];
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const uint32_t i = (uint32_t)j * kCompactBlock + threadIdx.x;
            inst[j] = 0xFFFFFFFFu;
            k0[j] = k1[j] = cnt[j] = 0;
            if (tb + i < a.cap)
                inst[j] = read_slot<K64>(a, tile, i, k0[j], k1[j], cnt[j]);
        }
        // Every thread has read the stage: refill it with tile k + S.
        __syncthreads();
        if (threadIdx.x == 0 && k + S < mine) {
            fence_proxy_async_smem();
            issue(k + S);
        }
        // Clear the taken slots for the next row.
#pragma unroll
        for (int j = 0; j < PER; j++)
            if (inst[j] != 0xFFFFFFFFu) {
                const unsigned long long i = tb + (unsigned long long)j * kCompactBlock + threadIdx.x;
                if constexpr (K64)
                    static_cast<ulonglong2 *>(a.table)[i] = make_ulonglong2(0, 0);
                else
                    static_cast<ulonglong4_32a *>(a.table)[i] = make_ulonglong4_32a(0, 0, 0, 0);
            }
        compact_tile<K64, PER>(a, sh, k0, k1, cnt, inst);
    }
    if (k < mine) {
        // A stage that did not arrive: report it, and let the copies still
        // in flight land (each wait bounded) before the block's shared memory
        // is given up.
        if (threadIdx.x == 0) {
            atomicOr(a.status, kStatusCompactStall);
            const unsigned long long last = mine < k + S ? mine : k + S;
            for (unsigned long long q = k; q < last; q++)
                mbar_wait_bounded(&bars[q % S],
                                  (uint32_t)((q / S) & 1ull));
        }
        __syncthreads();
    }
}

// Loads a tile straight into registers (no staging): the variant the staged
// kernel is measured against (D4E_COMPACT=ld).
template <bool K64>
__global__ void __launch_bounds__(kCompactBlock)
k_compact_ld(CompactArgs a) {
    constexpr int PER = compact_per<K64>();
    constexpr unsigned long long kTile = (unsigned long long)PER * kCompactBlock;
    __shared__ CompactShared<PER> sh;
    for (unsigned long long tb = (unsigned long long)blockIdx.x * kTile; tb < a.cap;
         tb += (unsigned long long)gridDim.x * kTile) {
        unsigned long long k0[PER], k1[PER], cnt[PER];
        uint32_t inst[PER];
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const unsigned long long i = tb + (unsigned long long)j * kCompactBlock + threadIdx.x;
            k0[j] = k1[j] = cnt[j] = 0;
            inst[j] = 0xFFFFFFFFu;
            if (i < a.cap) {
                if constexpr (K64) {
                    const ulonglong2 v = static_cast<const ulonglong2 *>(a.table)[i];
                    k0[j] = v.x;
                    cnt[j] = v.y;
                    if (v.x) {
                        inst[j] = (uint32_t)((v.x >> a.inst_off) & a.inst_mask);
                        static_cast<ulonglong2 *>(a.table)[i] = make_ulonglong2(0, 0);
                    }
                } else {
                    const ulonglong4_32a v = static_cast<const ulonglong4_32a *>(a.table)[i];
                    k0[j] = v.x;
                    k1[j] = v.y;
                    cnt[j] = v.z;
                    if (v.y) {
                        inst[j] = (uint32_t)((v.y & ~kMarker) >> kInstShift128);
                        static_cast<ulonglong4_32a *>(a.table)[i] =
                            make_ulonglong4_32a(0, 0, 0, 0);
                    }
                }
            }
        }
        compact_tile<K64, PER>(a, sh, k0, k1, cnt, inst);
    }
}

template <bool K64>
__global__ void k_keyset_insert(KeySetArgs t, const ulonglong2 *__restrict__ recs,
                                unsigned long long n) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const ulonglong2 k = recs[i];
        int r;
        if constexpr (K64)
            r = insert64(static_cast<Slot16 *>(t.table), t.cap, k.x, 0ull, t.max_probe);
        else
            r = insert128(static_cast<Slot32 *>(t.table), t.cap, k.x, k.y, 0ull, t.max_probe);
        if (r < 0)
            atomicOr(t.status, kStatusTableOverflow);
    }
}

template <bool K64>
__device__ __forceinline__ bool probe_child(const ProbeArgs &p, const Codec &cd,
                                            unsigned long long wd, unsigned long long ud,
                                            unsigned long long &ck0, unsigned long long &ck1) {
    if constexpr (K64) {
        ck0 = cd.child64(wd, ud);
        ck1 = 0ull;
        return find64(static_cast<const Slot16 *>(p.table), p.cap, ck0, p.max_probe);
    } else {
        ck0 = (wd >> cd.W) | cd.in_shift;
        ck1 = ud | cd.tag;
        return find128(static_cast<const Slot32 *>(p.table), p.cap, ck0, ck1, p.max_probe);
    }
}

template <bool K64>
__global__ void __launch_bounds__(kExpandBlock)
k_mark_alive(ProbeArgs p, const ulonglong2 *__restrict__ recs, unsigned long long n,
             unsigned char *__restrict__ alive) {
    __shared__ SmemTable st;
    load_table(st, p.insts + p.inst, p.plc);
    __syncthreads();
    const Codec cd = make_codec(st, p.hi_board, p.in_shift, p.tag);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const ulonglong2 k = recs[i];
        unsigned long long w, u;
        parse_key<K64>(cd, k.x, k.y, w, u);
        bool found = false;
        row_fills(st, w, u,
                  [&](unsigned long long wd, unsigned long long ud, unsigned long long, uint32_t,
                      uint32_t) {
                      unsigned long long a, b;
                      found = probe_child<K64>(p, cd, wd, ud, a, b);
                      return found;
                  });
        alive[i] = found ? 1 : 0;
    }
}

template <bool K64>
__global__ void __launch_bounds__(kExpandBlock)
k_extend_paths(ProbeArgs p, const PathNode *__restrict__ nodes, uint32_t n_nodes,
               PathNode *__restrict__ out, unsigned int *__restrict__ n_out, uint32_t max_out,
               unsigned int *__restrict__ status) {
    __shared__ SmemTable st;
    load_table(st, p.insts + p.inst, p.plc);
    __syncthreads();
    const Codec cd = make_codec(st, p.hi_board, p.in_shift, p.tag);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes;
         i += gridDim.x * blockDim.x) {
        const PathNode nd = nodes[i];
        unsigned long long w, u;
        parse_key<K64>(cd, nd.k0, nd.k1, w, u);
        row_fills(st, w, u,
                  [&](unsigned long long wd, unsigned long long ud, unsigned long long sidx,
                      uint32_t scol, uint32_t depth) {
                      unsigned long long ck0, ck1;
                      if (!probe_child<K64>(p, cd, wd, ud, ck0, ck1))
                          return false;
                      const unsigned pos = atomicAdd(n_out, 1u);
                      if (pos >= max_out) {
                          atomicOr(status, kStatusNodeOverflow);
                          return true;
                      }
                      PathNode o;
                      o.k0 = ck0;
                      o.k1 = ck1;
                      o.parent = i;
                      o.nfill = depth;
                      for (uint32_t d = 0; d < (uint32_t)kMaxWidth; d++) {
                          const uint32_t c = (scol >> (4 * d)) & 0xFu;
                          const uint32_t ix = (uint32_t)(sidx >> (8 * d)) & 0xFFu;
                          o.plc[d] = d < depth ? (uint16_t)(st.off[c] + ix) : (uint16_t)0xFFFFu;
                      }
                      out[pos] = o;
                      return false;
                  });
    }
}

// ---- listing over many instances: jobs dealt to blocks -----------------
// The job of block b: the last job whose blk_base <= b.
__device__ __forceinline__ uint32_t list_job_of(const ListJob *jobs, uint32_t n_jobs, uint32_t b) {
    uint32_t lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (jobs[mid].blk_base <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// The job's blocks: from its blk_base to the next job's (the last job runs
// to the grid's end).
__device__ __forceinline__ uint32_t list_job_blocks(const ListJob *jobs, uint32_t n_jobs,
                                                    uint32_t j) {
    return (j + 1 < n_jobs ? jobs[j + 1].blk_base : gridDim.x) - jobs[j].blk_base;
}

__device__ __forceinline__ ProbeArgs list_probe(const ProbeArgs &base, const ListJob &jb) {
    ProbeArgs p = base;
    p.inst = jb.inst;
    p.row = jb.row;
    p.in_shift = jb.in_shift;
    p.hi_board = jb.hi_board;
    p.tag = jb.tag;
    return p;
}

template <bool K64>
__global__ void k_keyset_insert_jobs(KeySetArgs t, const ListJob *__restrict__ jobs,
                                     uint32_t n_jobs) {
    const uint32_t j = list_job_of(jobs, n_jobs, blockIdx.x);
    const ListJob jb = jobs[j];
    const unsigned long long stride =
        (unsigned long long)list_job_blocks(jobs, n_jobs, j) * blockDim.x;
    for (unsigned long long i = (unsigned long long)(blockIdx.x - jb.blk_base) * blockDim.x +
                                threadIdx.x;
         i < jb.n; i += stride) {
        const ulonglong2 k = jb.recs[i];
        int r;
        if constexpr (K64)
            r = insert64(static_cast<Slot16 *>(t.table), t.cap, k.x, 0ull, t.max_probe);
        else
            r = insert128(static_cast<Slot32 *>(t.table), t.cap, k.x, k.y, 0ull, t.max_probe);
        if (r < 0)
            atomicOr(t.status, kStatusTableOverflow);
    }
}

template <bool K64>
__global__ void __launch_bounds__(kExpandBlock)
k_mark_select_jobs(ProbeArgs base, const ListJob *__restrict__ jobs, uint32_t n_jobs,
                   ulonglong2 *__restrict__ out, unsigned long long *__restrict__ n_out) {
    __shared__ SmemTable st;
    const uint32_t j = list_job_of(jobs, n_jobs, blockIdx.x);
    const ListJob jb = jobs[j];
    const ProbeArgs p = list_probe(base, jb);
    load_table(st, p.insts + p.inst, p.plc);
    __syncthreads();
    const Codec cd = make_codec(st, p.hi_board, p.in_shift, p.tag);
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride =
        (unsigned long long)list_job_blocks(jobs, n_jobs, j) * blockDim.x;
    // Warp-uniform trip count: every lane takes part in the ballot.
    for (unsigned long long base_i = (unsigned long long)(blockIdx.x - jb.blk_base) * blockDim.x;
         base_i < jb.n; base_i += stride) {
        const unsigned long long i = base_i + threadIdx.x;
        bool keep = false;
        ulonglong2 k = make_ulonglong2(0ull, 0ull);
        if (i < jb.n) {
            k = jb.recs[i];
            unsigned long long w, u;
            parse_key<K64>(cd, k.x, k.y, w, u);
            row_fills(st, w, u,
                      [&](unsigned long long wd, unsigned long long ud, unsigned long long,
                          uint32_t, uint32_t) {
                          unsigned long long a, b;
                          keep = probe_child<K64>(p, cd, wd, ud, a, b);
                          return keep;
                      });
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        unsigned long long b = 0;
        if (lane == 0 && m)
            b = atomicAdd(n_out + j, (unsigned long long)__popc(m));
        b = __shfl_sync(0xffffffffu, b, 0);
        if (keep)
            out[jb.out_off + b + __popc(m & ((1u << lane) - 1u))] = k;
    }
}

template <bool K64>
__global__ void __launch_bounds__(kExpandBlock)
k_extend_paths_jobs(ProbeArgs base, const ListJob *__restrict__ jobs, uint32_t n_jobs,
                    PathNode *__restrict__ out, unsigned int *__restrict__ n_out,
                    unsigned int *__restrict__ status) {
    __shared__ SmemTable st;
    const uint32_t j = list_job_of(jobs, n_jobs, blockIdx.x);
    const ListJob jb = jobs[j];
    const ProbeArgs p = list_probe(base, jb);
    load_table(st, p.insts + p.inst, p.plc);
    __syncthreads();
    const Codec cd = make_codec(st, p.hi_board, p.in_shift, p.tag);
    const unsigned long long stride =
        (unsigned long long)list_job_blocks(jobs, n_jobs, j) * blockDim.x;
    for (unsigned long long i = (unsigned long long)(blockIdx.x - jb.blk_base) * blockDim.x +
                                threadIdx.x;
         i < jb.n; i += stride) {
        const PathNode nd = jb.nodes[i];
        unsigned long long w, u;
        parse_key<K64>(cd, nd.k0, nd.k1, w, u);
        row_fills(st, w, u,
                  [&](unsigned long long wd, unsigned long long ud, unsigned long long sidx,
                      uint32_t scol, uint32_t depth) {
                      unsigned long long ck0, ck1;
                      if (!probe_child<K64>(p, cd, wd, ud, ck0, ck1))
                          return false;
                      const unsigned pos = atomicAdd(n_out + j, 1u);
                      if (pos >= jb.out_cap) {
                          atomicOr(status, kStatusNodeOverflow);
                          return true;
                      }
                      PathNode o;
                      o.k0 = ck0;
                      o.k1 = ck1;
                      o.parent = (uint32_t)i;
                      o.nfill = depth;
                      for (uint32_t d = 0; d < (uint32_t)kMaxWidth; d++) {
                          const uint32_t c = (scol >> (4 * d)) & 0xFu;
                          const uint32_t ix = (uint32_t)(sidx >> (8 * d)) & 0xFFu;
                          o.plc[d] = d < depth ? (uint16_t)(st.off[c] + ix) : (uint16_t)0xFFFFu;
                      }
                      out[jb.out_off + pos] = o;
                      return false;
                  });
    }
}

// Partitioned dedup, second half: one bucket per block iteration.
constexpr int kMergeBlock = 512;
constexpr unsigned kMergeProbe = 256;

__global__ void __launch_bounds__(kMergeBlock)
k_bucket_merge(MergeArgs m) {
    extern __shared__ Slot16 tab[];   // kBucketSlots slots
    __shared__ unsigned int s_over;
    const unsigned lane = threadIdx.x & 31u;
    for (unsigned i = threadIdx.x; i < kBucketSlots; i += blockDim.x)
        tab[i] = Slot16{0ull, 0ull};
    if (threadIdx.x == 0)
        s_over = 0;
    __syncthreads();
    for (unsigned long long b = blockIdx.x; b < m.n_bkt; b += gridDim.x) {
        const unsigned int n = min(m.bkt_cnt[b], (unsigned int)m.bkt_cap);
        const ulonglong2 *recs = m.bkt_recs + b * m.bkt_cap;
        for (unsigned int base = 0; base < n; base += blockDim.x) {
            const unsigned int i = base + threadIdx.x;
            int r = 2;
            uint32_t inst = 0xFFFFFFFFu;
            if (i < n) {
                const ulonglong2 rec = recs[i];
                inst = (uint32_t)((rec.x >> m.inst_off) & m.inst_mask);
                const bool wmax = (m.insts[inst].flags & kInstWitness) != 0u;
                // Bucket = high bits of the hash; the slot = its low bits.
                unsigned h = (unsigned)mix64(rec.x) & (kBucketSlots - 1u);
                r = -1;
                for (unsigned p = 0; p < kMergeProbe; ++p) {
                    unsigned long long k = *reinterpret_cast<volatile unsigned long long *>(&tab[h].key);
                    if (k == 0ull) {
                        k = atomicCAS(&tab[h].key, 0ull, rec.x);
                        if (k == 0ull) {
                            if (wmax)
                                atomicMax(&tab[h].cnt, rec.y);
                            else
                                atomicAdd(&tab[h].cnt, rec.y);
                            r = 1;
                            break;
                        }
                    }
                    if (k == rec.x) {
                        if (wmax)
                            atomicMax(&tab[h].cnt, rec.y);
                        else
                            atomicAdd(&tab[h].cnt, rec.y);
                        r = 0;
                        break;
                    }
                    h = (h + 1u) & (kBucketSlots - 1u);
                }
                if (r < 0)
                    s_over = 1;
            }
            // New keys per instance, warp-aggregated.
            const bool fresh = r == 1;
            const unsigned peers = __match_any_sync(0xffffffffu, fresh ? inst : 0xFFFFFFFFu);
            if (fresh && lane == (unsigned)(__ffs(peers) - 1))
                atomicAdd(&m.inst_unique[inst], (unsigned)__popc(peers));
        }
        __syncthreads();
        // The bucket's table, empties included, is its slice of dtab.
        Slot16 *out = m.dtab + b * kBucketSlots;
        for (unsigned i = threadIdx.x; i < kBucketSlots; i += blockDim.x) {
            out[i] = tab[i];
            tab[i] = Slot16{0ull, 0ull};
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && s_over)
        atomicOr(m.status, kStatusBucketOverflow);
}

__global__ void k_select(const ulonglong2 *__restrict__ recs, const unsigned char *__restrict__ alive,
                         unsigned long long n, ulonglong2 *__restrict__ out,
                         unsigned long long *__restrict__ n_out) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < n;
         base += stride) {
        const unsigned long long i = base + threadIdx.x;
        const bool keep = i < n && alive[i];
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        unsigned long long b = 0;
        if (lane == 0 && m)
            b = atomicAdd(n_out, (unsigned long long)__popc(m));
        b = __shfl_sync(0xffffffffu, b, 0);
        if (keep)
            out[b + __popc(m & ((1u << lane) - 1u))] = recs[i];
    }
}

__global__ void k_count_pattern(const ulonglong2 *__restrict__ recs, unsigned long long n,
                                unsigned long long mask, unsigned long long value,
                                unsigned long long *__restrict__ out) {
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long c = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride)
        c += (recs[i].x & mask) == value;
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c)
        atomicAdd(out, c);
}

}  // namespace

cudaError_t expand_max_blocks_per_sm(bool k64, int *n) {
    return k64 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                     n, k_expand<true, false, true, false>, kExpandBlock, 0)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                     n, k_expand<false, false, true, false>, kExpandBlock, 0);
}

void launch_expand(bool k64, const ExpandArgs &a, int grid, cudaStream_t s) {
    if (a.n_chunks == 0)
        return;
    const size_t dyn = a.stage_plc ? expand_stage_bytes(a.stage_plc) : 0;
    // Partition claims (multi-instance packed-key launches) are a separate
    // instantiation, so that the other launches keep the plain claim's
    // registers.
    if (k64 && a.parts)
        if (a.u32)
            a.single_word ? k_expand<true, true, false, true><<<grid, kExpandBlock, dyn, s>>>(a)
                          : k_expand<true, true, true, true><<<grid, kExpandBlock, dyn, s>>>(a);
        else
            a.single_word ? k_expand<true, false, false, true><<<grid, kExpandBlock, dyn, s>>>(a)
                          : k_expand<true, false, true, true><<<grid, kExpandBlock, dyn, s>>>(a);
    else if (k64)
        if (a.u32)
            a.single_word ? k_expand<true, true, false, false><<<grid, kExpandBlock, dyn, s>>>(a)
                          : k_expand<true, true, true, false><<<grid, kExpandBlock, dyn, s>>>(a);
        else
            a.single_word ? k_expand<true, false, false, false><<<grid, kExpandBlock, dyn, s>>>(a)
                          : k_expand<true, false, true, false><<<grid, kExpandBlock, dyn, s>>>(a);
    else
        a.single_word ? k_expand<false, false, false, false><<<grid, kExpandBlock, dyn, s>>>(a)
                      : k_expand<false, false, true, false><<<grid, kExpandBlock, dyn, s>>>(a);
}

namespace {
// D4E_COMPACT=ld selects the unstaged compaction (for measurements).
bool compact_unstaged() {
    static const bool ld = [] {
        const char *v = std::getenv("D4E_COMPACT");
        return v && std::strcmp(v, "ld") == 0;
    }();
    return ld;
}
}  // namespace

int compact_grid(unsigned long long cap, int sms, int per_sm) {
    // Tiles of 32 KB (2048 K64 or 1024 K128 slots; the smaller count bounds
    // the grid either way).
    const unsigned long long tiles = (cap + 1023) / 1024;
    const unsigned long long per = compact_unstaged() ? 8ull : (unsigned long long)per_sm;
    return (int)std::max<unsigned long long>(
        1ull, std::min<unsigned long long>(tiles, (unsigned long long)sms * per));
}

bool compact_plan_ok(int per_sm, uint32_t stages) {
    return per_sm >= 1 && stages >= 2 && stages <= (uint32_t)kCompactMaxStages &&
           (size_t)per_sm * stages * kCompactTileBytes <= 200u * 1024u;
}

void launch_compact(bool k64, const CompactArgs &a, int grid, cudaStream_t s) {
    if (a.cap == 0)
        return;
    if (compact_unstaged()) {
        if (k64)
            k_compact_ld<true><<<grid, kCompactBlock, 0, s>>>(a);
        else
            k_compact_ld<false><<<grid, kCompactBlock, 0, s>>>(a);
        return;
    }
    // The staging ring is dynamic shared memory beyond the default 48 KB.
    CompactArgs b = a;
    if (b.stages < 2 || b.stages > (uint32_t)kCompactMaxStages)
        b.stages = kCompactDefaultStages;
    const int smem = (int)b.stages * kCompactTileBytes;
    if (k64) {
        cudaFuncSetAttribute(k_compact<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        k_compact<true><<<grid, kCompactBlock, smem, s>>>(b);
    } else {
        cudaFuncSetAttribute(k_compact<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        k_compact<false><<<grid, kCompactBlock, smem, s>>>(b);
    }
}

void launch_keyset_insert(bool k64, const KeySetArgs &t, const ulonglong2 *recs,
                          unsigned long long n, int grid, cudaStream_t s) {
    if (n == 0)
        return;
    if (k64)
        k_keyset_insert<true><<<grid, 256, 0, s>>>(t, recs, n);
    else
        k_keyset_insert<false><<<grid, 256, 0, s>>>(t, recs, n);
}

void launch_mark_alive(bool k64, const ProbeArgs &p, const ulonglong2 *recs,
                       unsigned long long n, unsigned char *alive, int grid, cudaStream_t s) {
    if (n == 0)
        return;
    if (k64)
        k_mark_alive<true><<<grid, kExpandBlock, 0, s>>>(p, recs, n, alive);
    else
        k_mark_alive<false><<<grid, kExpandBlock, 0, s>>>(p, recs, n, alive);
}

void launch_extend_paths(bool k64, const ProbeArgs &p, const PathNode *nodes, uint32_t n_nodes,
                         PathNode *out, unsigned int *n_out, uint32_t max_out,
                         unsigned int *status, int grid, cudaStream_t s) {
    if (n_nodes == 0)
        return;
    if (k64)
        k_extend_paths<true><<<grid, kExpandBlock, 0, s>>>(p, nodes, n_nodes, out, n_out, max_out,
                                                           status);
    else
        k_extend_paths<false><<<grid, kExpandBlock, 0, s>>>(p, nodes, n_nodes, out, n_out,
                                                            max_out, status);
}

uint32_t list_blocks(unsigned long long n) {
    const unsigned long long b = (n + kExpandBlock - 1) / kExpandBlock;
    return (uint32_t)std::min<unsigned long long>(std::max<unsigned long long>(b, 1), kListMaxBlocks);
}

void launch_keyset_insert_jobs(bool k64, const KeySetArgs &t, const ListJob *jobs,
                               uint32_t n_jobs, uint32_t blocks, cudaStream_t s) {
    if (n_jobs == 0 || blocks == 0)
        return;
    if (k64)
        k_keyset_insert_jobs<true><<<blocks, kExpandBlock, 0, s>>>(t, jobs, n_jobs);
    else
        k_keyset_insert_jobs<false><<<blocks, kExpandBlock, 0, s>>>(t, jobs, n_jobs);
}

void launch_mark_select_jobs(bool k64, const ProbeArgs &p, const ListJob *jobs, uint32_t n_jobs,
                             uint32_t blocks, ulonglong2 *out, unsigned long long *n_out,
                             cudaStream_t s) {
    if (n_jobs == 0 || blocks == 0)
        return;
    if (k64)
        k_mark_select_jobs<true><<<blocks, kExpandBlock, 0, s>>>(p, jobs, n_jobs, out, n_out);
    else
        k_mark_select_jobs<false><<<blocks, kExpandBlock, 0, s>>>(p, jobs, n_jobs, out, n_out);
}

void launch_extend_paths_jobs(bool k64, const ProbeArgs &p, const ListJob *jobs, uint32_t n_jobs,
                              uint32_t blocks, PathNode *out, unsigned int *n_out,
                              unsigned int *status, cudaStream_t s) {
    if (n_jobs == 0 || blocks == 0)
        return;
    if (k64)
        k_extend_paths_jobs<true><<<blocks, kExpandBlock, 0, s>>>(p, jobs, n_jobs, out, n_out,
                                                                  status);
    else
        k_extend_paths_jobs<false><<<blocks, kExpandBlock, 0, s>>>(p, jobs, n_jobs, out, n_out,
                                                                   status);
}

void launch_select(const ulonglong2 *recs, const unsigned char *alive, unsigned long long n,
                   ulonglong2 *out, unsigned long long *n_out, int grid, cudaStream_t s) {
    if (n == 0)
        return;
    k_select<<<grid, 256, 0, s>>>(recs, alive, n, out, n_out);
}

void launch_count_pattern(const ulonglong2 *recs, unsigned long long n, unsigned long long mask,
                          unsigned long long value, unsigned long long *out, int grid,
                          cudaStream_t s) {
    if (n == 0)
        return;
    k_count_pattern<<<grid, 256, 0, s>>>(recs, n, mask, value, out);
}

cudaError_t bucket_merge_prepare() {
    return cudaFuncSetAttribute(k_bucket_merge, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(kBucketSlots * sizeof(Slot16)));
}

void launch_bucket_merge(const MergeArgs &m, int grid, cudaStream_t s) {
    if (m.n_bkt == 0)
        return;
    k_bucket_merge<<<grid, kMergeBlock, kBucketSlots * sizeof(Slot16), s>>>(m);
}

}  // namespace d4e
