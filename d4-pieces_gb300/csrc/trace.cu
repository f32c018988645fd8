// trace.cu -- solve-one reconstruction and range copies (sm_103a).
//
// A solve-one instance keeps every frontier level; each record's value is
// the largest witness (instance-free identity) of its parents.  The trace
// passes walk one chosen final state back to the root through those
// witnesses, level by level over all finished instances of a step at once
// (every record is read once, by the whole GPU), and k_trace_fill recovers
// the placements of every row.
#include "kernels.h"

#include <cuda_runtime.h>

#include "state_hash.cuh"

namespace d4e {

namespace {

constexpr int kTraceBlock = 256;
constexpr int kTraceWarps = kTraceBlock / 32;

// Board rows [row + dyn_rows, row + R) in window coordinates (K64 keys keep
// only the first dyn_rows rows of the window).
__device__ __forceinline__ unsigned long long hi_board(const InstDesc *d, uint32_t row) {
    const uint32_t W = d->width, R = d->win_rows;
    const uint32_t dyn_rows = d->dyn_bits / W;
    unsigned long long hi = 0;
    for (uint32_t i = dyn_rows; i < R; i++)
        if (row + i < d->height)
            hi |= (unsigned long long)d->rows[row + i] << (i * W);
    return hi;
}

// Board row row + R entering the last window row after the shift (K128).
__device__ __forceinline__ unsigned long long in_shift(const InstDesc *d, uint32_t row) {
    const uint32_t W = d->width, R = d->win_rows;
    const uint32_t src = row + R;
    return src < d->height ? (unsigned long long)d->rows[src] << ((R - 1) * W) : 0ull;
}

// Identity of a kept record (the value its children's witnesses use).
template <bool K64>
__device__ __forceinline__ unsigned long long record_id(const ulonglong2 &rec,
                                                        unsigned long long tag) {
    return K64 ? witness64(rec.x, tag) : witness128(rec.x, rec.y);
}

// Flattened record index -> segment (binary search over segment bases).
__device__ __forceinline__ uint32_t find_seg(const TraceSeg *segs, uint32_t n,
                                             unsigned long long i) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (segs[mid].base <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// pass 0: best identity of the final level; pass 1: choose the final state
// with it; pass 2: choose the parent matching the witness one level up.
template <bool K64>
__global__ void __launch_bounds__(kTraceBlock)
k_trace_pass(int pass, const LevelPtr *__restrict__ levels, const TraceJob *__restrict__ jobs,
             const TraceSeg *__restrict__ segs, uint32_t n_segs, unsigned long long total,
             TraceChain *__restrict__ chain) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
         i < total; i += stride) {
        const TraceSeg sg = segs[find_seg(segs, n_segs, i)];
        const TraceJob &jb = jobs[sg.job];
        const LevelPtr L = levels[jb.lvl + sg.level];
        const unsigned long long k = i - sg.base;
        const ulonglong2 rec = L.recs[k];
        const unsigned long long id = record_id<K64>(rec, jb.tag);
        TraceChain &ch = chain[sg.job];
        if (pass == 0) {
            atomicMax(&ch.best, id);
        } else {
            const unsigned long long want = pass == 1 ? ch.best : ch.tgt[sg.level + 1];
            // The identity names one state of the level (K64 exactly; K128
            // up to a 64-bit fingerprint collision).
            if (id == want) {
                ch.idx[sg.level] = k + 1;
                ch.tgt[sg.level] = K64 ? rec.y : L.cnts[k];
            }
        }
    }
}

// Parent state (w, u) of row r of a traced job, and what its chosen child
// says about the row's fill: the cells it covers below the current row
// (allow_hi) and the copies it places per type (delta, in counter-field
// coordinates: child counters - parent counters, field by field).
template <bool K64>
struct RowLink {
    unsigned long long w, u, allow_hi, delta;
    unsigned long long cx, cy, dynmask, tag, shin;
    uint32_t W, dyn_bits;
    __device__ __forceinline__ bool operator()(unsigned long long w2, unsigned long long u2) const {
        if constexpr (K64)
            return (((w2 >> W) & dynmask) | (u2 << dyn_bits) | tag) == cx;
        else
            return ((w2 >> W) | shin) == cx && (u2 | tag) == cy;
    }
};

template <bool K64>
__device__ __forceinline__ bool row_link(const InstDesc *d, const LevelPtr *lv,
                                         const TraceChain &ch, uint32_t r, unsigned long long tag,
                                         RowLink<K64> &L) {
    if (ch.idx[r] == 0 || ch.idx[r] - 1 >= lv[r].len || ch.idx[r + 1] == 0 ||
        ch.idx[r + 1] - 1 >= lv[r + 1].len)
        return false;
    const ulonglong2 p = lv[r].recs[ch.idx[r] - 1];
    const ulonglong2 c = lv[r + 1].recs[ch.idx[r + 1] - 1];
    L.W = d->width;
    L.dyn_bits = d->dyn_bits;
    L.dynmask = (1ull << d->dyn_bits) - 1ull;
    L.tag = tag;
    L.cx = c.x;
    L.cy = c.y;
    const unsigned long long usedmask = (1ull << d->used_bits) - 1ull;
    unsigned long long child_window, cu;
    if constexpr (K64) {
        L.w = (p.x & L.dynmask) | hi_board(d, r);
        L.u = (p.x >> d->dyn_bits) & usedmask;
        L.shin = 0;
        child_window = (c.x & L.dynmask) | hi_board(d, r + 1);
        cu = (c.x >> d->dyn_bits) & usedmask;
    } else {
        L.w = p.x;
        L.u = p.y & kUsedMask128;
        L.shin = in_shift(d, r);
        child_window = c.x ^ L.shin;
        cu = c.y & kUsedMask128;
    }
    // After the fill, window rows 1.. of the parent must equal the child's
    // rows 0.. : the fill covers exactly the parent's cells there that the
    // child no longer has.
    const unsigned long long row0 = (1ull << L.W) - 1ull;
    L.allow_hi = L.w & ~row0 & ~(child_window << L.W);
    L.delta = cu - L.u;   // fields never borrow: each child field >= the parent's
    return true;
}

// First fill (depth-first order, k_expand's) from the linked parent that
// gives the linked child.  Candidates are restricted to the child's cells
// and counter deltas, which removes only fills that cannot give the child,
// so the walk stays short.  On success sidx / scol / depth describe it.
template <bool K64>
__device__ __forceinline__ bool find_fill(const InstDesc *d, const Plc *plc, const RowLink<K64> &L,
                                          unsigned long long &sidx, uint32_t &scol,
                                          uint32_t &depth) {
    const uint32_t W = d->width;
    const uint32_t rowmask = (1u << W) - 1u;
    const unsigned long long row0 = (unsigned long long)rowmask;
    unsigned long long w = L.w, u = L.u, delta = L.delta;
    sidx = 0;
    scol = 0;
    depth = 0;
    uint32_t idx = 0;
    for (;;) {
        const uint32_t row = (uint32_t)w & rowmask;
        bool down = false;
        if (row == 0) {
            if (L(w, u))
                return true;
        } else {
            const uint32_t col = __ffs(row) - 1;
            const uint32_t off = d->col_off[col], len = d->col_len[col];
            for (; idx < len; ++idx) {
                const Plc pl = plc[off + idx];
                if ((pl.mask & ~w) || (pl.mask & ~row0 & ~L.allow_hi))
                    continue;
                const TypeField f = d->types[pl.type];
                if ((u & f.fm) >= f.cap || !(delta & f.fm))
                    continue;
                sidx |= (unsigned long long)idx << (8 * depth);
                scol |= col << (4 * depth);
                ++depth;
                w &= ~pl.mask;
                const unsigned long long one = f.fm & (0ull - f.fm);
                u += one;
                delta -= one;
                idx = 0;
                down = true;
                break;
            }
        }
        if (down)
            continue;
        if (depth == 0)
            return false;
        --depth;
        idx = (uint32_t)(sidx >> (8 * depth)) & 0xFFu;
        sidx &= ~(0xFFull << (8 * depth));
        const uint32_t col = (scol >> (4 * depth)) & 0xFu;
        scol &= ~(0xFu << (4 * depth));
        const Plc pl = plc[d->col_off[col] + idx];
        w |= pl.mask;
        const unsigned long long fm = d->types[pl.type].fm;
        const unsigned long long one = fm & (0ull - fm);
        u -= one;
        delta += one;
        ++idx;
    }
}

template <bool K64>
__global__ void __launch_bounds__(kTraceBlock)
k_trace_fill(const InstDesc *__restrict__ insts, const Plc *__restrict__ plc_all,
             const LevelPtr *__restrict__ levels, const TraceJob *__restrict__ jobs,
             uint32_t n_jobs, const TraceChain *__restrict__ chain, TraceOut *__restrict__ out) {
    const unsigned lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
    for (uint32_t j = blockIdx.x * kTraceWarps + wi; j < n_jobs; j += gridDim.x * kTraceWarps) {
        const TraceJob jb = jobs[j];
        const InstDesc *d = insts + jb.inst;
        const uint32_t H = jb.height;
        const LevelPtr *lv = levels + jb.lvl;
        bool ok = true, fill_fail = false;
        for (uint32_t r = lane; r <= H; r += 32)
            if (chain[j].idx[r] == 0 || chain[j].idx[r] - 1 >= lv[r].len)
                ok = false;
        ok = __all_sync(0xffffffffu, ok);
        if (ok) {
            for (uint32_t r = lane; r < H; r += 32) {
                RowLink<K64> L;
                unsigned long long sidx = 0;
                uint32_t scol = 0, depth = 0;
                const bool found = row_link<K64>(d, lv, chain[j], r, jb.tag, L) &&
                                   find_fill<K64>(d, plc_all + d->plc_off, L, sidx, scol, depth);
                if (found) {
                    out[j].nfill[r] = (uint8_t)depth;
                    for (uint32_t q = 0; q < depth; q++) {
                        const uint32_t col = (scol >> (4 * q)) & 0xFu;
                        const uint32_t ix = (uint32_t)(sidx >> (8 * q)) & 0xFFu;
                        out[j].plc[r][q] = (uint16_t)(d->col_off[col] + ix);
                    }
                } else {
                    out[j].nfill[r] = 0;
                    fill_fail = true;
                }
            }
        }
        const bool any_fail = __any_sync(0xffffffffu, fill_fail);
        if (lane == 0)
            out[j].status = !ok ? 1u : (any_fail ? 2u : 0u);
        __syncwarp();
    }
}

__global__ void __launch_bounds__(256)
k_copy_ranges(const ulonglong2 *__restrict__ src, const unsigned long long *__restrict__ src_cnts,
              ulonglong2 *__restrict__ dst, unsigned long long *__restrict__ dst_cnts,
              const CopyRange *__restrict__ ranges, uint32_t n) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n; k += warps) {
        const CopyRange rg = ranges[k];
        for (unsigned long long i = lane; i < rg.len; i += 32) {
            dst[rg.dst + i] = src[rg.src + i];
            if (src_cnts)
                dst_cnts[rg.dst + i] = src_cnts[rg.src + i];
        }
    }
}

}  // namespace

void launch_trace_pass(bool k64, int pass, const LevelPtr *levels, const TraceJob *jobs,
                       const TraceSeg *segs, uint32_t n_segs, unsigned long long total,
                       TraceChain *chain, int grid, cudaStream_t s) {
    if (n_segs == 0 || total == 0)
        return;
    if (k64)
        k_trace_pass<true><<<grid, kTraceBlock, 0, s>>>(pass, levels, jobs, segs, n_segs, total,
                                                        chain);
    else
        k_trace_pass<false><<<grid, kTraceBlock, 0, s>>>(pass, levels, jobs, segs, n_segs, total,
                                                         chain);
}

void launch_trace_fill(bool k64, const InstDesc *insts, const Plc *plc, const LevelPtr *levels,
                       const TraceJob *jobs, uint32_t n_jobs, const TraceChain *chain,
                       TraceOut *out, int grid, cudaStream_t s) {
    if (n_jobs == 0)
        return;
    if (k64)
        k_trace_fill<true><<<grid, kTraceBlock, 0, s>>>(insts, plc, levels, jobs, n_jobs, chain,
                                                        out);
    else
        k_trace_fill<false><<<grid, kTraceBlock, 0, s>>>(insts, plc, levels, jobs, n_jobs, chain,
                                                         out);
}

void launch_copy_ranges(const ulonglong2 *src, const unsigned long long *src_cnts, ulonglong2 *dst,
                        unsigned long long *dst_cnts, const CopyRange *ranges, uint32_t n,
                        int grid, cudaStream_t s) {
    if (n == 0)
        return;
    k_copy_ranges<<<grid, 256, 0, s>>>(src, src_cnts, dst, dst_cnts, ranges, n);
}

}  // namespace d4e
