// trace.cu -- solve-one reconstruction and range copies (sm_103a).
//
// A solve-one instance keeps every frontier level; each record's value is
// the largest witness (instance-free identity) of its parents.  k_trace
// walks one chosen final state back to the root through those witnesses and
// recovers the placements of every row, for all finished instances of a
// step in one launch.
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

// (wid, x, y) lexicographic order, for deterministic choices.
__device__ __forceinline__ bool tuple_gt(unsigned long long a0, unsigned long long a1,
                                         unsigned long long a2, unsigned long long b0,
                                         unsigned long long b1, unsigned long long b2) {
    if (a0 != b0)
        return a0 > b0;
    if (a1 != b1)
        return a1 > b1;
    return a2 > b2;
}

template <bool K64>
__global__ void __launch_bounds__(kTraceBlock)
k_trace(const InstDesc *__restrict__ insts, const Plc *__restrict__ plc_all,
        const LevelPtr *__restrict__ levels, const TraceJob *__restrict__ jobs, uint32_t n_jobs,
        TraceOut *__restrict__ out) {
    __shared__ unsigned long long chain[kTraceWarps][kMaxHeight + 1];
    const unsigned lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
    for (uint32_t j = blockIdx.x * kTraceWarps + wi; j < n_jobs; j += gridDim.x * kTraceWarps) {
        const TraceJob jb = jobs[j];
        const InstDesc *d = insts + jb.inst;
        const Plc *plc = plc_all + d->plc_off;
        const uint32_t H = jb.height;
        const LevelPtr *lv = levels + jb.lvl;
        bool ok = true;
        unsigned long long target = 0;
        // ---- back from the final level to the root -----------------------
        for (int r = (int)H; r >= 0; --r) {
            const LevelPtr L = lv[r];
            bool has = false;
            unsigned long long bw = 0, bx = 0, by = 0, bi = 0;
            for (unsigned long long i = lane; i < L.len; i += 32) {
                const ulonglong2 rec = L.recs[i];
                const unsigned long long wid =
                    K64 ? witness64(rec.x, jb.tag) : witness128(rec.x, rec.y);
                if ((r == (int)H || wid == target) &&
                    (!has || tuple_gt(wid, rec.x, rec.y, bw, bx, by))) {
                    has = true;
                    bw = wid;
                    bx = rec.x;
                    by = rec.y;
                    bi = i;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const bool oh = __shfl_xor_sync(0xffffffffu, has, o);
                const unsigned long long ow = __shfl_xor_sync(0xffffffffu, bw, o);
                const unsigned long long ox = __shfl_xor_sync(0xffffffffu, bx, o);
                const unsigned long long oy = __shfl_xor_sync(0xffffffffu, by, o);
                const unsigned long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (oh && (!has || tuple_gt(ow, ox, oy, bw, bx, by))) {
                    has = true;
                    bw = ow;
                    bx = ox;
                    by = oy;
                    bi = oi;
                }
            }
            if (!has) {
                ok = false;
                break;
            }
            if (lane == 0)
                chain[wi][r] = bi;
            if (r > 0)
                target = K64 ? L.recs[bi].y : L.cnts[bi];
        }
        __syncwarp();
        // ---- each row's fill from the chosen parent to the chosen child ----
        bool fill_fail = false;
        if (ok) {
            const uint32_t W = d->width;
            const uint32_t rowmask = (1u << W) - 1u;
            const unsigned long long dynmask = (1ull << d->dyn_bits) - 1ull;
            const unsigned long long usedmask = (1ull << d->used_bits) - 1ull;
            for (uint32_t r = lane; r < H; r += 32) {
                const ulonglong2 p = lv[r].recs[chain[wi][r]];
                const ulonglong2 c = lv[r + 1].recs[chain[wi][r + 1]];
                unsigned long long w, u;
                if constexpr (K64) {
                    w = (p.x & dynmask) | hi_board(d, r);
                    u = (p.x >> d->dyn_bits) & usedmask;
                } else {
                    w = p.x;
                    u = p.y & kUsedMask128;
                }
                const unsigned long long shin = K64 ? 0ull : in_shift(d, r);
                // Depth-first walk over the row's fills (same order as k_expand).
                unsigned long long sidx = 0;
                uint32_t scol = 0, depth = 0, idx = 0;
                bool found = false;
                for (;;) {
                    const uint32_t row = (uint32_t)w & rowmask;
                    bool down = false;
                    if (row == 0) {
                        bool match;
                        if constexpr (K64)
                            match = (((w >> W) & dynmask) | (u << d->dyn_bits) | jb.tag) == c.x;
                        else
                            match = ((w >> W) | shin) == c.x && (u | jb.tag) == c.y;
                        if (match) {
                            found = true;
                            break;
                        }
                    } else {
                        const uint32_t col = __ffs(row) - 1;
                        const uint32_t off = d->col_off[col], len = d->col_len[col];
                        for (; idx < len; ++idx) {
                            const Plc pl = plc[off + idx];
                            if (pl.mask & ~w)
                                continue;
                            const TypeField f = d->types[pl.type];
                            if ((u & f.fm) >= f.cap)
                                continue;
                            sidx |= (unsigned long long)idx << (8 * depth);
                            scol |= col << (4 * depth);
                            ++depth;
                            w &= ~pl.mask;
                            u += f.fm & (0ull - f.fm);
                            idx = 0;
                            down = true;
                            break;
                        }
                    }
                    if (down)
                        continue;
                    if (depth == 0)
                        break;
                    --depth;
                    idx = (uint32_t)(sidx >> (8 * depth)) & 0xFFu;
                    sidx &= ~(0xFFull << (8 * depth));
                    const uint32_t col = (scol >> (4 * depth)) & 0xFu;
                    scol &= ~(0xFu << (4 * depth));
                    const Plc pl = plc[d->col_off[col] + idx];
                    w |= pl.mask;
                    const unsigned long long fm = d->types[pl.type].fm;
                    u -= fm & (0ull - fm);
                    ++idx;
                }
                if (found) {
                    out[j].nfill[r] = (uint8_t)depth;
                    for (uint32_t k = 0; k < depth; k++) {
                        const uint32_t col = (scol >> (4 * k)) & 0xFu;
                        const uint32_t ix = (uint32_t)(sidx >> (8 * k)) & 0xFFu;
                        out[j].plc[r][k] = (uint16_t)(d->col_off[col] + ix);
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

void launch_trace(bool k64, const InstDesc *insts, const Plc *plc, const LevelPtr *levels,
                  const TraceJob *jobs, uint32_t n_jobs, TraceOut *out, int grid,
                  cudaStream_t s) {
    if (n_jobs == 0)
        return;
    if (k64)
        k_trace<true><<<grid, kTraceBlock, 0, s>>>(insts, plc, levels, jobs, n_jobs, out);
    else
        k_trace<false><<<grid, kTraceBlock, 0, s>>>(insts, plc, levels, jobs, n_jobs, out);
}

void launch_copy_ranges(const ulonglong2 *src, const unsigned long long *src_cnts, ulonglong2 *dst,
                        unsigned long long *dst_cnts, const CopyRange *ranges, uint32_t n,
                        int grid, cudaStream_t s) {
    if (n == 0)
        return;
    k_copy_ranges<<<grid, 256, 0, s>>>(src, src_cnts, dst, dst_cnts, ranges, n);
}

}  // namespace d4e
