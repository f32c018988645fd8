// kernels.cu -- sm_103a kernels of the row-by-row polyomino tiling engine.
//
// Hot path (one launch pair per board row):
//   k_expand  : replaces the reference's tiled_row_search / linear_row_search
//               + impl<H> (src/kernel.cuh:12-227).  Each state is expanded by
//               every whole-row fill -- a depth-first walk over placements
//               anchored at the lowest empty cell of the current row, with
//               the placement table staged in shared memory -- and each child
//               is inserted straight into an HBM-resident open-addressing
//               table (128-bit key CAS + 64-bit count add), which replaces
//               the reference's ring buffer + host hash-set Sorter
//               (src/device.cu:14-309, src/sorter.cpp:72-214).
//   k_compact : moves the table into the next frontier, instance by
//               instance, clearing it for the next row.
#include "kernels.h"

#include <cuda_runtime.h>

namespace d4e {

namespace {

constexpr int kExpandBlock = 256;
constexpr int kCompactBlock = 256;

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ unsigned long long hash_key(unsigned long long k0, unsigned long long k1) {
    return mix64(k0 ^ mix64(k1 ^ 0x9e3779b97f4a7c15ull));
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

// Home slot of a key in a table of `cap` slots (any capacity): the high
// half of hash * cap maps the 64-bit hash uniformly onto [0, cap).
__device__ __forceinline__ unsigned long long home_slot(unsigned long long k0, unsigned long long k1,
                                                        unsigned long long cap) {
    return __umul64hi(hash_key(k0, k1), cap);
}

// Insert (k0, k1) with multiplicity cnt (linear probing).  Returns 1 for a
// newly claimed key, 0 for an existing one, -1 when the probe limit was
// reached.
__device__ __forceinline__ int table_insert(Slot *__restrict__ T, unsigned long long cap,
                                            unsigned long long k0, unsigned long long k1,
                                            unsigned long long cnt, unsigned int max_probe) {
    unsigned long long h = home_slot(k0, k1, cap);
    for (unsigned int p = 0; p < max_probe; ++p) {
        unsigned long long o0, o1;
        cas128(&T[h].k0, 0ull, 0ull, k0, k1, o0, o1);
        const bool claimed = (o0 | o1) == 0ull;
        if (claimed || (o0 == k0 && o1 == k1)) {
            atomicAdd(&T[h].cnt, cnt);
            return claimed ? 1 : 0;
        }
        h = h + 1 == cap ? 0ull : h + 1;
    }
    return -1;
}

__device__ __forceinline__ bool table_find(const Slot *__restrict__ T, unsigned long long cap,
                                           unsigned long long k0, unsigned long long k1,
                                           unsigned int max_probe) {
    unsigned long long h = home_slot(k0, k1, cap);
    for (unsigned int p = 0; p < max_probe; ++p) {
        const ulonglong2 k = *reinterpret_cast<const ulonglong2 *>(&T[h].k0);
        if (k.x == k0 && k.y == k1)
            return true;
        if ((k.x | k.y) == 0ull)
            return false;
        h = h + 1 == cap ? 0ull : h + 1;
    }
    return false;
}

// Shared-memory copy of one instance's placement table.
struct SmemTable {
    Plc plc[kMaxPlc];
    uint16_t off[kMaxWidth];
    uint16_t len[kMaxWidth];
    uint32_t width;
};

__device__ __forceinline__ void load_table(SmemTable &st, const InstDesc *__restrict__ d,
                                           const Plc *__restrict__ plc_all) {
    const uint32_t np = d->n_plc;
    const Plc *src = plc_all + d->plc_off;
    for (uint32_t i = threadIdx.x; i < np; i += blockDim.x)
        st.plc[i] = src[i];
    if (threadIdx.x < kMaxWidth) {
        st.off[threadIdx.x] = d->col_off[threadIdx.x];
        st.len[threadIdx.x] = d->col_len[threadIdx.x];
    }
    if (threadIdx.x == 0)
        st.width = d->width;
}

// Depth-first enumeration of the whole-row fills of one state.  The fill
// stack lives in two registers: 8-bit placement index and 4-bit anchor
// column per depth (a row of <= 8 cells takes <= 8 placements).  A placement
// is undone by restoring its cells and dropping the highest used copy bit of
// its type.  `emit(child_window, used, sidx, scol, depth)` is called at every
// completed row; returning true stops the walk.
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
            if (emit(w >> W, u, sidx, scol, depth))
                return;
        } else {
            const uint32_t c = __ffs(row) - 1;
            const uint32_t off = st.off[c], len = st.len[c];
            for (; idx < len; ++idx) {
                const Plc p = st.plc[off + idx];
                if (p.mask & ~w)
                    continue;
                const unsigned long long ut = u & p.tm;
                const unsigned long long nb = (ut + (p.tm & (0ull - p.tm))) & p.tm;
                if (!nb)
                    continue;
                sidx |= (unsigned long long)idx << (8 * depth);
                scol |= c << (4 * depth);
                ++depth;
                w &= ~p.mask;
                u |= nb;
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
        const Plc p = st.plc[st.off[c] + idx];
        w |= p.mask;
        const unsigned long long ut = u & p.tm;
        u &= ~(ut & ~(ut >> 1));
        ++idx;
    }
}

__global__ void __launch_bounds__(kExpandBlock)
k_expand(ExpandArgs a) {
    __shared__ SmemTable st;
    __shared__ Seg s_seg;
    __shared__ unsigned long long s_ci;
    uint32_t loaded = 0xFFFFFFFFu;
    unsigned long long raw = 0;
    const unsigned lane = threadIdx.x & 31u;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned long long ci = atomicAdd(a.work, 1ull);
            s_ci = ci;
            if (ci < a.n_chunks) {
                // Segment holding chunk ci: last seg with chunk_base <= ci.
                uint32_t lo = 0, hi = a.n_segs - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (a.segs[mid].chunk_base <= ci)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                s_seg = a.segs[lo];
            }
        }
        __syncthreads();
        const unsigned long long ci = s_ci;
        if (ci >= a.n_chunks)
            break;
        const Seg sg = s_seg;
        if (sg.inst != loaded) {
            load_table(st, a.insts + sg.inst, a.plc);
            __syncthreads();
            loaded = sg.inst;
        }
        const unsigned long long first = sg.begin + (ci - sg.chunk_base) * a.chunk_states;
        const unsigned long long segend = sg.begin + sg.len;
        const unsigned long long last =
            first + a.chunk_states < segend ? first + a.chunk_states : segend;
        const unsigned long long in_shift = sg.in_shift;
        const uint32_t inst = sg.inst;
        for (unsigned long long s = first + threadIdx.x; s < last; s += blockDim.x) {
            const ulonglong2 key = a.keys[s];
            const unsigned long long cnt = a.cnts[s];
            row_fills(st, key.x, key.y,
                      [&](unsigned long long cw, unsigned long long u, unsigned long long,
                          uint32_t, uint32_t) {
                          ++raw;
                          const int r = table_insert(a.table, a.cap, cw | in_shift, u, cnt,
                                                     a.max_probe);
                          if (r < 0)
                              atomicOr(a.status, kStatusTableOverflow);
                          // All lanes of a warp work on the same chunk, hence the
                          // same instance: aggregate the new-key count per warp.
                          const unsigned act = __activemask();
                          const unsigned fresh = __ballot_sync(act, r == 1);
                          if (fresh && lane == (unsigned)(__ffs(fresh) - 1))
                              atomicAdd(&a.inst_unique[inst], (unsigned)__popc(fresh));
                          return false;
                      });
        }
    }
    // Reconverged here: one atomic per warp for the raw-children counter.
    unsigned long long tot = raw;
    for (int o = 16; o > 0; o >>= 1)
        tot += __shfl_down_sync(0xffffffffu, tot, o);
    if (lane == 0 && tot)
        atomicAdd(a.n_raw, tot);
}

__global__ void __launch_bounds__(kCompactBlock)
k_compact(CompactArgs a) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < a.cap;
         base += stride) {
        const unsigned long long i = base + threadIdx.x;
        Slot s{0, 0, 0, 0};
        if (i < a.cap) {
            const ulonglong4_32a v = *reinterpret_cast<const ulonglong4_32a *>(&a.table[i]);
            s.k0 = v.x;
            s.k1 = v.y;
            s.cnt = v.z;
        }
        const bool occ = s.k1 != 0ull;
        const uint32_t inst = occ ? (uint32_t)((s.k1 & ~kMarker) >> kInstShift) : 0xFFFFFFFFu;
        unsigned long long cur = occ ? a.cursor[inst] : 0ull;
        const bool fin = occ && cur == kCursorFinal;
        const bool store = occ && !fin;
        // Warp-aggregated cursor bump per instance.
        const unsigned peers = __match_any_sync(0xffffffffu, store ? inst : 0xFFFFFFFFu);
        if (store) {
            const unsigned leader = __ffs(peers) - 1;
            unsigned long long basepos = 0;
            if (lane == leader)
                basepos = atomicAdd(&a.cursor[inst], (unsigned long long)__popc(peers));
            basepos = __shfl_sync(peers, basepos, leader);
            const unsigned long long pos = basepos + __popc(peers & ((1u << lane) - 1u));
            a.out_keys[pos] = make_ulonglong2(s.k0, s.k1);
            a.out_cnts[pos] = s.cnt;
        }
        if (fin) {
            atomicAdd(&a.results[inst], s.cnt);
            atomicAdd(&a.final_states[inst], 1u);
        }
        if (occ)
            *reinterpret_cast<ulonglong4_32a *>(&a.table[i]) = make_ulonglong4_32a(0, 0, 0, 0);
    }
}

__global__ void k_keyset_insert(KeySetArgs t, const ulonglong2 *__restrict__ keys,
                                unsigned long long n) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const ulonglong2 k = keys[i];
        if (table_insert(t.table, t.cap, k.x, k.y, 0ull, t.max_probe) < 0)
            atomicOr(t.status, kStatusTableOverflow);
    }
}

__global__ void __launch_bounds__(kExpandBlock)
k_mark_alive(ProbeArgs p, const ulonglong2 *__restrict__ keys, unsigned long long n,
             unsigned char *__restrict__ alive) {
    __shared__ SmemTable st;
    load_table(st, p.insts + p.inst, p.plc);
    __syncthreads();
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const ulonglong2 k = keys[i];
        bool found = false;
        row_fills(st, k.x, k.y,
                  [&](unsigned long long cw, unsigned long long u, unsigned long long, uint32_t,
                      uint32_t) {
                      found = table_find(p.table, p.cap, cw | p.in_shift, u, p.max_probe);
                      return found;
                  });
        alive[i] = found ? 1 : 0;
    }
}

__global__ void __launch_bounds__(kExpandBlock)
k_extend_paths(ProbeArgs p, const PathNode *__restrict__ nodes, uint32_t n_nodes,
               PathNode *__restrict__ out, unsigned int *__restrict__ n_out, uint32_t max_out,
               unsigned int *__restrict__ status) {
    __shared__ SmemTable st;
    load_table(st, p.insts + p.inst, p.plc);
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes;
         i += gridDim.x * blockDim.x) {
        const PathNode nd = nodes[i];
        row_fills(st, nd.k0, nd.k1,
                  [&](unsigned long long cw, unsigned long long u, unsigned long long sidx,
                      uint32_t scol, uint32_t depth) {
                      const unsigned long long ck = cw | p.in_shift;
                      if (!table_find(p.table, p.cap, ck, u, p.max_probe))
                          return false;
                      const unsigned pos = atomicAdd(n_out, 1u);
                      if (pos >= max_out) {
                          atomicOr(status, kStatusNodeOverflow);
                          return true;
                      }
                      PathNode o;
                      o.k0 = ck;
                      o.k1 = u;
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

__global__ void k_select(const ulonglong2 *__restrict__ keys, const unsigned char *__restrict__ alive,
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
            out[b + __popc(m & ((1u << lane) - 1u))] = keys[i];
    }
}

__global__ void k_count_pattern(const ulonglong2 *__restrict__ keys, unsigned long long n,
                                unsigned long long mask, unsigned long long value,
                                unsigned long long *__restrict__ out) {
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long c = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += stride)
        c += (keys[i].x & mask) == value;
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c)
        atomicAdd(out, c);
}

}  // namespace

void launch_count_pattern(const ulonglong2 *keys, unsigned long long n, unsigned long long mask,
                          unsigned long long value, unsigned long long *out, int grid,
                          cudaStream_t s) {
    if (n == 0)
        return;
    k_count_pattern<<<grid, 256, 0, s>>>(keys, n, mask, value, out);
}

cudaError_t expand_max_blocks_per_sm(int *n) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, k_expand, kExpandBlock, 0);
}

void launch_expand(const ExpandArgs &a, int grid, cudaStream_t s) {
    if (a.n_chunks == 0)
        return;
    k_expand<<<grid, kExpandBlock, 0, s>>>(a);
}

void launch_compact(const CompactArgs &a, int grid, cudaStream_t s) {
    if (a.cap == 0)
        return;
    k_compact<<<grid, kCompactBlock, 0, s>>>(a);
}

void launch_keyset_insert(const KeySetArgs &t, const ulonglong2 *keys, unsigned long long n,
                          int grid, cudaStream_t s) {
    if (n == 0)
        return;
    k_keyset_insert<<<grid, 256, 0, s>>>(t, keys, n);
}

void launch_mark_alive(const ProbeArgs &p, const ulonglong2 *keys, unsigned long long n,
                       unsigned char *alive, int grid, cudaStream_t s) {
    if (n == 0)
        return;
    k_mark_alive<<<grid, kExpandBlock, 0, s>>>(p, keys, n, alive);
}

void launch_extend_paths(const ProbeArgs &p, const PathNode *nodes, uint32_t n_nodes,
                         PathNode *out, unsigned int *n_out, uint32_t max_out,
                         unsigned int *status, int grid, cudaStream_t s) {
    if (n_nodes == 0)
        return;
    k_extend_paths<<<grid, kExpandBlock, 0, s>>>(p, nodes, n_nodes, out, n_out, max_out, status);
}

void launch_select(const ulonglong2 *keys, const unsigned char *alive, unsigned long long n,
                   ulonglong2 *out, unsigned long long *n_out, int grid, cudaStream_t s) {
    if (n == 0)
        return;
    k_select<<<grid, 256, 0, s>>>(keys, alive, n, out, n_out);
}

}  // namespace d4e
