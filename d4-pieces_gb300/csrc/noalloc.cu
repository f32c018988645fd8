// noalloc.cu -- a tiling-count entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: processes that reserve their device
// memory once at start-up and may not grow it afterwards (a serving process
// sharing the GPU with other tenants under a fixed budget, where an
// allocation mid-request can fail or stall behind other work), or code that
// runs under a caller-owned memory pool that forbids the runtime allocator.
// d4e_count_noalloc serves them: every device buffer it needs -- placement
// table, instance descriptor, both frontier buffers, the de-duplication table
// and the counters -- is carved out of one file-scope __device__ array of
// kNoAllocScratchBytes, which every GPU that loads the library holds until
// the process exits.  The caller passes the puzzle (host memory) and
// receives the count (host memory).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/d4e.h"
#include "abi_util.h"
#include "engine.h"
#include "geometry.h"
#include "kernels.h"

namespace {

using namespace d4e;

constexpr size_t kNoAllocScratchBytes = (size_t)D4E_NOALLOC_SCRATCH_BYTES;

// The scratch array.  In host code its name is only a host-side stand-in:
// kernels get the device address resolved by cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, resolved once
// per device (the first call on each device does this set-up).
unsigned char *scratch_address(int dev) {
    if (dev < 0 || dev >= kMaxDevices)
        throw Error(kErrUnsupported, "device index beyond the scratch table");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
        g_scratch_ptr[dev] = p;
    }
    return static_cast<unsigned char *>(g_scratch_ptr[dev]);
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Largest candidate-filter block of one instance (the fixed layout of
// build_piece_lib): W * 2^(W-1) row-0 bitsets plus 2 * W * 2^W row-1 and
// row-2 bitsets, each of ceil(placements per column / 64) words; for W = 8
// and 255 placements per column that is (1024 + 4096) * 4 = 20480 words.
constexpr size_t kMaxFilterWords =
    ((size_t)kMaxWidth << (kMaxWidth - 1)) * ((kMaxPlcPerCol + 63) / 64) +
    2 * ((size_t)kMaxWidth << kMaxWidth) * ((kMaxPlcPerCol + 63) / 64);
static_assert(kMaxFilterWords == 20480, "filter region of the widest instance");

struct Layout {
    size_t desc, seg, misc, plc, filt, front[2], cnts[2], table;
    uint64_t cap_states, cap_slots;
};

// Fixed header (descriptor, segment, counters, placements), then two
// frontier buffers and a table of twice their capacity.
Layout make_layout(bool k64) {
    Layout L{};
    size_t off = 0;
    L.desc = off;
    off = align256(off + sizeof(InstDesc));
    L.seg = off;
    off = align256(off + sizeof(Seg));
    L.misc = off;
    off = align256(off + 256);
    L.plc = off;
    off = align256(off + sizeof(Plc) * kMaxPlc);
    L.filt = off;
    off = align256(off + sizeof(unsigned long long) * kMaxFilterWords);
    const size_t rec = 16, cntb = k64 ? 0 : 8, slot = k64 ? 16 : 32;
    const size_t per_state = 2 * (rec + cntb) + 2 * slot;
    const uint64_t n = (kNoAllocScratchBytes - off - 4 * 256) / per_state;
    L.cap_states = n;
    L.cap_slots = 2 * n;
    for (int i = 0; i < 2; i++) {
        L.front[i] = off;
        off = align256(off + rec * n);
        L.cnts[i] = off;
        off = align256(off + cntb * n);
    }
    L.table = off;
    return L;
}

}  // namespace

extern "C" int d4e_count_noalloc(const d4e_instance *inst, void *stream, uint64_t *count,
                                 uint64_t *states) {
    return abi_guarded([&] {
        if (!inst || !count || !inst->rows || (inst->n_pieces && (!inst->shapes || !inst->counts)))
            return abi_fail(D4E_ERR_INVALID, "null pointer");
        const uint32_t W = inst->width, H = inst->height;
        if (W < 1 || W > (uint32_t)kMaxWidth || H < 1 || H > (uint32_t)kMaxHeight)
            return abi_fail(D4E_ERR_INVALID, "board size out of range");
        for (uint32_t r = 0; r < H; r++)
            if (inst->rows[r] >> W)
                return abi_fail(D4E_ERR_INVALID, "board row has cells beyond the width");
        PieceLib lib;
        const std::string e = build_piece_lib(inst->shapes, inst->counts, inst->n_pieces, inst->sym,
                                              W, lib);
        if (!e.empty())
            return abi_fail(e.find("more than") != std::string::npos ? D4E_ERR_UNSUPPORTED
                                                                     : D4E_ERR_INVALID,
                            e);
        // The header regions are sized for the largest tables the builder
        // accepts; check anyway, so that a table never spills into the
        // frontier buffers that follow it.
        if (lib.filters.size() > kMaxFilterWords || lib.plc.size() > (size_t)kMaxPlc)
            return abi_fail(D4E_ERR_UNSUPPORTED,
                            "placement or filter tables larger than the no-alloc scratch "
                            "reserves for them");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        int dev = 0;
        cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        unsigned char *base = scratch_address(dev);

        const bool k64 = lib.dyn_bits + lib.used_bits <= 63;
        const Layout L = make_layout(k64);
        InstDesc d{};
        d.width = W;
        d.height = H;
        d.win_rows = 64 / W;
        d.n_plc = (uint32_t)lib.plc.size();
        d.plc_off = 0;
        d.filt_off = 0;
        d.fwords = lib.fwords;
        for (int c = 0; c < kMaxWidth; c++) {
            d.f0_off[c] = lib.f0_off[c];
            d.f1_off[c] = lib.f1_off[c];
            d.f2_off[c] = lib.f2_off[c];
        }
        d.n_types = (uint32_t)lib.fields.size();
        d.dyn_bits = lib.dyn_bits;
        d.used_bits = lib.used_bits;
        for (int c = 0; c < kMaxWidth; c++) {
            d.col_off[c] = lib.col_off[c];
            d.col_len[c] = lib.col_len[c];
        }
        for (uint32_t t = 0; t < d.n_types; t++)
            d.types[t] = lib.fields[t];
        for (uint32_t r = 0; r < H; r++)
            d.rows[r] = inst->rows[r];
        unsigned long long w0 = 0;
        for (uint32_t r = 0; r < std::min(d.win_rows, H); r++)
            w0 |= (unsigned long long)inst->rows[r] << (r * W);

        InstDesc *d_desc = reinterpret_cast<InstDesc *>(base + L.desc);
        Seg *d_seg = reinterpret_cast<Seg *>(base + L.seg);
        unsigned int *d_status = reinterpret_cast<unsigned int *>(base + L.misc);
        unsigned int *d_unique = d_status + 1;
        unsigned int *d_final = d_status + 2;
        unsigned long long *d_raw = reinterpret_cast<unsigned long long *>(base + L.misc + 64);
        unsigned long long *d_work = d_raw + 1;
        unsigned long long *d_cursor = d_raw + 2;
        unsigned long long *d_result = d_raw + 3;
        Plc *d_plc = reinterpret_cast<Plc *>(base + L.plc);
        unsigned long long *d_filt = reinterpret_cast<unsigned long long *>(base + L.filt);
        ulonglong2 *d_front[2] = {reinterpret_cast<ulonglong2 *>(base + L.front[0]),
                                  reinterpret_cast<ulonglong2 *>(base + L.front[1])};
        unsigned long long *d_cnts[2] = {
            reinterpret_cast<unsigned long long *>(base + L.cnts[0]),
            reinterpret_cast<unsigned long long *>(base + L.cnts[1])};
        void *d_table = base + L.table;
        const size_t slot = k64 ? 16 : 32;

        // Every call shares the scratch and finds the previous call's
        // contents there: clear what must start at zero.
        cuda_check(cudaMemcpyAsync(d_desc, &d, sizeof(d), cudaMemcpyHostToDevice, s), "upload");
        if (!lib.plc.empty())
            cuda_check(cudaMemcpyAsync(d_plc, lib.plc.data(), lib.plc.size() * sizeof(Plc),
                                       cudaMemcpyHostToDevice, s),
                       "upload");
        if (!lib.filters.empty())
            cuda_check(cudaMemcpyAsync(d_filt, lib.filters.data(),
                                       lib.filters.size() * sizeof(unsigned long long),
                                       cudaMemcpyHostToDevice, s),
                       "upload");
        cuda_check(cudaMemsetAsync(base + L.misc, 0, 256, s), "memset");
        cuda_check(cudaMemsetAsync(d_table, 0, L.cap_slots * slot, s), "memset");
        const unsigned long long tag = kMarker;   // instance 0
        ulonglong2 root;
        if (k64)
            root = make_ulonglong2((w0 & ((1ull << lib.dyn_bits) - 1ull)) | tag, 1ull);
        else
            root = make_ulonglong2(w0, tag);
        const unsigned long long one = 1ull;
        cuda_check(cudaMemcpyAsync(d_front[0], &root, sizeof(root), cudaMemcpyHostToDevice, s),
                   "upload");
        if (!k64)
            cuda_check(cudaMemcpyAsync(d_cnts[0], &one, sizeof(one), cudaMemcpyHostToDevice, s),
                       "upload");

        int sms = 0, occ = 0;
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
        cuda_check(expand_max_blocks_per_sm(k64, &occ), "occupancy");
        occ = std::max(occ, 1);
        const uint64_t slots = (uint64_t)sms * (uint64_t)occ;
        uint32_t fan_max = 1;
        for (int c = 0; c < kMaxWidth; c++)
            fan_max = std::max<uint32_t>(fan_max, lib.col_len[c]);
        const uint32_t dyn_rows = lib.dyn_bits / W;

        uint64_t n = 1, total_states = 0;
        int cur = 0;
        unsigned long long result = 0;
        for (uint32_t row = 0; row < H && n; row++) {
            const uint32_t R = d.win_rows;
            Seg sg{};
            sg.inst = 0;
            sg.row = row;
            const uint32_t src = row + R;
            sg.in_shift = (unsigned long long)(src < H ? inst->rows[src] : 0u) << ((R - 1) * W);
            unsigned long long hi = 0;
            for (uint32_t i = dyn_rows; i < R; i++)
                if (row + i < H)
                    hi |= (unsigned long long)inst->rows[row + i] << (i * W);
            sg.hi_board = hi;
            sg.tag = tag;
            sg.tbase = 0;
            sg.tcap = L.cap_slots;
            const uint32_t fan = n * 4 < slots * 256 && fan_max > 1 ? fan_max : 0;
            const bool fan2 = fan && n * fan * 4 < slots * 256;
            const uint64_t items = n * (fan ? (fan2 ? (uint64_t)fan * fan : fan) : 1);
            const uint64_t warps = slots * 8;
            uint64_t chunk = (items + 8 * warps - 1) / (8 * warps);
            chunk = std::min<uint64_t>(std::max<uint64_t>((chunk + 31) / 32 * 32, 32), 1024);
            sg.rec = 0;
            sg.begin = 0;
            sg.len = items;
            sg.chunk_base = 0;
            sg.fan = fan;
            sg.levels = fan ? (fan2 ? 2u : 1u) : 0u;
            const uint64_t n_chunks = (items + chunk - 1) / chunk;
            cuda_check(cudaMemcpyAsync(d_seg, &sg, sizeof(sg), cudaMemcpyHostToDevice, s),
                       "upload");
            cuda_check(cudaMemsetAsync(base + L.misc, 0, 64 + 16, s), "memset");

            ExpandArgs a{};
            a.segs = d_seg;
            a.n_segs = 1;
            a.n_chunks = n_chunks;
            a.chunk_states = chunk;
            a.insts = d_desc;
            a.plc = d_plc;
            a.filt = d_filt;
            a.recs = d_front[cur];
            a.cnts = d_cnts[cur];
            a.table = d_table;
            a.cap = L.cap_slots;
            a.inst_unique = d_unique;
            a.n_raw = d_raw;
            a.status = d_status;
            a.work = d_work;
            a.max_probe = 512;
            launch_expand(k64, a, (int)std::min<uint64_t>(n_chunks, slots), s);
            cuda_check(cudaGetLastError(), "k_expand launch");
            unsigned int h[2] = {0, 0};
            cuda_check(cudaMemcpyAsync(h, d_status, sizeof(h), cudaMemcpyDeviceToHost, s), "read");
            cuda_check(cudaStreamSynchronize(s), "k_expand");
            const uint64_t uniq = h[1];
            if ((h[0] & kStatusTableOverflow) || uniq > L.cap_states) {
                cuda_check(cudaMemsetAsync(d_table, 0, L.cap_slots * slot, s), "memset");
                cuda_check(cudaStreamSynchronize(s), "memset");
                return abi_fail(D4E_ERR_UNSUPPORTED,
                                "a row has more than " + std::to_string(L.cap_states) +
                                    " states: beyond the no-alloc scratch capacity");
            }
            const bool last = row + 1 == H;
            const unsigned long long cursor0 = last ? kCursorFinal : 0ull;
            cuda_check(cudaMemcpyAsync(d_cursor, &cursor0, sizeof(cursor0), cudaMemcpyHostToDevice,
                                       s),
                       "upload");
            CompactArgs c{};
            c.table = d_table;
            c.cap = L.cap_slots;
            c.cursor = d_cursor;
            c.out_recs = d_front[1 - cur];
            c.out_cnts = d_cnts[1 - cur];
            c.results = d_result;
            c.final_states = d_final;
            c.inst_off = lib.dyn_bits + lib.used_bits;
            c.inst_mask = 0;
            c.status = d_status;
            launch_compact(k64, c, compact_grid(L.cap_slots, sms), s);
            cuda_check(cudaGetLastError(), "k_compact launch");
            if (last) {
                cuda_check(cudaMemcpyAsync(&result, d_result, sizeof(result),
                                           cudaMemcpyDeviceToHost, s),
                           "read result");
            }
            unsigned int c_status = 0;
            cuda_check(cudaMemcpyAsync(&c_status, d_status, sizeof(c_status),
                                       cudaMemcpyDeviceToHost, s),
                       "read status");
            cuda_check(cudaStreamSynchronize(s), "k_compact");
            if (c_status & kStatusCompactStall)
                return abi_fail(D4E_ERR_CUDA, "k_compact: a staged table tile did not arrive");
            total_states += uniq;
            n = uniq;
            cur = 1 - cur;
        }
        *count = result;   // stays 0 when a row left no state
        if (states)
            *states = total_states;
        return D4E_OK;
    });
}
