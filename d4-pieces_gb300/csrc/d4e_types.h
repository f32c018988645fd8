// d4e_types.h -- data layouts shared by the host runtime and the sm_103a kernels.
//
// Frontier state (one per distinct partial tiling class at a row boundary):
//   key.x = window : 64-bit row-aligned occupancy window.  Bit (i*W + c) set
//                    means cell (row+i, c) still has to be covered, for the
//                    R = 64 / W board rows starting at the current row.
//   key.y = tag    : bits 0..39   used piece copies (copies of one type take a
//                                 contiguous bit range and are used
//                                 lowest-free-first, so the mask is the
//                                 per-type used-count vector),
//                    bits 40..62  instance id,
//                    bit  63      marker (a valid key is never all-zero).
//   count          : number of partial tilings reaching this state (u64).
// Keys and counts are stored structure-of-arrays: keys as 16-byte
// ulonglong2 (128-bit coalesced loads/stores), counts as u64.
//
// This replaces the reference's 20/24-byte R/RX records (src/record.h:5-32),
// whose packing of <= 16 used piece names and an 8-row window is exact only
// for boards of at most 8 rows and tracks piece *sets* without multiplicity.
#pragma once

#include <cstdint>

namespace d4e {

constexpr int kMaxWidth = 8;          // 8-wide boards, as the reference's frow tables
constexpr int kMaxHeight = 64;        // rows per board
constexpr int kMaxCopies = 40;        // piece copies per instance (bits 0..39 of the tag)
constexpr int kInstShift = 40;        // instance id position in the tag
constexpr uint32_t kMaxInstances = 1u << 23;
constexpr int kMaxPlcPerCol = 255;    // placements anchored at one column (8-bit DFS stack)
constexpr int kMaxPlc = kMaxWidth * kMaxPlcPerCol;
constexpr uint64_t kMarker = 1ull << 63;
constexpr uint64_t kUsedMask = (1ull << kInstShift) - 1;

// One placement anchored at a column of the current row: `mask` holds its
// cells in window coordinates (bit i*W + c), `tm` the copy bits of its type.
struct Plc {
    uint64_t mask;
    uint64_t tm;
};

// Per-instance constants, resident in device memory.
struct InstDesc {
    uint32_t width;
    uint32_t height;
    uint32_t win_rows;    // R = 64 / width
    uint32_t n_plc;
    uint32_t plc_off;     // first placement in the global placement array
    uint32_t pad0;
    uint16_t col_off[kMaxWidth];   // placements anchored at column c: [col_off, col_off + col_len)
    uint16_t col_len[kMaxWidth];
    uint8_t rows[kMaxHeight];      // board rows, bit c = cell to cover
};

// The frontier segment of one active instance.  It is cut into work chunks
// of `chunk_states` states; chunk_base is the global index of its first chunk.
struct Seg {
    uint32_t inst;
    uint32_t row;         // row being completed
    uint64_t begin;
    uint64_t len;
    uint64_t in_shift;    // board row (row + R) placed in window row R-1 after the shift
    uint64_t chunk_base;
};

// Open-addressing hash table slot (32 bytes = one DRAM sector).  An all-zero
// key is empty; valid keys always carry the marker bit.
struct alignas(32) Slot {
    unsigned long long k0;
    unsigned long long k1;
    unsigned long long cnt;
    unsigned long long pad;
};

// Device status word bits.
enum : uint32_t {
    kStatusTableOverflow = 1u,    // probe limit reached: table too small, level is redone
    kStatusNodeOverflow = 2u,     // solution path buffer full
};

// Cursor value marking an instance whose row being completed is its last:
// its states are summed into the per-instance result instead of stored.
constexpr unsigned long long kCursorFinal = ~0ull;

// Solution path node (one completed row of one partial tiling).
struct PathNode {
    unsigned long long k0, k1;   // state after the row
    uint32_t parent;             // node index in the previous row's list (~0u at row 0)
    uint32_t nfill;              // placements used to complete the row
    uint16_t plc[kMaxWidth];     // placement index (instance-relative) per fill step
};

}  // namespace d4e
