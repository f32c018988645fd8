// d4e_types.h -- data layouts shared by the host runtime and the sm_103a kernels.
//
// A frontier state is (row window, used piece copies) plus the number of
// partial tilings reaching it.
//   window : bit i*W + c set = cell (row+i, c) still has to be covered, for
//            the R = 64 / W board rows starting at the current row.
//   used   : per piece type a binary counter of copies placed, in a bit
//            field of bit_length(count) bits (fields packed from bit 0;
//            <= 40 bits in all).
// Two encodings of the key, chosen per engine:
//   K64  (packed, used whenever it fits): key = the window's first
//        W*(max piece rows - 1) bits (the only rows earlier placements can
//        reach; deeper rows are the board's) | used << those bits |
//        instance id << inst_off | marker bit 63.  Record = {key, count},
//        16 bytes; table slot 16 bytes; 64-bit CAS.
//   K128 (general): key.x = full 64-bit window, key.y = used (bits 0..39) |
//        instance id (bits 40..62) | marker (bit 63).  Record = 16-byte key +
//        8-byte count; table slot 32 bytes; 128-bit CAS.
// The marker bit makes every valid key non-zero, so a zeroed table is empty.
//
// This replaces the reference's 20/24-byte R/RX records (src/record.h:5-32),
// whose packing of <= 16 used piece names and an 8-row window is exact only
// for boards of at most 8 rows and tracks piece *sets* without multiplicity.
#pragma once

#include <cstdint>

namespace d4e {

constexpr int kMaxWidth = 8;          // 8-wide boards, as the reference's frow tables
constexpr int kMaxHeight = 64;        // rows per board
constexpr int kMaxUsedBits = 40;      // bits of all per-type copy counters together
constexpr int kMaxTypes = kMaxUsedBits;
constexpr int kInstShift128 = 40;     // instance id position in a K128 key's second word
constexpr uint32_t kMaxInstances = 1u << 23;
constexpr int kMaxPlcPerCol = 255;    // placements anchored at one column (8-bit DFS stack)
constexpr int kMaxPlc = kMaxWidth * kMaxPlcPerCol;
constexpr uint64_t kMarker = 1ull << 63;
constexpr uint64_t kUsedMask128 = (1ull << kInstShift128) - 1;

// One placement anchored at a column of the current row: its cells in window
// coordinates (bit i*W + c), its piece type, and that type's copy counter
// (bits off .. off + bits - 1 of `used`; a copy is free while the field is
// below count, and taking one adds 1 << off), so that the walk tests and
// takes a copy without another load.
struct Plc {
    uint64_t mask;
    uint8_t type;
    uint8_t next_type;    // column-relative index of the first placement of the next type
    uint8_t off;
    uint8_t bits;
    uint32_t count;
};
static_assert(sizeof(Plc) == 16, "placement record");

// Copy counter of one piece type: field mask and capacity (count << offset),
// both in `used` coordinates.  A copy is available when (used & fm) < cap;
// taking it adds the field's lowest bit.
struct TypeField {
    uint64_t fm;
    uint64_t cap;
};

// Per-instance constants, resident in device memory.
struct InstDesc {
    uint32_t width;
    uint32_t height;
    uint32_t win_rows;    // R = 64 / width
    uint32_t n_plc;
    uint32_t plc_off;     // first placement in the global placement array
    uint32_t n_types;
    uint32_t dyn_bits;    // width * (max piece rows - 1): window bits a K64 key keeps
    uint32_t used_bits;
    uint32_t flags;       // kInstWitness: records carry a parent witness, not a count
    uint32_t limit;       // distinct children per row beyond which the instance fails
                          // (0 = none): k_expand stops expanding it once passed
    uint16_t col_off[kMaxWidth];   // placements anchored at column c: [col_off, col_off + col_len)
    uint16_t col_len[kMaxWidth];
    // Candidate filters (bitsets over a column's placements, `fwords` u64
    // words each, in the global filter array from filt_off on):
    //   row-0 filter of column c, pattern p = current row >> (c + 1):
    //     placements whose row-0 cells fit  -> filt_off + f0_off[c] + p * fwords
    //   row-1 filter of column c, pattern q = next row:
    //     placements whose row-1 cells fit  -> filt_off + f1_off[c] + q * fwords
    uint32_t filt_off;
    uint32_t fwords;
    uint32_t f0_off[kMaxWidth];
    uint32_t f1_off[kMaxWidth];
    uint32_t f2_off[kMaxWidth];   // row-2 filter of column c, pattern = window row 2
    TypeField types[kMaxTypes];
    uint8_t rows[kMaxHeight];      // board rows, bit c = cell to cover
};

// InstDesc::flags.  A solve-one instance's records carry, instead of a
// count, the largest witness (instance-free key, see witness64/witness128 in
// kernels.cu) of the parents that produce them, so that one tiling can be
// traced back through its kept levels.
constexpr uint32_t kInstWitness = 1u;

// The frontier segment of one active instance.  It is cut into work chunks
// of `chunk_states` states; chunk_base is the global index of its first chunk.
struct Seg {
    uint32_t inst;
    uint32_t row;                 // row being completed
    uint64_t begin;               // first work item (items of all segments are consecutive)
    uint64_t len;                 // work items: states x items per state
    uint64_t chunk_base;
    uint64_t rec;                 // the segment's first frontier record
    // Work items per state: 1 (levels 0), or the state's walk cut by its
    // first placement (levels 1: fan items) or first two (levels 2: fan^2).
    uint32_t fan, levels;
    unsigned long long in_shift;  // K128: board row (row + R) entering window row R-1
    unsigned long long hi_board;  // K64: board rows [row + dyn_rows, row + R) in window coordinates
    unsigned long long tag;       // instance id bits | marker, in the mode's key coordinates
    unsigned long long tbase;     // the instance's hash-table region: slots [tbase, tbase + tcap)
    unsigned long long tcap;
};

// Per-instance new-key counter bit: the instance's table region overflowed
// (its row is redone with a larger region; k_expand stops expanding it).
constexpr uint32_t kUniqueOverflow = 0x80000000u;

// Table regions are whole compaction tiles (2048 slots), so every tile k_compact
// reads belongs to one instance.
constexpr unsigned long long kRegionAlign = 2048;

// Hash table slots.  A zero key is empty.
struct alignas(32) Slot32 {
    unsigned long long k0;
    unsigned long long k1;
    unsigned long long cnt;
    unsigned long long pad;
};
struct alignas(16) Slot16 {
    unsigned long long key;
    unsigned long long cnt;
};

// Device status word bits.
enum : uint32_t {
    kStatusTableOverflow = 1u,    // probe limit reached: table too small, level is redone
    kStatusNodeOverflow = 2u,     // solution path buffer full
    kStatusBucketOverflow = 4u,   // partitioned dedup: a bucket or its on-chip table was full
    kStatusCompactStall = 8u,     // k_compact: a staged tile did not arrive in time (launch ended)
};

// Partitioned dedup: on-chip table slots per bucket (k_bucket_merge) and the
// distinct states a bucket is sized for.
constexpr unsigned kBucketSlots = 4096;
constexpr unsigned kBucketTarget = 1536;

// Cursor value marking an instance whose row being completed is its last:
// its states are summed into the per-instance result instead of stored.
constexpr unsigned long long kCursorFinal = ~0ull;
// Cursor value of an instance whose children are discarded (it failed).
constexpr unsigned long long kCursorDrop = ~0ull - 1ull;

// Solution path node (one completed row of one partial tiling).
struct PathNode {
    unsigned long long k0, k1;   // state after the row (K64: k1 = 0)
    uint32_t parent;             // node index in the previous row's list
    uint32_t nfill;              // placements used to complete the row
    uint16_t plc[kMaxWidth];     // placement index (instance-relative) per fill step
};

}  // namespace d4e
