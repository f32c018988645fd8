// kernels.h -- launch wrappers for the sm_103a kernels of the tiling engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "d4e_types.h"

namespace d4e {

struct ExpandArgs {
    const Seg *segs;
    uint32_t n_segs;
    uint64_t n_chunks;
    uint64_t chunk_states;
    const InstDesc *insts;
    const Plc *plc;
    const ulonglong2 *keys;
    const unsigned long long *cnts;
    Slot *table;
    unsigned long long cap;         // table slots (any value >= 1)
    unsigned int *inst_unique;      // per instance: new keys claimed
    unsigned long long *n_raw;      // children produced (all instances)
    unsigned int *status;
    unsigned long long *work;       // dynamic chunk counter, zeroed before launch
    unsigned int max_probe;
};

struct CompactArgs {
    Slot *table;
    unsigned long long cap;
    unsigned long long *cursor;     // per instance: next output position, or kCursorFinal
    ulonglong2 *out_keys;
    unsigned long long *out_cnts;
    unsigned long long *results;    // per instance: summed counts of final states
    unsigned int *final_states;     // per instance: number of final states
};

// Resident k_expand blocks per SM (for sizing its persistent grid).
cudaError_t expand_max_blocks_per_sm(int *n);

// Expand every state of every chunk by every whole-row fill and insert the
// children into the open-addressing table (counts summed).
void launch_expand(const ExpandArgs &a, int grid, cudaStream_t s);

// Move the table's occupied slots into per-instance frontier segments (or into
// the per-instance results for instances finishing their last row) and clear
// the table.
void launch_compact(const CompactArgs &a, int grid, cudaStream_t s);

// Solution reconstruction -------------------------------------------------
struct KeySetArgs {
    Slot *table;
    unsigned long long cap;
    unsigned int *status;
    unsigned int max_probe;
};

// Insert n keys into the (cleared) table as a membership set.
void launch_keyset_insert(const KeySetArgs &t, const ulonglong2 *keys, unsigned long long n,
                          int grid, cudaStream_t s);

struct ProbeArgs {
    const InstDesc *insts;
    const Plc *plc;
    uint32_t inst;                  // single instance per launch
    uint32_t row;                   // row being completed
    unsigned long long in_shift;
    const Slot *table;              // membership set of the next level's live states
    unsigned long long cap;
    unsigned int max_probe;
};

// alive[i] = 1 when state i has at least one child in the set.
void launch_mark_alive(const ProbeArgs &p, const ulonglong2 *keys, unsigned long long n,
                       unsigned char *alive, int grid, cudaStream_t s);

// For every node, emit one PathNode per (row fill, child in the set).
void launch_extend_paths(const ProbeArgs &p, const PathNode *nodes, uint32_t n_nodes,
                         PathNode *out, unsigned int *n_out, uint32_t max_out,
                         unsigned int *status, int grid, cudaStream_t s);

// Keep keys whose alive flag is set (order preserved).
void launch_select(const ulonglong2 *keys, const unsigned char *alive, unsigned long long n,
                   ulonglong2 *out, unsigned long long *n_out, int grid, cudaStream_t s);

// *out += number of keys with (key.x & mask) == value.
void launch_count_pattern(const ulonglong2 *keys, unsigned long long n, unsigned long long mask,
                          unsigned long long value, unsigned long long *out, int grid,
                          cudaStream_t s);

}  // namespace d4e
