// kernels.h -- launch wrappers for the sm_103a kernels of the tiling engine.
//
// Frontier records are passed as ulonglong2 arrays in both key encodings:
// K64 records are {key, count}; K128 records are {window, tag} keys with the
// counts in a separate u64 array.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "d4e_types.h"

namespace d4e {

struct ExpandArgs {
    const Seg *segs;
    uint32_t n_segs;
    uint64_t n_chunks;
    uint64_t chunk_states;           // work items per chunk (a segment's split: Seg::levels)
    const InstDesc *insts;
    const Plc *plc;
    const unsigned long long *filt;  // candidate filter bitsets (InstDesc::filt_off)
    const ulonglong2 *recs;          // frontier (K64 records / K128 keys)
    const unsigned long long *cnts;  // K128 counts
    void *table;                     // Slot16[cap] (K64) or Slot32[cap] (K128)
    unsigned long long cap;          // table slots (any value >= 1)
    unsigned int *inst_unique;       // per instance: new keys claimed
    unsigned long long *n_raw;       // children produced (all instances)
    unsigned int *status;
    unsigned long long *work;        // dynamic chunk counter, zeroed before the row's first launch
    // parts > 0 (launches that are never preempted): the chunk range is cut
    // into `parts` contiguous partitions, each with its own counter in
    // part_ctr (zeroed before the launch); a warp claims from its SM's
    // partition first and from the next ones when it runs dry, so that an
    // SM's warps walk few instances at a time.
    uint32_t parts;
    unsigned long long part_step;    // chunks per partition (the last one may hold fewer)
    unsigned long long *part_ctr;
    // Cooperative preemption (nullptr = none): while *preempt is nonzero
    // (host memory mapped into the device), warps take no new chunk, finish
    // the items they hold and exit.  The launch then ends with *work <
    // n_chunks; launching again with the same arguments (counters kept)
    // processes the chunks not yet taken.
    const unsigned int *preempt;
    unsigned int max_probe;
    uint32_t prefetch;               // request each child's table line into L2 when staged
    // Single-instance launches (one segment): the instance's n_plc
    // placements (0 = not staged) and its descriptor are copied into shared
    // memory at block start (expand_stage_bytes(stage_plc) dynamic bytes).
    uint32_t stage_plc;
    uint32_t u32;                    // K64: every instance's copy counters fit 32 bits
    uint32_t single_word;            // every instance's candidate filters are one word each
                                     // (0, the default, is right for any launch)
    // Partitioned dedup (K64 only): children are appended to bucket
    // hi(hash(key) * n_bkt) instead of inserted into the table; bucket b
    // holds records [b * bkt_cap, b * bkt_cap + bkt_cnt[b]).
    uint32_t append;
    ulonglong2 *bkt_recs;
    unsigned int *bkt_cnt;
    unsigned long long n_bkt, bkt_cap;
};

// De-duplicates every bucket in an on-chip table (counts summed, witnesses
// maxed), adds each bucket's new keys to inst_unique, and writes the
// bucket's table of kBucketSlots slots to dtab[b * kBucketSlots ...]
// (empty slots zero), which k_compact then turns into the next frontier.
struct MergeArgs {
    const ulonglong2 *bkt_recs;
    const unsigned int *bkt_cnt;
    unsigned long long n_bkt, bkt_cap;
    Slot16 *dtab;
    const InstDesc *insts;
    uint32_t inst_off;
    unsigned long long inst_mask;
    unsigned int *inst_unique;
    unsigned int *status;
};
void launch_bucket_merge(const MergeArgs &m, int grid, cudaStream_t s);
cudaError_t bucket_merge_prepare();   // opts the kernel into its shared memory

struct CompactArgs {
    void *table;
    unsigned long long cap;
    unsigned long long *cursor;      // per instance: next output position, or kCursorFinal
    ulonglong2 *out_recs;
    unsigned long long *out_cnts;    // K128 counts
    unsigned long long *results;     // per instance: summed counts of final states
    unsigned int *final_states;      // per instance: number of final states
    uint32_t inst_off;               // K64: position of the instance id in a key
    unsigned long long inst_mask;    // K64: instance id mask (after shifting)
    // Per instance: keep a state only if its sample hash is <= keep_max
    // (~0 = keep all).  nullptr = no sampling.
    const unsigned long long *keep_max;
    unsigned int *status;            // kStatusCompactStall is or'ed in here
    uint32_t stages;                 // shared-memory ring depth (32 KB tiles), 2..6; 0 = default
};

// Default k_compact plan: two blocks per SM, three 32 KB stages each.
constexpr int kCompactDefaultCtas = 2;
constexpr uint32_t kCompactDefaultStages = 3;
// Plans the kernel accepts (blocks per SM x stages x 32 KB within the SM's
// shared memory).
bool compact_plan_ok(int per_sm, uint32_t stages);

// Shared-memory bytes of a staged instance: its descriptor (rounded to 16)
// and n_plc 16-byte placements.
constexpr size_t kStageDescBytes = (sizeof(InstDesc) + 15) / 16 * 16;
constexpr size_t expand_stage_bytes(uint32_t n_plc) { return kStageDescBytes + 16ull * n_plc; }
// Largest staged instance (4 resident blocks per SM keep their ~18 KB of
// child staging plus this, and leave most of L1 to the candidate filters).
constexpr size_t kStageMaxBytes = 24 * 1024;

// Warps per k_expand block.
constexpr int kExpandWarps = 8;

// Resident k_expand blocks per SM (for sizing its persistent grid).
cudaError_t expand_max_blocks_per_sm(bool k64, int *n);

// Expand every state of every chunk by every whole-row fill and insert the
// children into the open-addressing table (counts summed).
void launch_expand(bool k64, const ExpandArgs &a, int grid, cudaStream_t s);

// Move the table's occupied slots into per-instance frontier segments (or into
// the per-instance results for instances finishing their last row) and clear
// the table.
void launch_compact(bool k64, const CompactArgs &a, int grid, cudaStream_t s);

// k_compact grid for a table of `cap` slots (32 KB tiles, `per_sm` blocks
// per SM, each streaming its tiles through a shared-memory ring).
int compact_grid(unsigned long long cap, int sms, int per_sm = kCompactDefaultCtas);

// Solution reconstruction -------------------------------------------------
struct KeySetArgs {
    void *table;
    unsigned long long cap;
    unsigned int *status;
    unsigned int max_probe;
};

// Insert the keys of n records into the (cleared) table as a membership set.
void launch_keyset_insert(bool k64, const KeySetArgs &t, const ulonglong2 *recs,
                          unsigned long long n, int grid, cudaStream_t s);

struct ProbeArgs {
    const InstDesc *insts;
    const Plc *plc;
    uint32_t inst;                  // single instance per launch
    uint32_t row;                   // row being completed
    unsigned long long in_shift;    // K128
    unsigned long long hi_board;    // K64
    unsigned long long tag;
    const void *table;              // membership set of the next level's live states
    unsigned long long cap;
    unsigned int max_probe;
};

// alive[i] = 1 when state i has at least one child in the set.
void launch_mark_alive(bool k64, const ProbeArgs &p, const ulonglong2 *recs,
                       unsigned long long n, unsigned char *alive, int grid, cudaStream_t s);

// For every node, emit one PathNode per (row fill, child in the set).
void launch_extend_paths(bool k64, const ProbeArgs &p, const PathNode *nodes, uint32_t n_nodes,
                         PathNode *out, unsigned int *n_out, uint32_t max_out,
                         unsigned int *status, int grid, cudaStream_t s);

// Keep records whose alive flag is set (order not preserved).
void launch_select(const ulonglong2 *recs, const unsigned char *alive, unsigned long long n,
                   ulonglong2 *out, unsigned long long *n_out, int grid, cudaStream_t s);

// Solution listing over many instances at once: one job per instance and
// level, each launch covering every job (blocks are dealt to jobs by
// blk_base; a block works on one job and loads that instance's placement
// table).  The membership set holds the live states of every job's next
// level together: keys carry their instance.
struct ListJob {
    const ulonglong2 *recs;         // the job's level records (keyset / mark passes)
    const PathNode *nodes;          // the job's partial tilings (extend pass)
    unsigned long long n;           // records or nodes
    unsigned long long out_off;     // the job's region of the output buffer
    unsigned long long out_cap;     // its size (extend pass: nodes kept)
    unsigned long long in_shift, hi_board, tag;   // probe fields of the job's row
    uint32_t inst, row;
    uint32_t blk_base;              // first block of the job (jobs in block order)
    uint32_t pad;
};

// Blocks for a job of n items (at least one, at most kListMaxBlocks).
constexpr uint32_t kListMaxBlocks = 64;
uint32_t list_blocks(unsigned long long n);

// Insert every job's records into the membership set.
void launch_keyset_insert_jobs(bool k64, const KeySetArgs &t, const ListJob *jobs,
                               uint32_t n_jobs, uint32_t blocks, cudaStream_t s);

// Every job's records with a child in the set, appended to out + out_off
// (n_out[job] counts them; order not preserved).  p: instance tables and
// the set (per-job fields are taken from the jobs).
void launch_mark_select_jobs(bool k64, const ProbeArgs &p, const ListJob *jobs, uint32_t n_jobs,
                             uint32_t blocks, ulonglong2 *out, unsigned long long *n_out,
                             cudaStream_t s);

// For every job's nodes, one PathNode per (row fill, child in the set), at
// out + out_off + position (n_out[job] counts them; positions at or past
// out_cap are dropped and flag kStatusNodeOverflow).  parent = the node's
// index within its job.
void launch_extend_paths_jobs(bool k64, const ProbeArgs &p, const ListJob *jobs, uint32_t n_jobs,
                              uint32_t blocks, PathNode *out, unsigned int *n_out,
                              unsigned int *status, cudaStream_t s);

// *out += number of records with (rec.x & mask) == value.
void launch_count_pattern(const ulonglong2 *recs, unsigned long long n, unsigned long long mask,
                          unsigned long long value, unsigned long long *out, int grid,
                          cudaStream_t s);

}  // namespace d4e

namespace d4e {

// Solve-one ----------------------------------------------------------------
// A kept level of one solve-one instance.
struct LevelPtr {
    const ulonglong2 *recs;          // K64 {key, witness} records / K128 keys
    const unsigned long long *cnts;  // K128 witnesses
    unsigned long long len;
};

struct TraceJob {
    uint32_t inst;
    uint32_t height;
    uint32_t lvl;                    // first of height + 1 LevelPtr entries (level 0 = root)
    uint32_t pad;
    unsigned long long tag;          // the instance's key tag
};

struct TraceOut {
    uint32_t status;                 // 0 = traced; 1 = a witness had no parent; 2 = no fill
    uint8_t nfill[kMaxHeight];       // placements completing each row
    uint16_t plc[kMaxHeight][kMaxWidth];   // instance-relative placement indices
};

// Chosen record per kept level of a job, and the witness it carries.
struct TraceChain {
    unsigned long long idx[kMaxHeight + 1];   // chosen record + 1 (0 = none found)
    unsigned long long tgt[kMaxHeight + 1];   // witness of the chosen record
    unsigned long long best;                  // largest final-state identity
};

// Records of one job's level in a flattened pass over many jobs.
struct TraceSeg {
    uint32_t job;
    uint32_t level;                  // level index r of the job
    unsigned long long base;         // first flattened index
    unsigned long long len;
};

// Tracing runs in passes over the kept levels of all jobs at once:
//   final pass A : best[job] = largest identity among the final states;
//   final pass B : the final state with that identity is chosen;
//   level passes : from the final level down, the record of level r whose
//                  identity equals the witness chosen at level r + 1 (a
//                  unique state) is chosen;
//   fill         : per job and row, the first fill (depth-first order)
//                  leading from the chosen parent to the chosen child.
// `segs` covers the records of one pass (sorted by base, n_segs entries,
// `total` records).
void launch_trace_pass(bool k64, int pass, const LevelPtr *levels, const TraceJob *jobs,
                       const TraceSeg *segs, uint32_t n_segs, unsigned long long total,
                       TraceChain *chain, int grid, cudaStream_t s);
// Per job and row, the first fill (depth-first order) leading from the
// chosen parent to the chosen child; one warp per job, one lane per row.
void launch_trace_fill(bool k64, const InstDesc *insts, const Plc *plc, const LevelPtr *levels,
                       const TraceJob *jobs, uint32_t n_jobs, const TraceChain *chain,
                       TraceOut *out, int grid, cudaStream_t s);

// Copies record ranges (and K128 counts when cnts are given) between
// frontier buffers: one warp per range.
struct CopyRange {
    unsigned long long src, dst, len;
};
void launch_copy_ranges(const ulonglong2 *src, const unsigned long long *src_cnts, ulonglong2 *dst,
                        unsigned long long *dst_cnts, const CopyRange *ranges, uint32_t n,
                        int grid, cudaStream_t s);

}  // namespace d4e
