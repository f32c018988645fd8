// engine.h -- host runtime of the GB300 row-by-row polyomino tiling engine.
//
// One Engine drives any number of puzzle instances on one GPU.  Every
// active instance advances by one board row per step(); the union of their
// frontiers is expanded by one k_expand launch and compacted by one
// k_compact launch.  The plain single-puzzle path (CudaSearcher mirror) is an
// Engine holding one instance; the batched and serving paths add many.
//
// Replaces the reference's Device c/m threads, ring buffer and host Sorter
// (src/device.cu:14-309, src/sorter.cpp:72-214) with device-resident
// frontier segments and an HBM hash table; no child state crosses PCIe.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "d4e_types.h"
#include "geometry.h"
#include "kernels.h"

namespace d4e {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

enum ErrCode : int {
    kErrInvalid = -1,
    kErrCuda = -2,
    kErrNoMem = -3,
    kErrUnsupported = -4,
    kErrState = -5,
};

void cuda_check(cudaError_t e, const char *what);

// Stream-ordered allocation from the memory pool of the engine whose method
// is running on this thread (the device's default pool outside engines).
cudaError_t engine_malloc_async(void **p, size_t bytes, cudaStream_t s);

// Grow-only device buffer, allocated stream-ordered (engine_malloc_async /
// cudaFreeAsync on the owner's stream) so that growing it never
// synchronises the device: engines on other streams keep running.
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;
    cudaStream_t s = nullptr;   // stream of the last allocation
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p)
            cudaFreeAsync(p, s);
        p = nullptr;
        cap = 0;
    }
    // Ensures capacity >= n elements; keeps the first `keep` elements.
    void reserve(size_t n, cudaStream_t s, size_t keep = 0);
};

// Forgets the process-wide cache of measured launch plans.
void autotune_clear();

// Device bytes an allocation can still get: free memory plus what the
// device's stream-ordered pools hold in reserve.
size_t device_available_bytes(int device, size_t *total);
// Destroys the idle engine pools (the device memory they keep for the next
// engine goes back to the driver).
void release_idle_pools();

enum class KeyMode { Auto, K64, K128 };

struct EngineOpts {
    int device = 0;
    uint32_t max_probe = 512;
    bool keep_levels = false;      // retain every level (needed for solutions; one instance)
    double target_load = 0.5;      // hash table load factor aimed at when sizing
    uint64_t chunk_states = 1024;  // largest number of work items a warp takes at once
    uint64_t max_frontier = 0;     // abort when a row yields more states (0 = no limit)
    KeyMode key_mode = KeyMode::Auto;  // Auto: K64 when every instance's packed key fits
    // Device bytes the frontiers and the hash table may hold together
    // (0 = the whole device less 10%).
    uint64_t memory_budget = 0;
    // A failing instance (its frontier limit, or a row that cannot fit the
    // device alone) ends with an error status instead of failing step().
    bool isolate_failures = false;
    // K64 layout fixed at construction with this many instance-id bits
    // (0 = layout chosen from the instances, see fix_key_mode).  Instances
    // whose window + counter bits exceed 63 - k64_inst_bits are rejected.
    uint32_t k64_inst_bits = 0;
    // k_expand CTAs per SM (0 = as many as fit).  A lower value leaves room
    // on every SM for kernels of another engine running concurrently.
    int expand_ctas_per_sm = 0;
    bool high_priority = false;    // create the engine's stream at the highest priority
    // Cooperative preemption of k_expand (ExpandArgs::preempt): the device
    // address of a flag in mapped host memory, and a gate that step() calls
    // before each k_expand launch of a row with whether the row's previous
    // launch was preempted (false before its first).  The gate may wait; it
    // returns whether this launch honours the flag.  A preempted launch is
    // launched again until every chunk of the row is taken.
    const unsigned int *preempt_flag = nullptr;
    std::function<bool(bool)> preempt_gate;
    // Chunks per resident warp aimed at by the launch plan (0 = the default
    // plan).  More, smaller chunks let a preempted launch end sooner.
    uint32_t chunks_per_warp = 0;
    // Placements fixed per work item when a frontier is too small to fill
    // the GPU (1 or 2; see the launch plan).  Two levels fill the whole GPU
    // from a handful of states, which an engine sharing the GPU with a
    // latency-critical one should not do.
    uint32_t max_split_levels = 2;
    // Measure launch plans on the first row of 2^21..2^25 states and keep
    // the fastest (cached per key encoding, board width and device).
    bool autotune = false;
    // De-duplication of a row's children: Direct (Auto) inserts them into
    // the hash table as they are produced; Partitioned appends them into
    // hash buckets and merges each bucket on chip (packed keys, after the
    // first row; a bucket overflow redoes the row directly).  Measured on
    // the 8x15 enumeration, appending did not shorten k_expand (56 ms per
    // launch either way: the walk, not the insert, bounds it) and the merge
    // added ~200 ms, so Auto stays direct.
    enum class Dedup { Auto, Direct, Partitioned } dedup = Dedup::Auto;
};

// Launch plan of k_expand / k_compact and the table's load factor.
struct Tuning {
    bool set = false;                // measured (or taken from the cache)
    uint64_t chunk_cap = 1024;       // most work items a warp takes at once
    uint32_t chunks_per_warp = 8;    // chunks per resident warp aimed at
    int ctas_per_sm = 0;             // k_expand CTAs per SM (0 = occupancy)
    double load = 0.5;               // hash table load factor aimed at
    int compact_ctas = 2;            // k_compact blocks per SM
    uint32_t compact_stages = 3;     // k_compact shared-memory ring depth (32 KB tiles)
};

// Count: tilings.  SolveOne: one tiling.  Sets: the piece multisets that
// tile the board (the final row's used-copy counters), each with its number
// of tilings.
// List: the tilings themselves -- counting with every row's frontier kept
// per instance, from which solutions() lists them.
enum class Mode : uint32_t { Count = 0, SolveOne = 1, Sets = 2, List = 3 };

// One piece multiset of a Sets instance: copies per input piece type.
// Piece multisets of a Sets-mode instance: set k uses copies[k * n_types + t]
// copies of piece type t and has tilings[k] tilings; sets are in
// lexicographic order of their copies.
struct PieceSets {
    uint32_t n_types = 0;
    std::vector<uint8_t> copies;
    std::vector<uint64_t> tilings;
    size_t size() const { return tilings.size(); }
};

struct InstanceSpec {
    uint32_t width = 8;
    uint32_t height = 8;
    const uint8_t *rows = nullptr;       // height entries, bit c = cell (r, c) to cover
    const uint64_t *shapes = nullptr;    // Shape<8> layout
    const uint32_t *counts = nullptr;
    uint32_t n_pieces = 0;
    uint32_t sym = 0xFFu;
    Mode mode = Mode::Count;
    uint64_t max_states = 0;             // per-row frontier limit (0 = none)
    uint64_t beam = 0;                   // solve-one: first sampled-frontier width (0 = exact)
};

struct StepStats {
    uint64_t n_in = 0, n_raw = 0, n_out = 0;
    float expand_ms = 0.f, compact_ms = 0.f;
    uint32_t retries = 0;
    uint32_t paused = 0;          // instances that waited for memory this row
    uint32_t groups = 0;          // k_expand groups (after splits)
    uint32_t failed = 0;          // instances that ended with an error this row
    uint64_t table_cap = 0;
};

struct Totals {
    uint64_t steps = 0;
    uint64_t states_in = 0, states_raw = 0, states_out = 0;
    double expand_ms = 0.0, compact_ms = 0.0;
    uint64_t expand_launches = 0, compact_launches = 0, other_launches = 0, retries = 0;
    uint64_t paused = 0, splits = 0, failed = 0, restarts = 0;
    uint64_t preemptions = 0;      // k_expand launches ended early by preemption
    uint64_t peak_frontier = 0;
    uint64_t h2d_bytes = 0, d2h_bytes = 0;
    double run_ms = 0.0;           // CUDA-event time from the first step to the last
    // Host wall time inside step(), and the parts spent uploading new
    // instances, keeping solve-one levels and tracing solve-one tilings
    // (each including the device work it waits for).
    double step_wall_ms = 0.0, upload_ms = 0.0, keep_ms = 0.0, trace_ms = 0.0;
    double tune_ms = 0.0;          // host wall time spent in autotuning trials
    // Host wall time of step() phases: selecting / grouping instances,
    // preparing tables (layout, allocation, clears), waiting for k_expand
    // (launch to read-back), per-group bookkeeping, waiting for k_compact,
    // and the row's tail (carries, levels, advancing instances).
    double ph_select_ms = 0.0, ph_table_ms = 0.0, ph_expand_ms = 0.0, ph_post_ms = 0.0,
           ph_compact_ms = 0.0, ph_tail_ms = 0.0;
    uint64_t compact_slots = 0;    // table slots scanned by k_compact (sum over launches)
    uint64_t partitioned = 0;      // groups de-duplicated through buckets
    uint64_t partition_fallbacks = 0;   // ... of which redone with the direct table
    double merge_ms = 0.0;         // device time of k_bucket_merge
};

// One kept frontier level of a solve-one instance: `len` records from
// `first` on in level chunk `chunk` (a device block shared by the instances
// kept in the same step).
struct LevelRef {
    uint32_t chunk;
    uint64_t first, len;
};

class Engine {
public:
    explicit Engine(const EngineOpts &opts);
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    // Adds an instance (validated); its tables are uploaded and its root
    // state joins the frontier at the next step().  Returns the instance id.
    uint32_t add(const InstanceSpec &spec);

    // Advances every active instance by one row.
    StepStats step();
    void run();
    bool has_active() const { return n_active_ > 0 || !pending_.empty(); }

    // Per-instance queries.
    uint32_t n_instances() const { return (uint32_t)inst_.size(); }
    bool done(uint32_t id) const { return inst_.at(id).done; }
    uint32_t row(uint32_t id) const { return inst_.at(id).row; }
    uint32_t height(uint32_t id) const { return inst_.at(id).height; }
    uint32_t width(uint32_t id) const { return inst_.at(id).width; }
    // Device bytes (frontier records + table slots) the instance's next row
    // is expected to need, and the most any of its rows needed so far.
    uint64_t projected_bytes(uint32_t id) const;
    uint64_t peak_bytes(uint32_t id) const;
    uint64_t frontier_size(uint32_t id) const { return inst_.at(id).seg_len; }
    uint64_t count(uint32_t id);                        // tilings (valid once done)
    int status(uint32_t id) const { return inst_.at(id).status; }   // 0 or an ErrCode
    const std::string &error(uint32_t id) const { return inst_.at(id).error; }
    // Solve-one result: true and the tiling (row-major type grid, step grid,
    // width * height cells each, -1 = not covered) when one exists.
    bool solution(uint32_t id, int8_t *type_grid, int16_t *step_grid);
    // Sets-mode result (valid once done).
    const PieceSets &sets(uint32_t id) const { return inst_.at(id).sets; }
    // Frees a finished instance's id for reuse by a later add().
    void release(uint32_t id);
    // A held instance sits out the following steps (its frontier carried
    // unchanged) while some active instance is not held.
    void set_hold(uint32_t id, bool hold) { inst_.at(id).held = hold; }
    bool held(uint32_t id) const { return inst_.at(id).held; }
    const std::vector<uint64_t> &level_sizes(uint32_t id) const { return inst_.at(id).level_sizes; }
    uint64_t next_size_estimate(uint32_t id) const;
    // States of the instance's frontier whose current row equals `pattern`.
    uint64_t bucket_count(uint32_t id, uint32_t pattern);
    // Pulls the counts of instances finished since the last call.
    void sync_results();

    // Solutions of a finished instance: the one instance of an engine
    // created with keep_levels, or a Mode::List instance.  Writes up to max
    // grids of width * height cells (piece types, placement numbers; -1 =
    // not covered); returns the number of tilings reconstructed (== the
    // count unless max truncated it).
    uint64_t solutions(uint32_t id, uint64_t max, int8_t *type_grids, int16_t *step_grids,
                       bool single);
    // Tilings of many finished Mode::List instances at once, at most max_per
    // each: the backward (live-state) and forward (path) passes cover every
    // instance per level, one launch per level and pass.  out[k] receives
    // ids[k]'s tilings (none for a failed instance or one without tilings).
    struct TilingList {
        uint64_t n = 0;                  // tilings written
        std::vector<int8_t> types;       // n grids of width * height cells
        std::vector<int16_t> steps;
    };
    void list_solutions(const std::vector<uint32_t> &ids, uint64_t max_per,
                        std::vector<TilingList> &out);

    const Totals &totals() const { return tot_; }
    const Tuning &tuning() const { return tune_; }
    void set_max_frontier(uint64_t n) { opts_.max_frontier = n; }
    bool packed_keys() const { return k64_; }
    cudaStream_t stream() const { return stream_; }
    int sm_count() const { return sms_; }

private:
    struct Inst {
        PieceLib lib;
        InstDesc desc{};
        uint32_t width = 0, height = 0;
        uint32_t row = 0;
        bool active = false, done = false, result_ready = false;
        bool held = false;
        uint64_t seg_begin = 0, seg_len = 0;
        uint64_t result = 0;
        std::vector<uint64_t> level_sizes;
        unsigned long long root_window = 0;
        double growth = 256.0;       // expected children per state on the next row
        uint64_t min_region = 0;     // table slots at least (after a region overflow)
        Mode mode = Mode::Count;
        uint64_t limit = 0;          // per-row frontier limit (0 = none)
        int status = 0;              // 0 or the ErrCode it failed with
        std::string error;
        // Solve-one: sampled-frontier width of the current attempt (0 =
        // exact), whether a row was sampled, and the kept levels.
        uint64_t beam = 0;
        bool sampled = false;
        std::vector<LevelRef> levels;
        bool found = false;
        PieceSets sets;   // Sets mode result
        std::vector<int8_t> tgrid;
        std::vector<int16_t> sgrid;
    };

    StepStats step_impl();
    void autotune(const std::vector<uint32_t> &grp, double est, int occ,
                  const std::function<uint64_t(const Tuning &)> &plan,
                  const std::vector<Seg> &segs, const uint64_t &chunk, const uint64_t &n_chunks,
                  const int &grid);
    void ensure_inst_capacity(size_t n);
    void fail_instance(uint32_t id, int code, const std::string &msg);
    // Solve-one support: kept levels, tracing, restarts with a wider sample.
    void keep_levels_of(const std::vector<uint32_t> &ids);
    void drop_levels(Inst &in);
    void trace_solutions(const std::vector<uint32_t> &ids);
    void finish_solve_one(uint32_t id, bool found);
    void total_lists(const std::vector<uint32_t> &ids);
    void restart(uint32_t id);
    uint64_t frontier_bytes(int buf) const;
    double memory_limit(double device_avail) const;
    void fix_key_mode();
    void flush_uploads();
    int expand_occupancy();
    uint32_t stage_plc(const std::vector<Seg> &segs) const;
    bool counters_fit_u32(const std::vector<Seg> &segs) const;
    bool multi_word_filters(const std::vector<Seg> &segs) const;
    uint64_t table_limit();
    size_t slot_units() const { return k64_ ? 1 : 2; }   // table slot size in 16-byte units
    Seg seg_for(uint32_t id, uint32_t row) const;
    ulonglong2 root_record(uint32_t id) const;

    EngineOpts opts_;
    int sms_ = 0;
    int occ64_ = 0, occ128_ = 0;   // resident k_expand CTAs per SM
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev_[4] = {};
    cudaEvent_t ev_run_[2] = {};

    // Key encoding, fixed at the first step.
    bool mode_fixed_ = false;
    bool k64_ = false;
    uint32_t inst_off_ = 0;           // K64: instance id position
    unsigned long long inst_mask_ = 0;

    std::vector<Inst> inst_;
    std::vector<uint32_t> pending_;          // roots not yet in the frontier
    std::vector<uint32_t> pending_upload_;   // descriptors/tables not yet on the device
    std::vector<uint32_t> active_;           // instances with a frontier segment
    std::vector<uint32_t> unfetched_;        // finished, result still on the device
    std::vector<uint32_t> free_ids_;         // released ids, reused by add()
    uint32_t n_active_ = 0;

    DevBuf<Plc> plc_;
    uint64_t plc_total_ = 0, plc_uploaded_ = 0;
    DevBuf<unsigned long long> filt_;
    DevBuf<unsigned long long> part_ctr_;   // k_expand partition counters (ExpandArgs::parts)
    uint64_t filt_total_ = 0, filt_uploaded_ = 0;
    DevBuf<InstDesc> insts_;
    DevBuf<unsigned int> inst_unique_;
    DevBuf<unsigned long long> cursor_;
    DevBuf<unsigned long long> results_;
    DevBuf<unsigned int> final_states_;
    DevBuf<unsigned int> misc_;   // [0] status
    DevBuf<unsigned long long> nraw_;  // [0] raw children, [1] chunk work counter
    DevBuf<Seg> segs_;

    // Frontier (ping-pong): K64 {key, count} records, or K128 keys + counts.
    DevBuf<ulonglong2> keys_[2];
    DevBuf<unsigned long long> cnts_[2];
    int cur_ = 0;
    uint64_t n_cur_ = 0;

    DevBuf<ulonglong2> table_;    // slot_units() 16-byte units per slot
    // Partitioned dedup buffers: bucketed raw children, bucket counters,
    // merged bucket tables.
    DevBuf<ulonglong2> bkt_recs_;
    DevBuf<unsigned int> bkt_cnt_;
    DevBuf<ulonglong2> dtab_;
    double raw_ratio_ = 0.0;      // raw children per input state, last group
    bool merge_ready_ = false;
    uint64_t table_clean_ = 0;    // units [0, table_clean_) are known to be zero
    double growth_ = 8.0;

    // keep_levels storage: level r = states after completing r rows (r = 0 is the root).
    std::vector<ulonglong2 *> lvl_keys_;
    std::vector<unsigned long long *> lvl_cnts_;
    std::vector<uint64_t> lvl_n_;

    // Kept levels of solve-one instances: one block per step, allocated
    // stream-ordered, freed when no instance refers to it any more.
    struct LvlChunk {
        ulonglong2 *keys = nullptr;
        unsigned long long *cnts = nullptr;
        uint64_t bytes = 0;
        uint32_t refs = 0;
    };
    std::vector<LvlChunk> chunks_;
    std::vector<uint32_t> free_chunks_;
    uint64_t lvl_bytes_ = 0;
    cudaMemPool_t pool_ = nullptr;   // the engine's stream-ordered memory pool
    DevBuf<CopyRange> ranges_;
    DevBuf<unsigned long long> keep_max_;
    std::vector<unsigned long long> h_keep_max_;
    DevBuf<TraceJob> jobs_;
    DevBuf<LevelPtr> lvlptr_;
    DevBuf<TraceOut> trace_out_;
    DevBuf<TraceChain> chain_;
    DevBuf<TraceSeg> tsegs_;

    Tuning tune_;
    Totals tot_;
    bool run_started_ = false;
    std::vector<unsigned int> h_unique_;
    std::vector<unsigned int> h_grp_unique_;   // one group's read-back
    std::vector<unsigned long long> h_cursor_;
};

}  // namespace d4e
