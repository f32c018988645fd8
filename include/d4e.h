/*
 * d4e.h -- C ABI of the GB300 (sm_103a) row-by-row polyomino tiling engine.
 *
 * Drop-in boundary for the reference's GPU search path (b1f6c1c4/d4-pieces,
 * src/searcher_cuda.h, src/frow.h).  Plain pointers and sizes only; every
 * entry point returns D4E_OK (0) or a negative error code, with the message
 * available from d4e_last_error() (the reference throws std::runtime_error
 * from THROW / C(), src/util.hpp:73-74, src/util.cuh:23-40; the C++ facade in
 * d4-pieces_gb300/host/searcher_cuda.h turns the codes back into exceptions).
 *
 * Board layout: rows of up to 8 cells; bit c of row r set = cell (r, c) must
 * be covered.  The reference's `uint64_t empty_area` is the same layout for
 * an 8-wide board of up to 8 rows (bit 8*r + c, src/searcher_cuda.h:11).
 * Piece shapes use the reference's Shape<8> layout (bit 8*r + c,
 * src/Shape.hpp:20-24); `sym` selects transforms in Shape::transforms()
 * order (0xFF = all eight D4 transforms, 0x69 = rotations only).
 *
 * Results are exact: the number of tilings of the board by a sub-multiset of
 * the pieces (copies of one piece type are indistinguishable), as the
 * reference's CPU solver solve_count (src/Piece.cpp:104-139) counts them.
 *
 * Threading: one thread at a time per handle; distinct handles may be used
 * concurrently.  The library owns all device memory it allocates; callers
 * own their host buffers.
 */
#ifndef D4E_H
#define D4E_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define D4E_OK 0
#define D4E_ERR_INVALID (-1)     /* bad argument */
#define D4E_ERR_CUDA (-2)        /* CUDA runtime error (no device, launch failure, ...) */
#define D4E_ERR_NOMEM (-3)       /* device memory exhausted */
#define D4E_ERR_UNSUPPORTED (-4) /* outside the engine's limits (see below) */
#define D4E_ERR_STATE (-5)       /* call not valid in the handle's current state */

/* Limits: board width 1..8, height 1..64, <= 40 piece types whose copy
 * counters (bit_length(count) bits each) fit in 40 bits, <= 255 placements
 * anchored at one column, pieces no taller than 64/width rows. */

/* Message of the last failing call on this thread ("" if none). */
const char *d4e_last_error(void);

/* Library version string. */
const char *d4e_version(void);

/* Number of visible CUDA devices (0 when there is no driver or device); the
 * reference's transfer_frow_to_gpu counts them with cudaGetDeviceCount
 * (src/frow.cu:8-12). */
int d4e_device_count(int32_t *n);

/* Prints the CUDA devices (reference: show_gpu_devices, src/frow.cu:37-90). */
int d4e_show_gpu_devices(void);

/* ------------------------------------------------------------------------
 * Piece catalogue (reference: known_shapes / known_C_shapes, src/known.hpp:9-19,
 * src/known1.cpp, src/known2.cpp).  Canonical polyominoes of m cells
 * (m = 1..8) sorted by value; onesided != 0 selects the one-sided set.
 * Writes up to max values; *n receives the catalogue size.
 * ---------------------------------------------------------------------- */
int d4e_catalogue(uint32_t m, int32_t onesided, uint64_t *out, uint32_t max, uint32_t *n);

/* ------------------------------------------------------------------------
 * Placement ("frow") tables.
 * ---------------------------------------------------------------------- */
typedef struct d4e_frow d4e_frow;

/* Builds the placement tables of a piece library for boards of the given
 * width: every allowed orientation of every piece anchored at every column.
 * Replaces compute_frow_on_cpu(bool show_report) (src/frow.h:10,
 * src/frow.cpp:39-166), which reads the piece set from the globals g_nme /
 * g_sym; here the pieces are explicit.  show_report != 0 prints the
 * per-column placement counts like the reference's report. */
int d4e_frow_create(const uint64_t *shapes, const uint32_t *counts, uint32_t n_pieces,
                    uint32_t sym, uint32_t width, int32_t show_report, d4e_frow **out);

/* Binds the tables to a CUDA device (they are uploaded into each searcher's
 * device table slot when the searcher is created).  Replaces
 * transfer_frow_to_gpu() (src/frow.h:11, src/frow.cu:7-35); fails with
 * D4E_ERR_CUDA "no CUDA device" like the reference. */
int d4e_frow_transfer(d4e_frow *f, int32_t device);

/* Number of placements anchored at column col (the reference reports
 * h_frowInfoL/R[..].sz, src/frow.h:41-48). */
int d4e_frow_placements(const d4e_frow *f, uint32_t col, uint32_t *n);

void d4e_frow_destroy(d4e_frow *f);

/* ------------------------------------------------------------------------
 * Searcher: one puzzle, one board row per search_GPU() call.
 * Reference: struct CudaSearcher (src/searcher_cuda.h:10-38,
 * src/searcher_cuda.cu:12-90).
 * ---------------------------------------------------------------------- */
typedef struct d4e_searcher d4e_searcher;

#define D4E_KEEP_LEVELS 1u   /* retain every row's frontier: enables d4e_searcher_solutions */
#define D4E_AUTOTUNE 2u      /* measure launch plans on the first row of 2^21..2^25 states
                                (cached per process); replaces KSizing::optimize */
#define D4E_DEDUP_DIRECT 4u  /* de-duplicate every row by direct hash-table inserts */
#define D4E_DEDUP_PARTITIONED 8u  /* de-duplicate every eligible row (packed keys, after
                                     the first row) through hash buckets merged on chip
                                     (default: direct inserts) */

/* Forgets every launch plan measured so far in this process (the next
 * autotuned engine measures again). */
void d4e_autotune_clear(void);

/* Device memory kept for reuse: when an engine (a searcher, a batch call, a
 * server lane) ends, its memory pool, with the device memory it has mapped,
 * is kept for the next engine on that device (at most one pool per device),
 * so back-to-back calls do not map their memory again.  This call returns
 * the kept memory to the driver. */
void d4e_release_cached_memory(void);

/* CudaSearcher(uint64_t empty_area): 8-wide board, height = number of rows up
 * to the last cell to cover (src/searcher_cuda.cu:12-21).  The frow tables
 * must have width 8 and have been transferred. */
int d4e_searcher_create(const d4e_frow *f, uint64_t empty_area, d4e_searcher **out);

/* Board of any height 1..64 with the frow tables' width; flags = 0 or
 * D4E_KEEP_LEVELS | D4E_AUTOTUNE. */
int d4e_searcher_create_board(const d4e_frow *f, uint32_t height, const uint8_t *rows,
                              uint32_t flags, d4e_searcher **out);

/* Rows still to be completed (CudaSearcher::get_height). */
int d4e_searcher_get_height(const d4e_searcher *s, uint32_t *height);

/* Current frontier size in states (CudaSearcher::size()). */
int d4e_searcher_size(const d4e_searcher *s, uint64_t *n);

/* States of the current frontier whose current row equals the 8-bit pattern
 * `bucket` (CudaSearcher::size(unsigned i), the reference's 256 row-byte
 * buckets). */
int d4e_searcher_bucket_size(d4e_searcher *s, uint32_t bucket, uint64_t *n);

/* Estimated size of the next frontier (CudaSearcher::next_size()). */
int d4e_searcher_next_size(const d4e_searcher *s, uint64_t *n);

/* Completes one board row: expands every state by every whole-row fill and
 * de-duplicates the children on the device (CudaSearcher::search_GPU). */
int d4e_searcher_search_GPU(d4e_searcher *s);

/* Runs search_GPU until the height reaches 0. */
int d4e_searcher_run(d4e_searcher *s);

/* Number of tilings; valid once the height is 0. */
int d4e_searcher_count(d4e_searcher *s, uint64_t *count);

/* Tilings of a finished searcher created with D4E_KEEP_LEVELS, reconstructed
 * on the device from the per-row frontiers.  Each solution is a W*H grid of
 * piece type ids (type_grids) and of step indices in placement order
 * (step_grids), -1 outside the board, like the reference's
 * Solution::map + Step::piece_id (src/Piece.hpp:31-48).  single != 0 returns
 * one tiling (reference solve(..., single = true)).  Either grid pointer may
 * be NULL.  *n receives the number written (<= max). */
int d4e_searcher_solutions(d4e_searcher *s, uint64_t max, int32_t single, int8_t *type_grids,
                           int8_t *step_grids, uint64_t *n);

/* Per-row frontier sizes (states after each completed row); writes up to max
 * entries, *n receives the number of completed rows. */
int d4e_searcher_level_sizes(const d4e_searcher *s, uint64_t *sizes, uint32_t max, uint32_t *n);

typedef struct d4e_stats {
    uint64_t rows;              /* search_GPU steps run */
    uint64_t states_in;         /* frontier states expanded (sum over rows) */
    uint64_t states_raw;        /* children produced before de-duplication */
    uint64_t states_out;        /* distinct children (sum over rows) */
    uint64_t peak_frontier;     /* largest frontier */
    uint64_t expand_launches;   /* k_expand launches (including table-growth retries) */
    uint64_t compact_launches;  /* k_compact launches */
    uint64_t retries;           /* rows redone after a table overflow */
    uint64_t other_launches;    /* other kernels (bucket counts, ...) */
    uint64_t h2d_bytes;         /* host-to-device bytes copied by the engine */
    uint64_t d2h_bytes;         /* device-to-host bytes copied by the engine */
    double expand_ms;           /* device time of k_expand (CUDA events) */
    double compact_ms;          /* device time of k_compact (CUDA events) */
    double run_ms;              /* CUDA-event time from the first row's start to the last row's end */
    uint64_t record_bytes;      /* bytes per frontier state: 16 (packed 64-bit keys) or 24 */
    uint64_t slot_bytes;        /* bytes per hash-table slot: 16 or 32 */
    uint64_t paused;            /* instance-rows that waited for device memory */
    uint64_t splits;            /* batch groups split after a table overflow */
    uint64_t failed;            /* instances that ended with an error */
    uint64_t restarts;          /* solve-one attempts redone with a wider sample */
    double step_wall_ms;        /* host wall time inside the engine's row steps */
    double upload_ms;           /* ... of which: uploading new instances */
    double keep_ms;             /* ... keeping solve-one levels */
    double trace_ms;            /* ... tracing solve-one tilings */
    double tune_ms;             /* host time in autotuning trials */
    uint64_t tuned_chunk_cap;   /* launch plan in use: most items a warp takes at once */
    uint64_t tuned_chunks_per_warp; /* chunks per resident warp aimed at */
    uint64_t tuned_ctas_per_sm; /* k_expand CTAs per SM (0 = occupancy) */
    double tuned_load;          /* hash table load factor */
    uint64_t compact_slots;     /* hash-table slots scanned by k_compact (all launches) */
    double phase_ms[6];         /* host wall time inside row steps: selecting instances,
                                   preparing tables, waiting for k_expand, bookkeeping,
                                   waiting for k_compact, row tail */
    uint64_t partitioned;       /* row groups de-duplicated through buckets */
    uint64_t partition_fallbacks; /* ... redone with the direct table (bucket overflow) */
    double merge_ms;            /* device time of k_bucket_merge (also in compact_ms) */
    uint64_t tuned_compact_ctas;   /* k_compact blocks per SM in the launch plan */
    uint64_t tuned_compact_stages; /* k_compact shared-memory ring depth (32 KB tiles) */
} d4e_stats;

int d4e_searcher_stats(const d4e_searcher *s, d4e_stats *st);

/* Makes search_GPU fail with D4E_ERR_UNSUPPORTED once a row would produce
 * more than max_states distinct states (0 = no limit), a guard for
 * exploratory runs; the reference sizes its ring buffer from free memory
 * instead (src/device.cu:30-32). */
int d4e_searcher_set_limit(d4e_searcher *s, uint64_t max_states);

void d4e_searcher_destroy(d4e_searcher *s);

/* ------------------------------------------------------------------------
 * Batches: many independent puzzles.  The reference runs one CudaSearcher per
 * board configuration from a thread pool (SearcherFactory::run,
 * src/searcher.cpp:86-107).
 * ---------------------------------------------------------------------- */
typedef struct d4e_instance {
    uint32_t width;             /* 1..8 */
    uint32_t height;            /* 1..64 */
    const uint8_t *rows;        /* height row masks */
    uint32_t n_pieces;
    const uint64_t *shapes;     /* Shape<8> layout */
    const uint32_t *counts;     /* copies per piece type */
    uint32_t sym;               /* allowed transforms */
} d4e_instance;

#define D4E_BATCH_SEQUENTIAL 1u /* one puzzle at a time, one launch sequence per puzzle */
#define D4E_BATCH_WIDE_KEYS 2u  /* d4e_batch_run: the general 128-bit key encoding for all */
#define D4E_BATCH_AUTOTUNE 4u   /* d4e_batch_run: measure launch plans (see D4E_AUTOTUNE) */
#define D4E_BATCH_DEDUP_DIRECT 8u        /* see D4E_DEDUP_DIRECT */
#define D4E_BATCH_DEDUP_PARTITIONED 16u  /* see D4E_DEDUP_PARTITIONED */

/* Counts the tilings of every instance.  Default: all instances advance
 * together, one k_expand + one k_compact launch per board row for the whole
 * batch.  With D4E_BATCH_SEQUENTIAL each instance runs alone (the plain
 * per-puzzle path).  counts[i] receives instance i's count.  st may be NULL. */
int d4e_batch_count(const d4e_instance *insts, uint32_t n, uint32_t flags, int32_t device,
                    uint64_t *counts, d4e_stats *st);

#define D4E_MODE_COUNT 0u      /* solve-all: count every tiling */
#define D4E_MODE_SOLVE_ONE 1u  /* one tiling, or none when there is none */
#define D4E_MODE_SETS 2u       /* the piece multisets that tile the board (the pieces'
                                  counts are maxima), each with its number of tilings;
                                  results: count = all tilings, found = number of sets */
#define D4E_MODE_LIST 3u       /* every tiling itself (d4e_batch_solutions only) */

typedef struct d4e_batch_opts {
    uint32_t mode;              /* D4E_MODE_* for every instance */
    uint32_t flags;             /* D4E_BATCH_SEQUENTIAL */
    int32_t device;
    uint32_t reserved;
    uint64_t memory_budget;     /* device bytes for frontiers + table (0 = device less 10%) */
    uint64_t max_states;        /* per-instance limit on one row's frontier (0 = none) */
    uint64_t beam;              /* solve-one: states kept per row on the first attempt
                                   (0 = exact); see d4e_batch_run */
} d4e_batch_opts;

/* Result of one instance (batch) or request (server). */
typedef struct d4e_result {
    uint64_t tag;               /* batch: instance index; server: the submit tag */
    int32_t status;             /* D4E_OK, or the error the instance ended with */
    uint32_t mode;              /* D4E_MODE_* */
    uint64_t count;             /* count mode: tilings; solve-one: 1 when found */
    uint32_t found;             /* solve-one: grid holds a tiling */
    uint32_t rows;              /* board rows completed */
    double queued_ms;           /* server: submit -> admitted to the device */
    double latency_ms;          /* submit (server) or batch start -> result */
    int8_t grid[512];           /* solve-one: piece type per cell, row-major
                                   (width * height cells), -1 = not covered */
    int16_t steps[512];         /* solve-one: placement number per cell (anchor
                                   order), -1 = not covered */
} d4e_result;

/* Runs a batch.  Instances advance together, one k_expand + k_compact pair
 * per board row for the whole batch (grouped when memory runs short;
 * instances that do not fit wait, in order, until memory frees up).  With
 * D4E_BATCH_SEQUENTIAL each instance runs alone instead.  A failing
 * instance (its max_states, or a row the device cannot hold) gets an error
 * status; the others are unaffected.
 *
 * Solve-one: every row is de-duplicated as in counting; with beam > 0 a row
 * whose distinct states exceed beam keeps about beam of them, chosen by a
 * hash of the state alone.  When such an attempt dies out it is redone with
 * a 16x wider sample, and exactly once the sample width has passed 2^20
 * states, so "not found" is always exact.  The tiling reported is the same
 * whether the instance runs alone or in any batch.  results[i].tag = i. */
int d4e_batch_run(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *opts,
                  d4e_result *results, d4e_stats *st);

/* Piece-set mode over a batch (the reference's research use: which piece
 * combinations tile each board of a family, src/search.cpp:25-54, with the
 * ledger of Naming ranks, src/naming.inl:6-72, left to the caller).  Every
 * instance runs in D4E_MODE_SETS; its multisets are set_offsets[i] ..
 * set_offsets[i+1]-1, sorted by copies; set k has set_copies[k * 64 + p]
 * copies of piece p and set_tilings[k] tilings.  set_offsets has n + 1
 * entries; when more than max_sets sets exist the call fails with
 * D4E_ERR_INVALID and set_offsets[n] holds the number needed. */
#define D4E_SET_PIECES 64u
int d4e_batch_sets(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *opts,
                   d4e_result *results, uint64_t *set_offsets, uint8_t *set_copies,
                   uint64_t *set_tilings, uint64_t max_sets, d4e_stats *st);

/* Lists the tilings of every instance of a batch: the reference's Solution /
 * Step list (src/Piece.hpp:31-48, src/Piece.cpp:25-54; d4e_searcher_solutions
 * for one board) for many boards in one run.  The instances advance together
 * as in counting, each keeping every row's frontier on the device (device
 * memory grows with the sum of all rows of all instances); each instance's
 * tilings are then reconstructed from its own rows.  Instance i's tilings
 * are sol_offsets[i] .. sol_offsets[i+1]-1 (at most max_per_instance, in no
 * particular order); tiling k has piece type type_grids[k * D4E_GRID_CELLS + c]
 * and placement number step_grids[k * D4E_GRID_CELLS + c] at cell c (row-major,
 * width * height cells, -1 = not covered or beyond the board).
 * results[i].count = all tilings of instance i.  sol_offsets has n + 1
 * entries; when more than max_total tilings would be listed the call fails
 * with D4E_ERR_INVALID and sol_offsets[n] holds the number needed.  Boards of
 * up to 512 cells; opts->mode and opts->beam are ignored. */
#define D4E_GRID_CELLS 512u
int d4e_batch_solutions(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *opts,
                        uint64_t max_per_instance, d4e_result *results, uint64_t *sol_offsets,
                        int8_t *type_grids, int16_t *step_grids, uint64_t max_total,
                        d4e_stats *st);

/* ------------------------------------------------------------------------
 * Serving: a request loop on a native worker thread.  No counterpart in the
 * reference (its SearcherFactory runs a fixed job list).
 *
 * Requests queue on submit and are admitted in arrival order while the
 * projected device bytes of the admitted requests (frontier + hash table of
 * their next row) stay within memory_budget; admitted requests join the
 * running batch at its next row, so work of requests that arrived at
 * different times shares each k_expand / k_compact launch.  Two lanes run
 * concurrently on their own streams: every request starts in the fast lane
 * (rows of at most 2^17 distinct states); one that outgrows it restarts in
 * the slow lane, whose kernels leave room on every SM for the fast lane's,
 * whose heavy row steps wait for (and whose k_expand launches are preempted
 * by) fast-lane work, and whose heaviest requests sit out some row steps so
 * that lighter ones are not paced by them.  A request that runs out of
 * device memory beside others restarts in the slow lane (at most twice).
 * Results are the same as alone (counts exact; solve-one tilings as in
 * d4e_batch_run).
 * ---------------------------------------------------------------------- */
typedef struct d4e_server d4e_server;

typedef struct d4e_server_opts {
    int32_t device;
    uint32_t max_active;        /* fast-lane requests on the device at once (0 = 4096);
                                   the slow lane takes max_active / 16 (at least 16) */
    uint64_t memory_budget;     /* admission budget in bytes (0 = 150 GB, capped at the
                                   device's memory less 10%) */
    uint64_t max_states;        /* per-request limit on one row's frontier (0 = none) */
    uint64_t beam;              /* solve-one first sample width (0 = exact) */
} d4e_server_opts;

int d4e_server_create(const d4e_server_opts *opts, d4e_server **out);

/* Queues a request (the instance is copied).  Thread-safe. */
int d4e_server_submit(d4e_server *s, const d4e_instance *inst, uint32_t mode, uint64_t tag);

/* Moves up to max finished results into out; *n receives the number.
 * Thread-safe. */
int d4e_server_poll(d4e_server *s, d4e_result *out, uint32_t max, uint32_t *n);

/* Waits until every submitted request has a result (or timeout_s passes:
 * D4E_ERR_STATE). */
int d4e_server_drain(d4e_server *s, double timeout_s);

typedef struct d4e_server_stats {
    uint64_t submitted, admitted, completed, failed;
    uint64_t steps;             /* batch rows run */
    uint64_t peak_active;       /* most requests on the device at once */
    uint64_t peak_projected;    /* largest projected bytes admitted */
    uint64_t states_out;        /* distinct states produced (all requests) */
    double busy_ms;             /* worker time spent in device steps (both lanes) */
    uint64_t moved;             /* requests restarted in the slow lane */
    uint64_t lane_steps[2];     /* per lane (fast, slow): engine steps */
    double lane_busy_ms[2];     /* per lane: wall time in engine steps */
    double lane_kernel_ms[2];   /* per lane: k_expand + k_compact device time */
    uint64_t lane_inst_rows[2]; /* per lane: instance-rows advanced */
    uint64_t restarts;          /* solve-one attempts redone with a wider sample */
    uint64_t paused;            /* instance-rows that waited for memory */
    double lane_admit_ms[2];    /* per lane: admitting requests (placement tables built) */
    double lane_collect_ms[2];  /* per lane: handing out finished results */
    double lane_upload_ms[2];   /* per lane, inside steps: uploading new instances */
    double lane_solve_one_ms[2];/* per lane, inside steps: keeping levels + tracing */
    uint64_t lane_retries[2];   /* per lane: table-region overflows redone */
    double lane_phase_ms[2][6]; /* per lane: the row-step phases of d4e_stats.phase_ms */
    uint64_t preemptions;       /* slow-lane k_expand launches ended early for the fast lane */
} d4e_server_stats;

int d4e_server_stats_get(d4e_server *s, d4e_server_stats *st);

/* Stops the worker (requests still queued are dropped) and frees the device
 * memory. */
void d4e_server_destroy(d4e_server *s);

/* ------------------------------------------------------------------------
 * Counting without device allocation.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: processes that reserve their
 * device memory once at start-up and may not grow it afterwards (a server
 * sharing the GPU with other tenants under a fixed budget, where an
 * allocation in the middle of a request can fail or stall behind other
 * work), and code running under a caller-owned memory pool that forbids the
 * runtime allocator.  d4e_count_noalloc allocates no device memory and calls
 * no allocating library routine: every buffer it needs (descriptor,
 * placement table, two frontier buffers, the de-duplication table, counters)
 * lives in one file-scope __device__ array of D4E_NOALLOC_SCRATCH_BYTES that
 * every GPU loading the library holds until the process exits.
 *
 * Works on the current CUDA device; stream may be NULL (legacy default
 * stream).  The first call on each device resolves the array's device
 * address (cudaGetSymbolAddress) and keeps it for the life of the process,
 * so do not call it again on a device after cudaDeviceReset.  Every call
 * synchronises its stream after each board row (it reads the row's state
 * count back to the host), so it must never be called while that stream is
 * being captured.  All calls share the array and it keeps the last call's
 * contents (each call clears what it needs): calls that overlap on the GPU
 * -- from several host threads or on several streams of one device -- race
 * and must be serialised by the caller.  A puzzle whose row frontier exceeds
 * the array's capacity (about 1.0M states with packed 64-bit keys, 0.59M
 * otherwise) fails with D4E_ERR_UNSUPPORTED.  *count receives the number of
 * tilings; states (may be NULL) the sum of the per-row frontier sizes. */
#define D4E_NOALLOC_SCRATCH_BYTES (64u << 20)

int d4e_count_noalloc(const d4e_instance *inst, void *stream, uint64_t *count,
                      uint64_t *states);

/* Canonical D4 form of a solution type grid over the board's own symmetry
 * (lexicographic minimum over the transforms mapping the board onto
 * itself). */
int d4e_canonical_grid(uint32_t width, uint32_t height, const uint8_t *rows, const int8_t *grid,
                       int8_t *out);

#ifdef __cplusplus
}
#endif

#endif /* D4E_H */
