/*
 * d4oracle.h -- CPU oracle for the row-by-row polyomino tiling engine.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is used by tests/ (as the checker), by
 * __graft_entry__.smoke() (as the checker) and by bench.py's cpu_baseline /
 * `--impl reference` leg (as the timed CPU baseline).
 *
 * Two independent restatements of the reference's algorithms:
 *
 *  1. or_solve_count / or_solve: the reference's CPU backtracking solver
 *     (src/Piece.cpp:104-139 solve_count, src/Piece.cpp:65-102 solve,
 *     src/Piece.inl:5-24 Piece::cover, src/Piece.cpp:12-22 Piece::Piece),
 *     generalised from Shape<8>/Shape<11> to a W x H board (W <= 11,
 *     W*H <= 128) held in a 128-bit bitboard with row stride W.  Same
 *     lowest-cell-first order, same piece/placement/anchor iteration order,
 *     same max_tiles/min_tiles prunes, same per-type `count` semantics
 *     (copies of a piece type are indistinguishable).
 *
 *  2. or_rowdp: the reference's row-by-row level search
 *     (src/searcher_cuda.cu:12-90 CudaSearcher, src/kernel.cuh:12-49 impl)
 *     restated EXACTLY: one level per board row, each state expanded by
 *     every set of placements anchored in the current row that covers all
 *     of its empty cells (no L/R half split, no island pruning), states
 *     de-duplicated per level with tiling multiplicities summed.  It yields
 *     per-level frontier sizes and the tiling count.  or_rowdp_lean is the
 *     same DP with children de-duplicated as they are produced (for
 *     frontiers of 10^8 states and more).
 *
 * Parity of (1) is pinned against the reference's own solver, compiled from
 * the reference sources by oracle/Makefile into oracle/_ref/d4ref, through
 * the committed fixtures in tests/golden/.
 */
#ifndef D4ORACLE_H
#define D4ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_problem {
    int32_t width;            /* 1..11 */
    int32_t height;           /* width*height <= 128 */
    const uint16_t *rows;     /* rows[r] bit c set: cell (r,c) must be covered */
    int32_t n_pieces;
    const uint64_t *shapes;   /* Shape<8> layout: bit 8*r + c */
    const uint32_t *counts;   /* copies of each piece type */
    uint32_t sym;             /* allowed transforms, bit i = Shape::transforms()[i] */
} or_problem;

/* Number of tilings (reference solve_count).  Returns -1 on bad input. */
int64_t or_solve_count(const or_problem *p);

/* Reference solve(lib, board, single).  Writes up to max_solutions solutions:
 * type_grids[k*W*H + cell] = piece type id covering the cell (-1 if the cell
 * is not part of the board), step_grids[...] = index of the placement (step)
 * covering the cell.  Either output pointer may be NULL.  Returns the number
 * of solutions found (all of them, even beyond max_solutions), -1 on error. */
int64_t or_solve(const or_problem *p, int32_t single, int64_t max_solutions,
                 int8_t *type_grids, int8_t *step_grids);

/* Canonical D4 form of a type grid: lexicographic minimum over the board's
 * own symmetry transforms (those mapping the board's cell set onto itself),
 * transforms taken in Shape::transforms() order.  out has W*H entries. */
void or_canonical_grid(const or_problem *p, const int8_t *grid, int8_t *out);

/* Exact row-by-row frontier DP.  level_sizes[r] = number of distinct states
 * after completing row r (r = 0..H-1).  *count = number of tilings (mod
 * 2^64).  threads >= 1.  max_seconds > 0 stops once the elapsed time passes
 * the budget and max_children > 0 once a level's children exceed it (host
 * memory bound), both in the middle of a level if need be; when the cap
 * stops a level with time left, the rest of that level is sampled in
 * memory-bounded batches (expanded and de-duplicated, then dropped) until
 * the budget is spent.  *levels_done reports how many rows were completed
 * and *states_total how many frontier states were expanded (whole rows plus
 * the expanded part of the interrupted row).
 * Returns 0 on success, -1 on bad input. */
int32_t or_rowdp(const or_problem *p, int32_t threads, double max_seconds,
                 uint64_t max_children, uint64_t *level_sizes, uint64_t *count,
                 int32_t *levels_done, uint64_t *states_total);

/* The same exact row DP with bounded memory: children are de-duplicated as
 * they are produced (hash shards with one lock each) instead of stored
 * first, so memory holds each level's distinct states only (32 bytes each,
 * plus the shards' free slots).  level_sizes[r] = distinct states after
 * row r, raw_sizes[r] = children produced while completing row r (either
 * may be NULL); *count = tilings (mod 2^64; 0 unless every row ran);
 * *seconds = elapsed time.  max_rows > 0 stops after that many whole rows
 * (a timed sample of the first rows), otherwise every row runs.  Returns 0,
 * -1 on bad input, -2 when host memory ran out. */
int32_t or_rowdp_lean(const or_problem *p, int32_t threads, int32_t max_rows,
                      uint64_t *level_sizes, uint64_t *raw_sizes, uint64_t *count,
                      double *seconds);

/* Independent cover check of one tiling given as placements:
 * piece type + cell mask (lo/hi 64-bit halves of the W-stride bitboard).
 * Returns 1 when the placements are pairwise disjoint, cover exactly the
 * board, each is an allowed transform of its type's shape, and no type is
 * used more often than its count.  Returns 0 otherwise. */
int32_t or_check_tiling(const or_problem *p, int32_t n, const int32_t *types,
                        const uint64_t *mask_lo, const uint64_t *mask_hi);

#ifdef __cplusplus
}
#endif

#endif
