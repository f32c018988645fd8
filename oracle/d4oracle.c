/*
 * d4oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see d4oracle.h).
 *
 * Restates, in plain C, the reference's CPU backtracking solver and its
 * row-by-row level search.  Each function cites the reference file:line it
 * follows.  The product library never links or calls this file.
 */
#include "d4oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef unsigned __int128 u128;

#define OR_MAX_TYPES 128
#define OR_MAX_COPIES 64

/* ------------------------------------------------------------------------
 * Shape<8> geometry on a uint64 (bit 8*r + c), reference src/Shape.hpp:182-191
 * (normalize) and src/Shape.cpp:6-40 (transform / transforms order).
 * ---------------------------------------------------------------------- */
static uint64_t s8_normalize(uint64_t v)
{
    if (!v)
        return 0;
    while (!(v & 0xFFull))
        v >>= 8;
    while (!(v & 0x0101010101010101ull))
        v >>= 1;
    return v;
}

/* Transform index t follows Shape::transforms(): bit0 = FlipX, bit1 = FlipY,
 * bit2 = Swap; out(r,c) = in(ir,ic) (src/Shape.cpp:12-21), then normalize. */
static uint64_t s8_transform(uint64_t v, int t)
{
    int sw = (t >> 2) & 1, fx = t & 1, fy = (t >> 1) & 1;
    uint64_t out = 0;
    for (int r = 0; r < 8; r++)
        for (int c = 0; c < 8; c++) {
            int ir = sw ? c : r, ic = sw ? r : c;
            if (fx)
                ic = 7 - ic;
            if (fy)
                ir = 7 - ir;
            if ((v >> (ir * 8 + ic)) & 1u)
                out |= 1ull << (r * 8 + c);
        }
    return s8_normalize(out);
}

static int popc128(u128 v)
{
    return __builtin_popcountll((uint64_t)v) + __builtin_popcountll((uint64_t)(v >> 64));
}

static int ctz128(u128 v)
{
    uint64_t lo = (uint64_t)v;
    return lo ? __builtin_ctzll(lo) : 64 + __builtin_ctzll((uint64_t)(v >> 64));
}

/* ------------------------------------------------------------------------
 * Piece library, reference src/Piece.cpp:12-22 (Piece::Piece): one entry per
 * transform allowed by `sym`, in transforms() order; a transform equal to an
 * earlier one is kept but disabled.
 * ---------------------------------------------------------------------- */
typedef struct {
    uint64_t normal;   /* normalized Shape<8> value */
    int h, w;          /* bounding box */
    int enabled;
    int ncells;
    int cr[64], cc[64]; /* cells in increasing bit order (Shape iteration) */
} or_plc;

typedef struct {
    uint32_t count;
    int size;
    int nplc;
    or_plc plc[8];
} or_piece;

typedef struct {
    int W, H;
    u128 board;
    int n;
    or_piece *lib;
} or_ctx;

static int build_ctx(const or_problem *p, or_ctx *c)
{
    if (!p || p->width < 1 || p->width > 11 || p->height < 1 ||
        p->width * p->height > 128 || p->n_pieces < 0 || p->n_pieces > OR_MAX_TYPES)
        return -1;
    c->W = p->width;
    c->H = p->height;
    c->n = p->n_pieces;
    c->board = 0;
    for (int r = 0; r < c->H; r++)
        for (int x = 0; x < c->W; x++)
            if ((p->rows[r] >> x) & 1u)
                c->board |= (u128)1 << (r * c->W + x);
    c->lib = (or_piece *)calloc(c->n ? c->n : 1, sizeof(or_piece));
    for (int i = 0; i < c->n; i++) {
        or_piece *pc = &c->lib[i];
        uint64_t s = p->shapes[i];
        if (!s) {
            free(c->lib);
            return -1;
        }
        pc->count = p->counts[i];
        pc->size = __builtin_popcountll(s);
        pc->nplc = 0;
        unsigned sym = p->sym;
        for (int t = 0; t < 8; t++, sym >>= 1) {
            if (!(sym & 1u))
                continue;
            uint64_t sh = s8_transform(s, t);
            or_plc *pl = &pc->plc[pc->nplc++];
            pl->normal = sh;
            pl->enabled = 1;
            for (int k = 0; k < pc->nplc - 1; k++)
                if (pc->plc[k].normal == sh)
                    pl->enabled = 0;
            pl->h = pl->w = 0;
            pl->ncells = 0;
            for (int b = 0; b < 64; b++)
                if ((sh >> b) & 1u) {
                    int r = b / 8, x = b % 8;
                    pl->cr[pl->ncells] = r;
                    pl->cc[pl->ncells] = x;
                    pl->ncells++;
                    if (r + 1 > pl->h)
                        pl->h = r + 1;
                    if (x + 1 > pl->w)
                        pl->w = x + 1;
                }
        }
    }
    return 0;
}

/* Placement cell mask with its top-left corner at (y, x) of the W-stride board. */
static u128 plc_mask(const or_ctx *c, const or_plc *pl, int y, int x)
{
    u128 m = 0;
    for (int k = 0; k < pl->ncells; k++)
        m |= (u128)1 << ((pl->cr[k] + y) * c->W + pl->cc[k] + x);
    return m;
}

/* ------------------------------------------------------------------------
 * Backtracking solver, reference src/Piece.cpp:57-139 and src/Piece.inl:5-24.
 * ---------------------------------------------------------------------- */
typedef struct {
    or_ctx *c;
    uint32_t used[OR_MAX_TYPES];
    int max_tiles;
    uint64_t count;
    /* solve() */
    int single;
    int64_t nsol, maxsol;
    int nstep;
    int step_type[128];
    u128 step_mask[128];
    int8_t *type_grids, *step_grids;
} or_search;

/* min_tiles, src/Piece.cpp:57-63 */
static int min_tiles(const or_search *s)
{
    int m = 1 << 30;
    for (int i = 0; i < s->c->n; i++)
        if (s->used[i] < s->c->lib[i].count && s->c->lib[i].size < m)
            m = s->c->lib[i].size;
    return m;
}

static void record_solution(or_search *s)
{
    if (s->nsol < s->maxsol) {
        int cells = s->c->W * s->c->H;
        int8_t *tg = s->type_grids ? s->type_grids + s->nsol * cells : NULL;
        int8_t *sg = s->step_grids ? s->step_grids + s->nsol * cells : NULL;
        for (int cell = 0; cell < cells; cell++) {
            int id = -1;
            for (int k = 0; k < s->nstep; k++)
                if ((s->step_mask[k] >> cell) & 1u) {
                    id = k;
                    break;
                }
            if (tg)
                tg[cell] = (int8_t)(id < 0 ? -1 : s->step_type[id]);
            if (sg)
                sg[cell] = (int8_t)id;
        }
    }
    s->nsol++;
}

/* The recursive lambda `f` of solve / solve_count.  Returns 1 to stop
 * (solve with single == true found a solution). */
static int search_rec(or_search *s, u128 open, int want_solutions)
{
    const or_ctx *c = s->c;
    int sz = popc128(open);
    if (sz > s->max_tiles)
        return 0;
    if (!open) {
        if (want_solutions) {
            record_solution(s);
            return s->single;
        }
        s->count++;
        return 0;
    }
    if (sz < min_tiles(s))
        return 0;
    int pos = ctz128(open);
    int ty = pos / c->W, tx = pos % c->W;
    for (int id = 0; id < c->n; id++) {
        const or_piece *pc = &c->lib[id];
        if (s->used[id] == pc->count)
            continue;
        s->used[id]++;
        s->max_tiles -= pc->size;
        /* Piece::cover(pos, func), src/Piece.inl:5-24: every enabled
         * placement, every cell of it as the one landing on pos. */
        for (int t = 0; t < pc->nplc; t++) {
            const or_plc *pl = &pc->plc[t];
            if (!pl->enabled)
                continue;
            for (int k = 0; k < pl->ncells; k++) {
                int x = tx - pl->cc[k], y = ty - pl->cr[k];
                if (x < 0 || y < 0 || x + pl->w > c->W || y + pl->h > c->H)
                    continue;
                u128 placed = plc_mask(c, pl, y, x);
                if (placed & ~open)
                    continue;
                if (want_solutions) {
                    s->step_type[s->nstep] = id;
                    s->step_mask[s->nstep] = placed;
                    s->nstep++;
                }
                int stop = search_rec(s, open & ~placed, want_solutions);
                if (want_solutions)
                    s->nstep--;
                if (stop)
                    return 1;
            }
        }
        s->max_tiles += pc->size;
        s->used[id]--;
    }
    return 0;
}

static void init_search(or_search *s, or_ctx *c)
{
    memset(s, 0, sizeof(*s));
    s->c = c;
    for (int i = 0; i < c->n; i++)
        s->max_tiles += c->lib[i].size * (int)c->lib[i].count;
}

int64_t or_solve_count(const or_problem *p)
{
    or_ctx c;
    if (build_ctx(p, &c))
        return -1;
    or_search *s = (or_search *)malloc(sizeof(or_search));
    init_search(s, &c);
    search_rec(s, c.board, 0);
    int64_t r = (int64_t)s->count;
    free(s);
    free(c.lib);
    return r;
}

int64_t or_solve(const or_problem *p, int32_t single, int64_t max_solutions,
                 int8_t *type_grids, int8_t *step_grids)
{
    or_ctx c;
    if (build_ctx(p, &c))
        return -1;
    or_search *s = (or_search *)malloc(sizeof(or_search));
    init_search(s, &c);
    s->single = single ? 1 : 0;
    s->maxsol = max_solutions;
    s->type_grids = type_grids;
    s->step_grids = step_grids;
    search_rec(s, c.board, 1);
    int64_t r = s->nsol;
    free(s);
    free(c.lib);
    return r;
}

/* ------------------------------------------------------------------------
 * Canonical D4 form of a solution grid.  The reference has no solution
 * canonicalisation; this applies Shape::transform's cell mapping
 * (src/Shape.cpp:12-21) to the W x H grid and keeps the transforms that map
 * the board onto itself.
 * ---------------------------------------------------------------------- */
void or_canonical_grid(const or_problem *p, const int8_t *grid, int8_t *out)
{
    int W = p->width, H = p->height, cells = W * H;
    int8_t tmp[128];
    int have = 0;
    for (int t = 0; t < 8; t++) {
        int sw = (t >> 2) & 1, fx = t & 1, fy = (t >> 1) & 1;
        if (sw && W != H)
            continue;
        int ok = 1;
        for (int r = 0; r < H && ok; r++)
            for (int x = 0; x < W; x++) {
                int ir = sw ? x : r, ic = sw ? r : x;
                if (fx)
                    ic = W - 1 - ic;
                if (fy)
                    ir = H - 1 - ir;
                int a = (p->rows[r] >> x) & 1u, b = (p->rows[ir] >> ic) & 1u;
                if (a != b) {
                    ok = 0;
                    break;
                }
                tmp[r * W + x] = grid[ir * W + ic];
            }
        if (!ok)
            continue;
        /* lexicographic over signed cell values */
        int less = !have;
        for (int i = 0; have && i < cells; i++)
            if (tmp[i] != out[i]) {
                less = tmp[i] < out[i];
                break;
            }
        if (less)
            memcpy(out, tmp, (size_t)cells);
        have = 1;
    }
}

/* ------------------------------------------------------------------------
 * Exact row-by-row frontier DP (restating the level structure of
 * src/searcher_cuda.cu:32-82 and the per-record expansion of
 * src/kernel.cuh:12-49 with whole-row fills).
 * State = (open cells of the whole board, used-copy mask).  Copies of a type
 * occupy a contiguous bit range and are taken lowest-free-first, so the mask
 * encodes the per-type used counts.
 * ---------------------------------------------------------------------- */
typedef struct {
    u128 open;
    uint64_t used;
    uint64_t cnt;
} dp_state;

typedef struct {
    dp_state *v;
    size_t n, cap;
} dp_vec;

static void vec_push(dp_vec *a, const dp_state *s)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? a->cap * 2 : 1024;
        a->v = (dp_state *)realloc(a->v, a->cap * sizeof(dp_state));
    }
    a->v[a->n++] = *s;
}

typedef struct {
    uint64_t rel;   /* placement mask relative to its row, anchored at column col */
    uint64_t rel_hi;
    uint64_t tmask; /* copy bits of its piece type */
    int h;          /* rows spanned */
} dp_plc;

typedef struct {
    int W, H, T;
    u128 board;
    int nplc[11];
    dp_plc *plc[11];
} dp_tab;

static uint64_t mix64(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

static uint64_t dp_hash(const dp_state *s)
{
    return mix64((uint64_t)s->open ^ mix64((uint64_t)(s->open >> 64) ^ mix64(s->used)));
}

typedef struct {
    const dp_tab *tab;
    int row;
    dp_vec *shards; /* T shard buffers for this worker */
    int T;
    uint64_t cnt;
    uint64_t pushed, limit; /* children produced by this worker, cap (0 = none) */
    volatile int *abort;
} dp_expand_ctx;

static void dp_fill(dp_expand_ctx *e, u128 open, uint64_t used)
{
    const dp_tab *t = e->tab;
    int W = t->W;
    u128 rowm = (((u128)1 << W) - 1) << (e->row * W);
    if (*e->abort)
        return;
    if (!(open & rowm)) {
        dp_state s = { open, used, e->cnt };
        vec_push(&e->shards[dp_hash(&s) % (uint64_t)e->T], &s);
        if (e->limit && ++e->pushed > e->limit)
            *e->abort = 1;
        return;
    }
    int pos = ctz128(open);
    int col = pos % W;
    for (int i = 0; i < t->nplc[col]; i++) {
        const dp_plc *pl = &t->plc[col][i];
        if (e->row + pl->h > t->H)
            continue;
        u128 m = (((u128)pl->rel_hi << 64) | pl->rel) << (e->row * W);
        if (m & ~open)
            continue;
        uint64_t tm = pl->tmask;
        uint64_t nb = ((used & tm) + (tm & (~tm + 1))) & tm;
        if (!nb)
            continue;
        dp_fill(e, open & ~m, used | nb);
    }
}

typedef struct {
    const dp_tab *tab;
    int row, T, id;
    const dp_state *in;
    size_t lo, hi;
    dp_vec **shards; /* [worker][shard] */
    dp_vec *out;     /* per shard output */
    uint64_t limit;  /* children per worker (0 = none) */
    volatile int *abort;
    double deadline; /* absolute time limit (0 = none) */
    size_t expanded; /* input states fully expanded */
} dp_job;

static double now_s(void);

static void *dp_expand_worker(void *arg)
{
    dp_job *j = (dp_job *)arg;
    dp_expand_ctx e;
    e.tab = j->tab;
    e.row = j->row;
    e.T = j->T;
    e.shards = j->shards[j->id];
    e.pushed = 0;
    e.limit = j->limit;
    e.abort = j->abort;
    j->expanded = 0;
    for (size_t i = j->lo; i < j->hi && !*j->abort; i++) {
        if (j->deadline > 0 && ((i - j->lo) & 255) == 0 && now_s() > j->deadline) {
            *j->abort = 1;
            break;
        }
        e.cnt = j->in[i].cnt;
        dp_fill(&e, j->in[i].open, j->in[i].used);
        if (!*j->abort)
            j->expanded++;
    }
    return NULL;
}

static void *dp_merge_worker(void *arg)
{
    dp_job *j = (dp_job *)arg;
    size_t total = 0;
    for (int w = 0; w < j->T; w++)
        total += j->shards[w][j->id].n;
    size_t cap = 16;
    while (cap < total * 2)
        cap *= 2;
    dp_state *tab = (dp_state *)calloc(cap, sizeof(dp_state));
    unsigned char *occ = (unsigned char *)calloc(cap, 1);
    dp_vec *out = &j->out[j->id];
    out->n = 0;
    for (int w = 0; w < j->T; w++) {
        dp_vec *v = &j->shards[w][j->id];
        for (size_t i = 0; i < v->n; i++) {
            const dp_state *s = &v->v[i];
            size_t h = (size_t)(mix64(dp_hash(s)) & (cap - 1));
            for (;;) {
                if (!occ[h]) {
                    occ[h] = 1;
                    tab[h] = *s;
                    break;
                }
                if (tab[h].open == s->open && tab[h].used == s->used) {
                    tab[h].cnt += s->cnt;
                    break;
                }
                h = (h + 1) & (cap - 1);
            }
        }
        v->n = 0;
    }
    for (size_t h = 0; h < cap; h++)
        if (occ[h])
            vec_push(out, &tab[h]);
    free(tab);
    free(occ);
    return NULL;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Placements anchored at (row 0, col) of the W-stride board, anchor = the
 * placement's lowest cell (the order of Piece::cover's anchors,
 * src/Piece.inl:5-24); each carries its type's copy bits. */
static void dp_build_tab(const or_ctx *cp, dp_tab *tp)
{
    const or_ctx c = *cp;
    memset(tp, 0, sizeof(*tp));
    tp->W = c.W;
    tp->H = c.H;
    tp->board = c.board;
    int base = 0;
    for (int i = 0; i < c.n; i++) {
        const or_piece *pc = &c.lib[i];
        uint64_t tm = pc->count ? (((pc->count >= 64) ? ~0ull : ((1ull << pc->count) - 1)) << base) : 0;
        base += (int)pc->count;
        for (int t = 0; t < pc->nplc; t++) {
            const or_plc *pl = &pc->plc[t];
            if (!pl->enabled || !tm)
                continue;
            for (int col = 0; col < c.W; col++) {
                int x = col - pl->cc[0];
                if (x < 0 || x + pl->w > c.W || pl->h > c.H)
                    continue;
                u128 m = plc_mask(&c, pl, 0, x);
                tp->plc[col] = (dp_plc *)realloc(tp->plc[col], (size_t)(tp->nplc[col] + 1) * sizeof(dp_plc));
                dp_plc *d = &tp->plc[col][tp->nplc[col]++];
                d->rel = (uint64_t)m;
                d->rel_hi = (uint64_t)(m >> 64);
                d->tmask = tm;
                d->h = pl->h;
            }
        }
    }
}

int32_t or_rowdp(const or_problem *p, int32_t threads, double max_seconds,
                 uint64_t max_children, uint64_t *level_sizes, uint64_t *count,
                 int32_t *levels_done, uint64_t *states_total)
{
    or_ctx c;
    if (build_ctx(p, &c))
        return -1;
    if (threads < 1)
        threads = 1;
    int copies = 0;
    for (int i = 0; i < c.n; i++)
        copies += (int)c.lib[i].count;
    if (copies > OR_MAX_COPIES) {
        free(c.lib);
        return -1;
    }
    dp_tab tab;
    dp_build_tab(&c, &tab);
    int T = threads;
    dp_vec cur = { 0, 0, 0 };
    dp_state root = { c.board, 0, 1 };
    vec_push(&cur, &root);
    dp_vec **shards = (dp_vec **)calloc((size_t)T, sizeof(dp_vec *));
    for (int w = 0; w < T; w++)
        shards[w] = (dp_vec *)calloc((size_t)T, sizeof(dp_vec));
    dp_vec *outs = (dp_vec *)calloc((size_t)T, sizeof(dp_vec));
    dp_job *jobs = (dp_job *)calloc((size_t)T, sizeof(dp_job));
    pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
    double t0 = now_s();
    uint64_t tot = 0;
    int done = 0;
    volatile int abort_flag = 0;
    for (int r = 0; r < c.H; r++) {
        for (int w = 0; w < T; w++) {
            jobs[w].tab = &tab;
            jobs[w].row = r;
            jobs[w].T = T;
            jobs[w].id = w;
            jobs[w].in = cur.v;
            jobs[w].lo = cur.n * (size_t)w / (size_t)T;
            jobs[w].hi = cur.n * (size_t)(w + 1) / (size_t)T;
            jobs[w].shards = shards;
            jobs[w].out = outs;
            jobs[w].limit = max_children ? (max_children + (uint64_t)T - 1) / (uint64_t)T : 0;
            jobs[w].abort = &abort_flag;
            jobs[w].deadline = max_seconds > 0 ? t0 + max_seconds : 0;
        }
        const size_t jobs_in = cur.n;
        if (T == 1)
            dp_expand_worker(&jobs[0]);
        else {
            for (int w = 0; w < T; w++)
                pthread_create(&th[w], NULL, dp_expand_worker, &jobs[w]);
            for (int w = 0; w < T; w++)
                pthread_join(th[w], NULL);
        }
        if (abort_flag) {
            /* Interrupted level.  Count the states expanded and drop their
             * children; with time left (the memory cap stopped it), keep
             * sampling the rest of the level in batches small enough for the
             * cap, each expanded and de-duplicated, until the deadline. */
            size_t pos = 0;
            for (int w = 0; w < T; w++) {
                tot += jobs[w].expanded;
                for (int s = 0; s < T; s++)
                    shards[w][s].n = 0;
            }
            for (int w = 0; w < T; w++)
                pos += jobs[w].expanded;
            size_t batch = pos / 4 + (size_t)T;
            while (max_seconds > 0 && now_s() < t0 + max_seconds && batch) {
                abort_flag = 0;
                size_t lo = pos % cur.n, hi = lo + batch < cur.n ? lo + batch : cur.n;
                for (int w = 0; w < T; w++) {
                    jobs[w].lo = lo + (hi - lo) * (size_t)w / (size_t)T;
                    jobs[w].hi = lo + (hi - lo) * (size_t)(w + 1) / (size_t)T;
                }
                for (int w = 0; w < T; w++)
                    pthread_create(&th[w], NULL, dp_expand_worker, &jobs[w]);
                for (int w = 0; w < T; w++)
                    pthread_join(th[w], NULL);
                size_t got = 0;
                for (int w = 0; w < T; w++)
                    got += jobs[w].expanded;
                if (!abort_flag) {
                    for (int w = 0; w < T; w++)
                        pthread_create(&th[w], NULL, dp_merge_worker, &jobs[w]);
                    for (int w = 0; w < T; w++)
                        pthread_join(th[w], NULL);
                } else {
                    batch /= 2;
                }
                for (int w = 0; w < T; w++)
                    for (int s = 0; s < T; s++)
                        shards[w][s].n = 0;
                tot += got;
                pos = hi;
            }
            break;
        }
        if (T == 1)
            dp_merge_worker(&jobs[0]);
        else {
            for (int w = 0; w < T; w++)
                pthread_create(&th[w], NULL, dp_merge_worker, &jobs[w]);
            for (int w = 0; w < T; w++)
                pthread_join(th[w], NULL);
        }
        cur.n = 0;
        for (int w = 0; w < T; w++)
            for (size_t i = 0; i < outs[w].n; i++)
                vec_push(&cur, &outs[w].v[i]);
        if (level_sizes)
            level_sizes[r] = cur.n;
        tot += jobs_in;
        done = r + 1;
        if (max_seconds > 0 && now_s() - t0 > max_seconds)
            break;
    }
    uint64_t cnt = 0;
    if (done == c.H)
        for (size_t i = 0; i < cur.n; i++)
            cnt += cur.v[i].cnt;
    if (count)
        *count = cnt;
    if (levels_done)
        *levels_done = done;
    if (states_total)
        *states_total = tot;
    for (int w = 0; w < T; w++) {
        for (int s = 0; s < T; s++)
            free(shards[w][s].v);
        free(shards[w]);
        free(outs[w].v);
    }
    free(shards);
    free(outs);
    free(jobs);
    free(th);
    free(cur.v);
    for (int col = 0; col < 11; col++)
        free(tab.plc[col]);
    free(c.lib);
    return 0;
}

/* ------------------------------------------------------------------------
 * Memory-lean exact row DP: the same levels, whole-row fills and
 * de-duplication as or_rowdp (src/searcher_cuda.cu:32-82,
 * src/kernel.cuh:12-49), but children go straight into hash shards (one lock
 * each, filled through small per-thread buffers) instead of being stored
 * before a merge, so memory holds the distinct states only.
 * ---------------------------------------------------------------------- */
#define LEAN_SHARD_BITS 12
#define LEAN_SHARDS (1u << LEAN_SHARD_BITS)
#define LEAN_BUF 16

typedef struct {
    pthread_mutex_t mu;
    dp_state *tab; /* cnt == 0: empty slot (every state reaches here with cnt >= 1) */
    size_t cap, n;
} lean_shard;

typedef struct {
    const dp_tab *tab;
    int row;
    const dp_state *in;
    size_t n_in;
    size_t *next;       /* shared work cursor (chunks of parents) */
    lean_shard *shards;
    dp_state *buf;      /* LEAN_SHARDS x LEAN_BUF */
    uint8_t *bufn;
    uint64_t cnt;       /* multiplicity of the parent being expanded */
    uint64_t raw;       /* children produced */
} lean_worker;

static void lean_shard_put(lean_shard *sh, const dp_state *s, uint64_t h)
{
    size_t i = (size_t)h & (sh->cap - 1);
    for (;;) {
        dp_state *t = &sh->tab[i];
        if (!t->cnt) {
            *t = *s;
            sh->n++;
            return;
        }
        if (t->open == s->open && t->used == s->used) {
            t->cnt += s->cnt;
            return;
        }
        i = (i + 1) & (sh->cap - 1);
    }
}

static void lean_shard_grow(lean_shard *sh)
{
    size_t oc = sh->cap;
    dp_state *old = sh->tab;
    sh->cap = oc ? oc * 2 : 1024;
    sh->tab = (dp_state *)calloc(sh->cap, sizeof(dp_state));
    sh->n = 0;
    for (size_t i = 0; i < oc; i++)
        if (old[i].cnt)
            lean_shard_put(sh, &old[i], dp_hash(&old[i]));
    free(old);
}

static void lean_flush(lean_worker *w, uint32_t b)
{
    lean_shard *sh = &w->shards[b];
    pthread_mutex_lock(&sh->mu);
    if ((sh->n + w->bufn[b]) * 10 > sh->cap * 6)
        lean_shard_grow(sh);
    for (uint32_t k = 0; k < w->bufn[b]; k++) {
        const dp_state *s = &w->buf[(size_t)b * LEAN_BUF + k];
        lean_shard_put(sh, s, dp_hash(s));
    }
    pthread_mutex_unlock(&sh->mu);
    w->bufn[b] = 0;
}

/* dp_fill with the child sent to its shard's buffer. */
static void lean_fill(lean_worker *w, u128 open, uint64_t used)
{
    const dp_tab *t = w->tab;
    int W = t->W;
    u128 rowm = (((u128)1 << W) - 1) << (w->row * W);
    if (!(open & rowm)) {
        dp_state s = { open, used, w->cnt };
        uint32_t b = (uint32_t)(dp_hash(&s) >> (64 - LEAN_SHARD_BITS));
        w->buf[(size_t)b * LEAN_BUF + w->bufn[b]++] = s;
        if (w->bufn[b] == LEAN_BUF)
            lean_flush(w, b);
        w->raw++;
        return;
    }
    int pos = ctz128(open);
    int col = pos % W;
    for (int i = 0; i < t->nplc[col]; i++) {
        const dp_plc *pl = &t->plc[col][i];
        if (w->row + pl->h > t->H)
            continue;
        u128 m = (((u128)pl->rel_hi << 64) | pl->rel) << (w->row * W);
        if (m & ~open)
            continue;
        uint64_t tm = pl->tmask;
        uint64_t nb = ((used & tm) + (tm & (~tm + 1))) & tm;
        if (!nb)
            continue;
        lean_fill(w, open & ~m, used | nb);
    }
}

static void *lean_worker_run(void *arg)
{
    lean_worker *w = (lean_worker *)arg;
    const size_t chunk = 4096;
    for (;;) {
        size_t lo = __atomic_fetch_add(w->next, chunk, __ATOMIC_RELAXED);
        if (lo >= w->n_in)
            break;
        size_t hi = lo + chunk < w->n_in ? lo + chunk : w->n_in;
        for (size_t i = lo; i < hi; i++) {
            w->cnt = w->in[i].cnt;
            lean_fill(w, w->in[i].open, w->in[i].used);
        }
    }
    for (uint32_t b = 0; b < LEAN_SHARDS; b++)
        if (w->bufn[b])
            lean_flush(w, b);
    return NULL;
}

typedef struct {
    lean_shard *shards;
    uint32_t lo, hi;
    const size_t *offs;
    dp_state *out;
} lean_collect_job;

static void *lean_collect_run(void *arg)
{
    lean_collect_job *j = (lean_collect_job *)arg;
    for (uint32_t b = j->lo; b < j->hi; b++) {
        lean_shard *sh = &j->shards[b];
        dp_state *o = j->out + j->offs[b];
        for (size_t i = 0; i < sh->cap; i++)
            if (sh->tab[i].cnt)
                *o++ = sh->tab[i];
        free(sh->tab);
        sh->tab = NULL;
        sh->cap = sh->n = 0;
    }
    return NULL;
}

int32_t or_rowdp_lean(const or_problem *p, int32_t threads, int32_t max_rows,
                      uint64_t *level_sizes, uint64_t *raw_sizes, uint64_t *count,
                      double *seconds)
{
    or_ctx c;
    if (build_ctx(p, &c))
        return -1;
    if (threads < 1)
        threads = 1;
    int copies = 0;
    for (int i = 0; i < c.n; i++)
        copies += (int)c.lib[i].count;
    if (copies > OR_MAX_COPIES) {
        free(c.lib);
        return -1;
    }
    dp_tab tab;
    dp_build_tab(&c, &tab);
    const double t0 = now_s();
    const int T = threads;
    lean_shard *shards = (lean_shard *)calloc(LEAN_SHARDS, sizeof(lean_shard));
    for (uint32_t b = 0; b < LEAN_SHARDS; b++)
        pthread_mutex_init(&shards[b].mu, NULL);
    lean_worker *ws = (lean_worker *)calloc((size_t)T, sizeof(lean_worker));
    for (int k = 0; k < T; k++) {
        ws[k].buf = (dp_state *)malloc((size_t)LEAN_SHARDS * LEAN_BUF * sizeof(dp_state));
        ws[k].bufn = (uint8_t *)calloc(LEAN_SHARDS, 1);
    }
    pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
    size_t n_cur = 1;
    dp_state *cur = (dp_state *)malloc(sizeof(dp_state));
    cur[0].open = c.board;
    cur[0].used = 0;
    cur[0].cnt = 1;
    int32_t rc = 0;
    const int rows = (max_rows > 0 && max_rows < c.H) ? max_rows : c.H;
    for (int r = 0; r < rows; r++) {
        size_t next = 0;
        for (int k = 0; k < T; k++) {
            ws[k].tab = &tab;
            ws[k].row = r;
            ws[k].in = cur;
            ws[k].n_in = n_cur;
            ws[k].next = &next;
            ws[k].shards = shards;
            ws[k].raw = 0;
            pthread_create(&th[k], NULL, lean_worker_run, &ws[k]);
        }
        uint64_t raw = 0;
        for (int k = 0; k < T; k++) {
            pthread_join(th[k], NULL);
            raw += ws[k].raw;
        }
        free(cur);
        size_t *offs = (size_t *)calloc(LEAN_SHARDS + 1, sizeof(size_t));
        for (uint32_t b = 0; b < LEAN_SHARDS; b++)
            offs[b + 1] = offs[b] + shards[b].n;
        n_cur = offs[LEAN_SHARDS];
        cur = (dp_state *)malloc((n_cur ? n_cur : 1) * sizeof(dp_state));
        if (!cur) {
            rc = -2;
            free(offs);
            break;
        }
        lean_collect_job *jobs = (lean_collect_job *)calloc((size_t)T, sizeof(lean_collect_job));
        for (int k = 0; k < T; k++) {
            jobs[k].shards = shards;
            jobs[k].lo = (uint32_t)((uint64_t)LEAN_SHARDS * (uint64_t)k / (uint64_t)T);
            jobs[k].hi = (uint32_t)((uint64_t)LEAN_SHARDS * (uint64_t)(k + 1) / (uint64_t)T);
            jobs[k].offs = offs;
            jobs[k].out = cur;
            pthread_create(&th[k], NULL, lean_collect_run, &jobs[k]);
        }
        for (int k = 0; k < T; k++)
            pthread_join(th[k], NULL);
        free(jobs);
        free(offs);
        if (level_sizes)
            level_sizes[r] = n_cur;
        if (raw_sizes)
            raw_sizes[r] = raw;
    }
    uint64_t cnt = 0;
    if (rc == 0 && rows == c.H)
        for (size_t i = 0; i < n_cur; i++)
            cnt += cur[i].cnt;
    if (count)
        *count = cnt;
    if (seconds)
        *seconds = now_s() - t0;
    free(cur);
    for (int k = 0; k < T; k++) {
        free(ws[k].buf);
        free(ws[k].bufn);
    }
    free(ws);
    free(th);
    for (uint32_t b = 0; b < LEAN_SHARDS; b++) {
        pthread_mutex_destroy(&shards[b].mu);
        free(shards[b].tab);
    }
    free(shards);
    for (int col = 0; col < 11; col++)
        free(tab.plc[col]);
    free(c.lib);
    return rc;
}

/* ------------------------------------------------------------------------
 * Independent cover check (used for solve-one answers).
 * ---------------------------------------------------------------------- */
int32_t or_check_tiling(const or_problem *p, int32_t n, const int32_t *types,
                        const uint64_t *mask_lo, const uint64_t *mask_hi)
{
    or_ctx c;
    if (build_ctx(p, &c))
        return 0;
    uint32_t used[OR_MAX_TYPES];
    memset(used, 0, sizeof(used));
    u128 acc = 0;
    int ok = 1;
    for (int i = 0; i < n && ok; i++) {
        int t = types[i];
        u128 m = ((u128)mask_hi[i] << 64) | mask_lo[i];
        if (t < 0 || t >= c.n || !m || (m & acc)) {
            ok = 0;
            break;
        }
        acc |= m;
        if (++used[t] > c.lib[t].count) {
            ok = 0;
            break;
        }
        int minr = 1 << 30, minc = 1 << 30;
        for (int b = 0; b < c.W * c.H; b++)
            if ((m >> b) & 1u) {
                if (b / c.W < minr)
                    minr = b / c.W;
                if (b % c.W < minc)
                    minc = b % c.W;
            }
        uint64_t v = 0;
        for (int b = 0; b < c.W * c.H && ok; b++)
            if ((m >> b) & 1u) {
                int r = b / c.W - minr, x = b % c.W - minc;
                if (r >= 8 || x >= 8)
                    ok = 0;
                else
                    v |= 1ull << (r * 8 + x);
            }
        if (!ok)
            break;
        int match = 0;
        for (int k = 0; k < c.lib[t].nplc; k++)
            if (c.lib[t].plc[k].normal == v)
                match = 1;
        if (!match)
            ok = 0;
    }
    if (ok && acc != c.board)
        ok = 0;
    free(c.lib);
    return ok;
}
