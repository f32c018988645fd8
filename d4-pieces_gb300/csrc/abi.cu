// abi.cu -- extern "C" boundary (include/d4e.h) over the engine.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/d4e.h"
#include "abi_util.h"
#include "engine.h"
#include "kernels.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

template <class F>
int guarded(F &&f) {
    try {
        g_err.clear();
        return f();
    } catch (const d4e::Error &e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc &) {
        return fail(D4E_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(D4E_ERR_INVALID, e.what());
    }
}

}  // namespace

namespace d4e {

int abi_fail(int code, const std::string &msg) { return fail(code, msg); }

void abi_clear_error() { g_err.clear(); }

}  // namespace d4e

struct d4e_frow {
    std::vector<uint64_t> shapes;
    std::vector<uint32_t> counts;
    uint32_t sym = 0xFF;
    uint32_t width = 8;
    d4e::PieceLib lib;
    int device = -1;
};

struct d4e_searcher {
    std::unique_ptr<d4e::Engine> eng;
    uint32_t id = 0;
    uint32_t width = 8, height = 0;
    std::vector<uint8_t> rows;
};

extern "C" {

const char *d4e_last_error(void) { return g_err.c_str(); }

const char *d4e_version(void) { return "d4e 0.1 (sm_103a)"; }

int d4e_device_count(int32_t *n) {
    return guarded([&] {
        if (!n)
            return fail(D4E_ERR_INVALID, "null pointer");
        int c = 0;
        if (cudaGetDeviceCount(&c) != cudaSuccess) {
            cudaGetLastError();
            c = 0;
        }
        *n = c;
        return D4E_OK;
    });
}

int d4e_show_gpu_devices(void) {
    return guarded([&] {
        int n = 0;
        d4e::cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        std::printf("Number of devices: %d\n", n);
        for (int i = 0; i < n; i++) {
            cudaDeviceProp p;
            d4e::cuda_check(cudaGetDeviceProperties(&p, i), "cudaGetDeviceProperties");
            std::printf("Device Number: %d\n", i);
            std::printf("  Device name: %s\n", p.name);
            std::printf("  Capability: %d.%d\n", p.major, p.minor);
            std::printf("  MP: %d\n", p.multiProcessorCount);
            std::printf("  Memory Bus Width (bits): %d\n", p.memoryBusWidth);
            std::printf("  Global mem (MiB): %.1f\n", p.totalGlobalMem / 1048576.0);
            std::printf("  L2 Cache Size (B): %d\n", p.l2CacheSize);
            std::printf("  Shared mem per block optin (B): %zu\n", p.sharedMemPerBlockOptin);
            std::printf("  Shared mem per mp (B): %zu\n", p.sharedMemPerMultiprocessor);
            std::printf("  Threads/mp: %d\n", p.maxThreadsPerMultiProcessor);
            std::printf("  Registers per mp: %d\n", p.regsPerMultiprocessor);
        }
        return D4E_OK;
    });
}

int d4e_catalogue(uint32_t m, int32_t onesided, uint64_t *out, uint32_t max, uint32_t *n) {
    return guarded([&] {
        if (m < 1 || m > 8)
            return fail(D4E_ERR_INVALID, "catalogue covers 1..8 cells");
        const auto &v = onesided ? d4e::catalogue_onesided((int)m) : d4e::catalogue_free((int)m);
        if (n)
            *n = (uint32_t)v.size();
        for (uint32_t i = 0; out && i < max && i < v.size(); i++)
            out[i] = v[i];
        return D4E_OK;
    });
}

int d4e_frow_create(const uint64_t *shapes, const uint32_t *counts, uint32_t n_pieces,
                    uint32_t sym, uint32_t width, int32_t show_report, d4e_frow **out) {
    return guarded([&] {
        if (!out || (n_pieces && (!shapes || !counts)))
            return fail(D4E_ERR_INVALID, "null pointer");
        auto f = std::make_unique<d4e_frow>();
        f->shapes.assign(shapes, shapes + n_pieces);
        f->counts.assign(counts, counts + n_pieces);
        f->sym = sym;
        f->width = width;
        const std::string err = d4e::build_piece_lib(shapes, counts, n_pieces, sym, width, f->lib);
        if (!err.empty())
            return fail(err.find("more than") != std::string::npos ? D4E_ERR_UNSUPPORTED
                                                                   : D4E_ERR_INVALID,
                        err);
        if (show_report) {
            for (uint32_t c = 0; c < width; c++)
                std::printf("[col %u] => %u placements\n", c, (unsigned)f->lib.col_len[c]);
        }
        *out = f.release();
        return D4E_OK;
    });
}

int d4e_frow_transfer(d4e_frow *f, int32_t device) {
    return guarded([&] {
        if (!f)
            return fail(D4E_ERR_INVALID, "null frow");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
            cudaGetLastError();
            return fail(D4E_ERR_CUDA, "no CUDA device");
        }
        if (device < 0 || device >= n)
            return fail(D4E_ERR_INVALID, "no such CUDA device");
        f->device = device;
        return D4E_OK;
    });
}

int d4e_frow_placements(const d4e_frow *f, uint32_t col, uint32_t *n) {
    return guarded([&] {
        if (!f || !n)
            return fail(D4E_ERR_INVALID, "null pointer");
        if (col >= f->width)
            return fail(D4E_ERR_INVALID, "column out of range");
        *n = f->lib.col_len[col];
        return D4E_OK;
    });
}

void d4e_frow_destroy(d4e_frow *f) { delete f; }

static int make_searcher(const d4e_frow *f, uint32_t height, const uint8_t *rows, uint32_t flags,
                         d4e_searcher **out) {
    if (!f || !out || !rows)
        return fail(D4E_ERR_INVALID, "null pointer");
    if (f->device < 0)
        return fail(D4E_ERR_STATE, "frow tables not transferred to a device");
    auto s = std::make_unique<d4e_searcher>();
    d4e::EngineOpts o;
    o.device = f->device;
    o.keep_levels = (flags & D4E_KEEP_LEVELS) != 0;
    o.autotune = (flags & D4E_AUTOTUNE) != 0;
    if (flags & D4E_DEDUP_DIRECT)
        o.dedup = d4e::EngineOpts::Dedup::Direct;
    if (flags & D4E_DEDUP_PARTITIONED)
        o.dedup = d4e::EngineOpts::Dedup::Partitioned;
    s->eng = std::make_unique<d4e::Engine>(o);
    d4e::InstanceSpec sp;
    sp.width = f->width;
    sp.height = height;
    sp.rows = rows;
    sp.shapes = f->shapes.data();
    sp.counts = f->counts.data();
    sp.n_pieces = (uint32_t)f->shapes.size();
    sp.sym = f->sym;
    s->id = s->eng->add(sp);
    s->width = f->width;
    s->height = height;
    s->rows.assign(rows, rows + height);
    *out = s.release();
    return D4E_OK;
}

int d4e_searcher_create(const d4e_frow *f, uint64_t empty_area, d4e_searcher **out) {
    return guarded([&] {
        if (!f)
            return fail(D4E_ERR_INVALID, "null frow");
        if (f->width != 8)
            return fail(D4E_ERR_INVALID, "empty_area boards are 8 wide");
        // height = ceil(bit_width(empty_area) / 8), src/searcher_cuda.cu:13
        uint32_t bw = 0;
        for (uint64_t v = empty_area; v; v >>= 1)
            bw++;
        const uint32_t h = (bw + 7) / 8;
        if (h == 0)
            return fail(D4E_ERR_INVALID, "empty board");
        uint8_t rows[8];
        for (uint32_t r = 0; r < 8; r++)
            rows[r] = (uint8_t)(empty_area >> (8 * r));
        return make_searcher(f, h, rows, 0, out);
    });
}

int d4e_searcher_create_board(const d4e_frow *f, uint32_t height, const uint8_t *rows,
                              uint32_t flags, d4e_searcher **out) {
    return guarded([&] { return make_searcher(f, height, rows, flags, out); });
}

int d4e_searcher_get_height(const d4e_searcher *s, uint32_t *height) {
    return guarded([&] {
        if (!s || !height)
            return fail(D4E_ERR_INVALID, "null pointer");
        *height = s->height - s->eng->row(s->id);
        if (s->eng->done(s->id))
            *height = 0;
        return D4E_OK;
    });
}

int d4e_searcher_size(const d4e_searcher *s, uint64_t *n) {
    return guarded([&] {
        if (!s || !n)
            return fail(D4E_ERR_INVALID, "null pointer");
        *n = s->eng->done(s->id) ? 0 : std::max<uint64_t>(s->eng->frontier_size(s->id), 1);
        return D4E_OK;
    });
}

int d4e_searcher_bucket_size(d4e_searcher *s, uint32_t bucket, uint64_t *n) {
    return guarded([&] {
        if (!s || !n)
            return fail(D4E_ERR_INVALID, "null pointer");
        if (bucket > 255)
            return fail(D4E_ERR_INVALID, "bucket is an 8-bit row pattern");
        *n = s->eng->bucket_count(s->id, bucket);
        return D4E_OK;
    });
}

int d4e_searcher_next_size(const d4e_searcher *s, uint64_t *n) {
    return guarded([&] {
        if (!s || !n)
            return fail(D4E_ERR_INVALID, "null pointer");
        *n = s->eng->next_size_estimate(s->id);
        return D4E_OK;
    });
}

int d4e_searcher_search_GPU(d4e_searcher *s) {
    return guarded([&] {
        if (!s)
            return fail(D4E_ERR_INVALID, "null searcher");
        if (s->eng->done(s->id))
            return fail(D4E_ERR_STATE, "height is already 0");
        s->eng->step();
        return D4E_OK;
    });
}

int d4e_searcher_run(d4e_searcher *s) {
    return guarded([&] {
        if (!s)
            return fail(D4E_ERR_INVALID, "null searcher");
        s->eng->run();
        return D4E_OK;
    });
}

int d4e_searcher_count(d4e_searcher *s, uint64_t *count) {
    return guarded([&] {
        if (!s || !count)
            return fail(D4E_ERR_INVALID, "null pointer");
        *count = s->eng->count(s->id);
        return D4E_OK;
    });
}

int d4e_searcher_solutions(d4e_searcher *s, uint64_t max, int32_t single, int8_t *type_grids,
                           int8_t *step_grids, uint64_t *n) {
    return guarded([&] {
        if (!s || !n)
            return fail(D4E_ERR_INVALID, "null pointer");
        // Step numbers come as int16 (boards of up to 512 cells); this
        // interface's grids are int8, like the reference's Step::piece_id.
        std::vector<int16_t> steps;
        if (step_grids) {
            const uint64_t cells = (uint64_t)s->eng->width(s->id) * s->eng->height(s->id);
            const bool ok = s->eng->done(s->id) && !s->eng->status(s->id);
            uint64_t rows = std::min<uint64_t>(max, ok ? s->eng->count(s->id) : 0);
            if (single != 0)
                rows = std::min<uint64_t>(rows, 1);
            steps.resize(rows * cells);
        }
        *n = s->eng->solutions(s->id, max, type_grids, step_grids ? steps.data() : nullptr,
                               single != 0);
        if (step_grids) {
            const uint64_t cells = (uint64_t)s->eng->width(s->id) * s->eng->height(s->id);
            for (uint64_t k = 0; k < *n * cells; k++)
                step_grids[k] = (int8_t)steps[k];
        }
        return D4E_OK;
    });
}

int d4e_searcher_level_sizes(const d4e_searcher *s, uint64_t *sizes, uint32_t max, uint32_t *n) {
    return guarded([&] {
        if (!s || !n)
            return fail(D4E_ERR_INVALID, "null pointer");
        const auto &v = s->eng->level_sizes(s->id);
        *n = (uint32_t)v.size();
        for (uint32_t i = 0; sizes && i < max && i < v.size(); i++)
            sizes[i] = v[i];
        return D4E_OK;
    });
}

// Adds an engine's totals to *st (add = false: overwrites).
static void fill_stats(const d4e::Engine &e, d4e_stats *st, bool add = false) {
    const d4e::Totals &t = e.totals();
    if (!add)
        std::memset(st, 0, sizeof(*st));
    st->rows += t.steps;
    st->states_in += t.states_in;
    st->states_raw += t.states_raw;
    st->states_out += t.states_out;
    st->peak_frontier = std::max<uint64_t>(st->peak_frontier, t.peak_frontier);
    st->expand_launches += t.expand_launches;
    st->compact_launches += t.compact_launches;
    st->retries += t.retries;
    st->other_launches += t.other_launches;
    st->h2d_bytes += t.h2d_bytes;
    st->d2h_bytes += t.d2h_bytes;
    st->expand_ms += t.expand_ms;
    st->compact_ms += t.compact_ms;
    st->run_ms += t.run_ms;
    if (!add || !st->record_bytes) {
        st->record_bytes = e.packed_keys() ? 16 : 24;
        st->slot_bytes = e.packed_keys() ? 16 : 32;
    }
    st->paused += t.paused;
    st->splits += t.splits;
    st->failed += t.failed;
    st->restarts += t.restarts;
    st->step_wall_ms += t.step_wall_ms;
    st->upload_ms += t.upload_ms;
    st->keep_ms += t.keep_ms;
    st->trace_ms += t.trace_ms;
    st->tune_ms += t.tune_ms;
    const d4e::Tuning &tu = e.tuning();
    st->tuned_chunk_cap = tu.chunk_cap;
    st->tuned_chunks_per_warp = tu.chunks_per_warp;
    st->tuned_ctas_per_sm = (uint64_t)std::max(tu.ctas_per_sm, 0);
    st->tuned_load = tu.load;
    st->tuned_compact_ctas = (uint64_t)tu.compact_ctas;
    st->tuned_compact_stages = tu.compact_stages;
    st->compact_slots += t.compact_slots;
    const double ph[6] = {t.ph_select_ms, t.ph_table_ms, t.ph_expand_ms, t.ph_post_ms,
                          t.ph_compact_ms, t.ph_tail_ms};
    for (int i = 0; i < 6; i++)
        st->phase_ms[i] += ph[i];
    st->partitioned += t.partitioned;
    st->partition_fallbacks += t.partition_fallbacks;
    st->merge_ms += t.merge_ms;
}

int d4e_searcher_stats(const d4e_searcher *s, d4e_stats *st) {
    return guarded([&] {
        if (!s || !st)
            return fail(D4E_ERR_INVALID, "null pointer");
        fill_stats(*s->eng, st);
        return D4E_OK;
    });
}

int d4e_searcher_set_limit(d4e_searcher *s, uint64_t max_states) {
    return guarded([&] {
        if (!s)
            return fail(D4E_ERR_INVALID, "null searcher");
        s->eng->set_max_frontier(max_states);
        return D4E_OK;
    });
}

void d4e_searcher_destroy(d4e_searcher *s) { delete s; }

int d4e_batch_count(const d4e_instance *insts, uint32_t n, uint32_t flags, int32_t device,
                    uint64_t *counts, d4e_stats *st) {
    return guarded([&] {
        if ((!insts && n) || (!counts && n))
            return fail(D4E_ERR_INVALID, "null pointer");
        d4e::EngineOpts o;
        o.device = device;
        d4e::Engine eng(o);
        auto spec = [&](uint32_t i) {
            d4e::InstanceSpec sp;
            sp.width = insts[i].width;
            sp.height = insts[i].height;
            sp.rows = insts[i].rows;
            sp.shapes = insts[i].shapes;
            sp.counts = insts[i].counts;
            sp.n_pieces = insts[i].n_pieces;
            sp.sym = insts[i].sym;
            return sp;
        };
        if (flags & D4E_BATCH_SEQUENTIAL) {
            for (uint32_t i = 0; i < n; i++) {
                const uint32_t id = eng.add(spec(i));
                eng.run();
                counts[i] = eng.count(id);
            }
        } else {
            std::vector<uint32_t> ids(n);
            for (uint32_t i = 0; i < n; i++)
                ids[i] = eng.add(spec(i));
            eng.run();
            for (uint32_t i = 0; i < n; i++)
                counts[i] = eng.count(ids[i]);
        }
        if (st)
            fill_stats(eng, st);
        return D4E_OK;
    });
}

}  // extern "C"

namespace {

d4e::InstanceSpec to_spec(const d4e_instance &in, uint32_t mode, uint64_t max_states,
                          uint64_t beam) {
    d4e::InstanceSpec sp;
    sp.width = in.width;
    sp.height = in.height;
    sp.rows = in.rows;
    sp.shapes = in.shapes;
    sp.counts = in.counts;
    sp.n_pieces = in.n_pieces;
    sp.sym = in.sym;
    sp.mode = mode == D4E_MODE_SOLVE_ONE ? d4e::Mode::SolveOne
              : mode == D4E_MODE_SETS    ? d4e::Mode::Sets
              : mode == D4E_MODE_LIST    ? d4e::Mode::List
                                         : d4e::Mode::Count;
    sp.max_states = max_states;
    sp.beam = beam;
    return sp;
}

uint32_t id_bits(uint32_t n) {
    uint32_t b = 1;
    while (b < 23 && (1ull << b) < n)
        b++;
    return b;
}

}  // namespace

namespace d4e {

// Result of one finished engine instance.
void engine_result(Engine &eng, uint32_t id, uint32_t mode, d4e_result *r) {
    r->mode = mode;
    r->status = eng.status(id);
    r->rows = eng.row(id);
    r->count = 0;
    r->found = 0;
    std::memset(r->grid, -1, sizeof(r->grid));
    std::memset(r->steps, -1, sizeof(r->steps));
    if (r->status)
        return;
    if (mode == D4E_MODE_SOLVE_ONE) {
        const uint32_t cells = eng.width(id) * eng.height(id);
        if (cells > sizeof(r->grid))
            throw Error(kErrInvalid, "solve-one boards are limited to 512 cells");
        r->found = eng.solution(id, r->grid, r->steps) ? 1u : 0u;
        r->count = r->found;
    } else {
        r->count = eng.count(id);
        if (mode == D4E_MODE_SETS)
            r->found = (uint32_t)eng.sets(id).size();
    }
}

}  // namespace d4e

extern "C" {

void d4e_autotune_clear(void) { d4e::autotune_clear(); }

void d4e_release_cached_memory(void) { d4e::release_idle_pools(); }

}  // extern "C"

namespace {

// Called once per engine of a batch after it ran, before its results are
// taken and its instances released: (engine, [(engine id, instance index)]).
using BatchHook =
    std::function<void(d4e::Engine &, const std::vector<std::pair<uint32_t, uint32_t>> &)>;

// The batch runner behind d4e_batch_run, d4e_batch_sets and
// d4e_batch_solutions; `sets` receives each instance's piece multisets in
// Sets mode, `hook` (list mode) sees each engine's finished instances.
int batch_impl(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *opts,
               d4e_result *results, d4e_stats *st,
               std::vector<d4e::PieceSets> *sets, const BatchHook &hook = nullptr) {
    return guarded([&] {
        if ((!insts && n) || (!results && n))
            return fail(D4E_ERR_INVALID, "null pointer");
        const d4e_batch_opts o = opts ? *opts : d4e_batch_opts{};
        if (o.mode > D4E_MODE_LIST || (o.mode == D4E_MODE_LIST) != (bool)hook)
            return fail(D4E_ERR_INVALID, o.mode == D4E_MODE_LIST
                                             ? "list mode runs through d4e_batch_solutions"
                                             : "unknown mode");
        for (uint32_t i = 0; i < n; i++)
            if (insts[i].width * insts[i].height > sizeof(results[i].grid) &&
                (o.mode == D4E_MODE_SOLVE_ONE || o.mode == D4E_MODE_LIST))
                return fail(D4E_ERR_INVALID, "solve-one and list boards are limited to 512 cells");
        if (sets)
            sets->assign(n, {});
        const auto t0 = std::chrono::steady_clock::now();
        auto finish = [&](d4e::Engine &eng, uint32_t id, uint32_t i) {
            d4e::engine_result(eng, id, o.mode, &results[i]);
            if (sets && results[i].status == 0)
                (*sets)[i] = eng.sets(id);
            results[i].tag = i;
            results[i].queued_ms = 0;
            results[i].latency_ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                    .count();
        };
        d4e::EngineOpts eo;
        eo.device = o.device;
        eo.memory_budget = o.memory_budget;
        eo.isolate_failures = true;
        if (o.flags & D4E_BATCH_WIDE_KEYS)
            eo.key_mode = d4e::KeyMode::K128;
        eo.autotune = (o.flags & D4E_BATCH_AUTOTUNE) != 0;
        if (o.flags & D4E_BATCH_DEDUP_DIRECT)
            eo.dedup = d4e::EngineOpts::Dedup::Direct;
        if (o.flags & D4E_BATCH_DEDUP_PARTITIONED)
            eo.dedup = d4e::EngineOpts::Dedup::Partitioned;
        if (st)
            std::memset(st, 0, sizeof(*st));
        if (o.flags & D4E_BATCH_SEQUENTIAL) {
            d4e::Engine eng(eo);
            for (uint32_t i = 0; i < n; i++) {
                const uint32_t id = eng.add(to_spec(insts[i], o.mode, o.max_states, o.beam));
                eng.run();
                if (hook)
                    hook(eng, {{id, i}});
                finish(eng, id, i);
                eng.release(id);
            }
            if (st)
                fill_stats(eng, st);
            return D4E_OK;
        }
        // Packed 64-bit keys for every instance that fits them, the general
        // encoding for the rest (a second engine, run after the first).
        std::vector<uint32_t> rest;
        if (o.flags & D4E_BATCH_WIDE_KEYS) {
            for (uint32_t i = 0; i < n; i++)
                rest.push_back(i);
        } else {
            d4e::EngineOpts e64 = eo;
            e64.k64_inst_bits = id_bits(n);
            d4e::Engine eng(e64);
            std::vector<std::pair<uint32_t, uint32_t>> ids;   // (engine id, index)
            for (uint32_t i = 0; i < n; i++) {
                try {
                    ids.push_back({eng.add(to_spec(insts[i], o.mode, o.max_states, o.beam)), i});
                } catch (const d4e::Error &err) {
                    if (err.code != d4e::kErrUnsupported ||
                        std::string(err.what()).find("packed key") == std::string::npos)
                        throw;
                    rest.push_back(i);
                }
            }
            eng.run();
            if (hook)
                hook(eng, ids);
            for (const auto &[id, i] : ids)
                finish(eng, id, i);
            if (st)
                fill_stats(eng, st, true);
        }
        if (!rest.empty()) {
            d4e::EngineOpts e128 = eo;
            e128.key_mode = d4e::KeyMode::K128;
            d4e::Engine eng(e128);
            std::vector<uint32_t> ids;
            for (uint32_t i : rest)
                ids.push_back(eng.add(to_spec(insts[i], o.mode, o.max_states, o.beam)));
            eng.run();
            if (hook) {
                std::vector<std::pair<uint32_t, uint32_t>> pairs;
                for (size_t k = 0; k < rest.size(); k++)
                    pairs.push_back({ids[k], rest[k]});
                hook(eng, pairs);
            }
            for (size_t k = 0; k < rest.size(); k++)
                finish(eng, ids[k], rest[k]);
            if (st)
                fill_stats(eng, st, true);
        }
        return D4E_OK;
    });
}

}  // namespace

extern "C" {

int d4e_batch_run(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *opts,
                  d4e_result *results, d4e_stats *st) {
    return batch_impl(insts, n, opts, results, st, nullptr);
}

int d4e_batch_sets(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *opts,
                   d4e_result *results, uint64_t *set_offsets, uint8_t *set_copies,
                   uint64_t *set_tilings, uint64_t max_sets, d4e_stats *st) {
    std::vector<d4e::PieceSets> sets;
    d4e_batch_opts o = opts ? *opts : d4e_batch_opts{};
    o.mode = D4E_MODE_SETS;
    if (n && !set_offsets)
        return fail(D4E_ERR_INVALID, "null pointer");
    for (uint32_t i = 0; i < n; i++)
        if (insts && insts[i].n_pieces > D4E_SET_PIECES)
            return fail(D4E_ERR_INVALID, "piece-set mode takes at most 64 piece types");
    const int rc = batch_impl(insts, n, &o, results, st, &sets);
    if (rc != D4E_OK)
        return rc;
    return guarded([&] {
        uint64_t total = 0;
        for (uint32_t i = 0; i < n; i++) {
            set_offsets[i] = total;
            total += sets[i].size();
        }
        set_offsets[n] = total;
        if (total > max_sets)
            return fail(D4E_ERR_INVALID, "max_sets too small: " + std::to_string(total) +
                                             " piece sets (set_offsets[n])");
        if (total && (!set_copies || !set_tilings))
            return fail(D4E_ERR_INVALID, "null pointer");
        uint64_t k = 0;
        for (uint32_t i = 0; i < n; i++) {
            const d4e::PieceSets &ps = sets[i];
            const size_t nt = std::min<size_t>(ps.n_types, D4E_SET_PIECES);
            for (size_t j = 0; j < ps.size(); j++, k++) {
                std::memset(set_copies + k * D4E_SET_PIECES, 0, D4E_SET_PIECES);
                std::memcpy(set_copies + k * D4E_SET_PIECES, ps.copies.data() + j * ps.n_types,
                            nt);
                set_tilings[k] = ps.tilings[j];
            }
        }
        return D4E_OK;
    });
}

int d4e_batch_solutions(const d4e_instance *insts, uint32_t n, const d4e_batch_opts *opts,
                        uint64_t max_per_instance, d4e_result *results, uint64_t *sol_offsets,
                        int8_t *type_grids, int16_t *step_grids, uint64_t max_total,
                        d4e_stats *st) {
    d4e_batch_opts o = opts ? *opts : d4e_batch_opts{};
    o.mode = D4E_MODE_LIST;
    o.beam = 0;
    if (n && !sol_offsets)
        return fail(D4E_ERR_INVALID, "null pointer");
    // The tilings of each engine's instances are reconstructed together
    // while the engine still holds their rows, into host buffers of
    // D4E_GRID_CELLS cells per tiling.
    std::vector<std::vector<int8_t>> tg(n);
    std::vector<std::vector<int16_t>> sg(n);
    std::vector<uint64_t> got(n, 0);
    const BatchHook hook = [&](d4e::Engine &eng,
                               const std::vector<std::pair<uint32_t, uint32_t>> &ids) {
        std::vector<uint32_t> eids;
        for (const auto &[id, i] : ids)
            eids.push_back(id);
        std::vector<d4e::Engine::TilingList> lists;
        eng.list_solutions(eids, max_per_instance, lists);
        for (size_t q = 0; q < ids.size(); q++) {
            const uint32_t id = ids[q].first, i = ids[q].second;
            const uint64_t cells = (uint64_t)eng.width(id) * eng.height(id);
            const d4e::Engine::TilingList &l = lists[q];
            got[i] = l.n;
            tg[i].assign(l.n * D4E_GRID_CELLS, -1);
            sg[i].assign(l.n * D4E_GRID_CELLS, -1);
            for (uint64_t k = 0; k < l.n; k++) {
                std::memcpy(tg[i].data() + k * D4E_GRID_CELLS, l.types.data() + k * cells, cells);
                std::memcpy(sg[i].data() + k * D4E_GRID_CELLS, l.steps.data() + k * cells,
                            cells * sizeof(int16_t));
            }
        }
    };
    const int rc = batch_impl(insts, n, &o, results, st, nullptr, hook);
    if (rc != D4E_OK)
        return rc;
    return guarded([&] {
        uint64_t total = 0;
        for (uint32_t i = 0; i < n; i++) {
            sol_offsets[i] = total;
            total += got[i];
        }
        sol_offsets[n] = total;
        if (total > max_total)
            return fail(D4E_ERR_INVALID, "max_total too small: " + std::to_string(total) +
                                             " tilings (sol_offsets[n])");
        if (total && (!type_grids || !step_grids))
            return fail(D4E_ERR_INVALID, "null pointer");
        for (uint32_t i = 0; i < n; i++) {
            if (!got[i])
                continue;
            std::memcpy(type_grids + sol_offsets[i] * D4E_GRID_CELLS, tg[i].data(), tg[i].size());
            std::memcpy(step_grids + sol_offsets[i] * D4E_GRID_CELLS, sg[i].data(),
                        sg[i].size() * sizeof(int16_t));
        }
        return D4E_OK;
    });
}

int d4e_canonical_grid(uint32_t width, uint32_t height, const uint8_t *rows, const int8_t *grid,
                       int8_t *out) {
    return guarded([&] {
        if (!rows || !grid || !out)
            return fail(D4E_ERR_INVALID, "null pointer");
        if (width < 1 || width > 8 || height < 1 || height > 64)
            return fail(D4E_ERR_INVALID, "board size out of range");
        d4e::canonical_grid(width, height, rows, grid, out);
        return D4E_OK;
    });
}

}  // extern "C"
