// server.cu -- serving loop: continuous batching of tiling requests on one GPU.
//
// A native worker thread owns two engines (packed 64-bit keys for requests
// that fit them, the general 128-bit encoding for the rest).  Each loop
// iteration admits queued requests in arrival order while the projected
// device bytes of everything admitted stay within the budget, then advances
// every admitted request by one board row (one k_expand + k_compact pair per
// engine for all of them), then hands out the requests that finished.  A
// request that arrives while others run joins at their next row.
//
// No counterpart in the reference: its SearcherFactory (src/searcher.cpp:86-107)
// runs a fixed job list, one CudaSearcher per job.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/d4e.h"
#include "abi_util.h"
#include "engine.h"

namespace d4e {

void engine_result(Engine &eng, uint32_t id, uint32_t mode, d4e_result *r);

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Instance ids of the packed-key engine: 14 bits, so up to 16384 requests
// on the device at once; requests whose window and counter bits exceed 49
// use the general engine.
constexpr uint32_t kServerIdBits = 14;

struct Request {
    uint32_t width = 0, height = 0, n_pieces = 0, sym = 0, mode = 0;
    std::vector<uint8_t> rows;
    std::vector<uint64_t> shapes;
    std::vector<uint32_t> counts;
    uint64_t tag = 0;
    Clock::time_point t_submit, t_admit;
    double projected = 0;   // bytes charged against the budget at admission
};

}  // namespace

class Server {
public:
    explicit Server(const d4e_server_opts &o) : opts_(o) {
        if (!opts_.max_active)
            opts_.max_active = 8192;
        opts_.max_active = std::min<uint32_t>(opts_.max_active, 1u << kServerIdBits);
        int n = 0;
        cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (opts_.device < 0 || opts_.device >= n)
            throw Error(kErrInvalid, "no such CUDA device");
        cuda_check(cudaSetDevice(opts_.device), "cudaSetDevice");
        size_t free_b = 0, total_b = 0;
        cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
        const uint64_t cap = (uint64_t)((double)total_b * 0.9);
        budget_ = opts_.memory_budget ? opts_.memory_budget
                                      : std::min<uint64_t>(150ull << 30, cap);
        EngineOpts eo;
        eo.device = opts_.device;
        eo.isolate_failures = true;
        eo.memory_budget = budget_;
        EngineOpts e64 = eo;
        e64.k64_inst_bits = kServerIdBits;
        eng_[0] = std::make_unique<Engine>(e64);
        EngineOpts e128 = eo;
        e128.key_mode = KeyMode::K128;
        eng_[1] = std::make_unique<Engine>(e128);
        worker_ = std::thread([this] { loop(); });
    }

    ~Server() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        if (worker_.joinable())
            worker_.join();
    }

    void submit(const d4e_instance &in, uint32_t mode, uint64_t tag) {
        if (mode > D4E_MODE_SOLVE_ONE)
            throw Error(kErrInvalid, "unknown mode");
        if (in.width < 1 || in.width > 8 || in.height < 1 || in.height > 64)
            throw Error(kErrInvalid, "board size out of range");
        if (!in.rows || (in.n_pieces && (!in.shapes || !in.counts)))
            throw Error(kErrInvalid, "null pointer in instance");
        if (mode == D4E_MODE_SOLVE_ONE && in.width * in.height > 512)
            throw Error(kErrInvalid, "solve-one boards are limited to 512 cells");
        Request r;
        r.width = in.width;
        r.height = in.height;
        r.n_pieces = in.n_pieces;
        r.sym = in.sym;
        r.mode = mode;
        r.rows.assign(in.rows, in.rows + in.height);
        r.shapes.assign(in.shapes, in.shapes + in.n_pieces);
        r.counts.assign(in.counts, in.counts + in.n_pieces);
        r.tag = tag;
        r.t_submit = Clock::now();
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (worker_error_)
                throw Error(worker_code_, worker_msg_);
            queue_.push_back(std::move(r));
            st_.submitted++;
        }
        cv_.notify_all();
    }

    uint32_t poll(d4e_result *out, uint32_t max) {
        std::lock_guard<std::mutex> lk(mu_);
        const uint32_t n = (uint32_t)std::min<size_t>(max, results_.size());
        for (uint32_t i = 0; i < n; i++) {
            out[i] = results_.front();
            results_.pop_front();
        }
        return n;
    }

    bool drain(double timeout_s) {
        std::unique_lock<std::mutex> lk(mu_);
        const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                                 std::chrono::duration<double>(timeout_s));
        while (st_.completed + st_.failed < st_.submitted && !worker_error_) {
            if (done_cv_.wait_until(lk, deadline) == std::cv_status::timeout)
                return false;
        }
        if (worker_error_)
            throw Error(worker_code_, worker_msg_);
        return true;
    }

    d4e_server_stats stats() {
        std::lock_guard<std::mutex> lk(mu_);
        return st_;
    }

private:
    // Bytes a running request is expected to hold on its next row.
    double running_projection(int e, uint32_t id) const {
        return (double)eng_[e]->projected_bytes(id);
    }

    // Bytes charged for a request not yet started: solve-one requests are
    // bounded by their sample width; counting requests are charged the
    // average peak of the counting requests finished so far.
    double initial_projection(const Request &r) const {
        const double per_state = 16.0 + 16.0 / 0.5;   // record + table slot at load 0.5
        const double floor_b = 1.0 * 1024 * 1024;
        if (r.mode == D4E_MODE_SOLVE_ONE && opts_.beam)
            return std::max(floor_b, (double)opts_.beam * 64.0 * per_state);
        return std::max(floor_b, avg_peak_bytes_);
    }

    void loop() {
        try {
            cuda_check(cudaSetDevice(opts_.device), "cudaSetDevice");
            for (;;) {
                admit();
                bool busy = false;
                for (int e = 0; e < 2; e++) {
                    if (!eng_[e]->has_active())
                        continue;
                    busy = true;
                    const auto t0 = Clock::now();
                    const StepStats s = eng_[e]->step();
                    const auto t1 = Clock::now();
                    collect(e);
                    std::lock_guard<std::mutex> lk(mu_);
                    st_.steps++;
                    st_.states_out += s.n_out;
                    st_.busy_ms += ms_between(t0, t1);
                }
                if (!busy) {
                    std::unique_lock<std::mutex> lk(mu_);
                    if (stop_)
                        return;
                    if (queue_.empty())
                        cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
                    if (stop_)
                        return;
                } else {
                    std::lock_guard<std::mutex> lk(mu_);
                    if (stop_)
                        return;
                }
            }
        } catch (const Error &e) {
            std::lock_guard<std::mutex> lk(mu_);
            worker_error_ = true;
            worker_code_ = e.code;
            worker_msg_ = e.what();
        } catch (const std::exception &e) {
            std::lock_guard<std::mutex> lk(mu_);
            worker_error_ = true;
            worker_code_ = kErrInvalid;
            worker_msg_ = e.what();
        }
        done_cv_.notify_all();
    }

    // Admission: arrival order, while the projected bytes of the running
    // requests plus the candidate fit the budget (the first request always
    // fits) and fewer than max_active run.
    void admit() {
        std::deque<Request> take;
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (queue_.empty())
                return;
            double proj = 0;
            for (int e = 0; e < 2; e++)
                for (const auto &[id, r] : running_[e])
                    proj += running_projection(e, id);
            size_t active = running_[0].size() + running_[1].size();
            while (!queue_.empty() && active < opts_.max_active) {
                const double p = initial_projection(queue_.front());
                if (active > 0 && proj + p > (double)budget_)
                    break;
                take.push_back(std::move(queue_.front()));
                take.back().projected = p;
                queue_.pop_front();
                proj += p;
                active++;
            }
            st_.peak_projected = std::max<uint64_t>(st_.peak_projected, (uint64_t)proj);
        }
        for (Request &r : take) {
            r.t_admit = Clock::now();
            d4e_instance in{};
            in.width = r.width;
            in.height = r.height;
            in.rows = r.rows.data();
            in.n_pieces = r.n_pieces;
            in.shapes = r.shapes.data();
            in.counts = r.counts.data();
            in.sym = r.sym;
            InstanceSpec sp;
            sp.width = in.width;
            sp.height = in.height;
            sp.rows = in.rows;
            sp.shapes = in.shapes;
            sp.counts = in.counts;
            sp.n_pieces = in.n_pieces;
            sp.sym = in.sym;
            sp.mode = r.mode == D4E_MODE_SOLVE_ONE ? Mode::SolveOne : Mode::Count;
            sp.max_states = opts_.max_states;
            sp.beam = opts_.beam;
            int e = 0;
            uint32_t id = 0;
            try {
                try {
                    id = eng_[0]->add(sp);
                } catch (const Error &err) {
                    if (err.code != kErrUnsupported ||
                        std::string(err.what()).find("packed key") == std::string::npos)
                        throw;
                    e = 1;
                    id = eng_[1]->add(sp);
                }
            } catch (const Error &err) {
                // Invalid or unsupported request: it fails on its own.
                d4e_result res{};
                res.tag = r.tag;
                res.status = err.code;
                res.mode = r.mode;
                std::memset(res.grid, -1, sizeof(res.grid));
                std::memset(res.steps, -1, sizeof(res.steps));
                res.queued_ms = ms_between(r.t_submit, r.t_admit);
                res.latency_ms = res.queued_ms;
                std::lock_guard<std::mutex> lk(mu_);
                results_.push_back(res);
                st_.failed++;
                done_cv_.notify_all();
                continue;
            }
            std::lock_guard<std::mutex> lk(mu_);
            running_[e].emplace(id, std::move(r));
            st_.admitted++;
            st_.peak_active = std::max<uint64_t>(st_.peak_active,
                                                 running_[0].size() + running_[1].size());
        }
    }

    void collect(int e) {
        Engine &eng = *eng_[e];
        std::vector<uint32_t> fin;
        for (const auto &[id, r] : running_[e])
            if (eng.done(id))
                fin.push_back(id);
        if (fin.empty())
            return;
        eng.sync_results();
        const auto now = Clock::now();
        std::vector<d4e_result> out(fin.size());
        for (size_t k = 0; k < fin.size(); k++) {
            const uint32_t id = fin[k];
            const Request &r = running_[e].at(id);
            d4e_result &res = out[k];
            engine_result(eng, id, r.mode, &res);
            res.tag = r.tag;
            res.queued_ms = ms_between(r.t_submit, r.t_admit);
            res.latency_ms = ms_between(r.t_submit, now);
            if (r.mode == D4E_MODE_COUNT && res.status == 0) {
                const double peak = (double)eng.peak_bytes(id);
                avg_peak_bytes_ = n_peaks_ ? 0.95 * avg_peak_bytes_ + 0.05 * peak : peak;
                n_peaks_++;
            }
            eng.release(id);
        }
        std::lock_guard<std::mutex> lk(mu_);
        for (size_t k = 0; k < fin.size(); k++) {
            running_[e].erase(fin[k]);
            results_.push_back(out[k]);
            if (out[k].status)
                st_.failed++;
            else
                st_.completed++;
        }
        done_cv_.notify_all();
    }

    d4e_server_opts opts_;
    uint64_t budget_ = 0;
    std::unique_ptr<Engine> eng_[2];
    std::thread worker_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<Request> queue_;
    std::unordered_map<uint32_t, Request> running_[2];   // by engine instance id
    std::deque<d4e_result> results_;
    d4e_server_stats st_{};
    double avg_peak_bytes_ = 0;
    uint64_t n_peaks_ = 0;
    bool stop_ = false;
    bool worker_error_ = false;
    int worker_code_ = 0;
    std::string worker_msg_;
};

}  // namespace d4e

struct d4e_server {
    std::unique_ptr<d4e::Server> srv;
};

extern "C" {

int d4e_server_create(const d4e_server_opts *opts, d4e_server **out) {
    return d4e::abi_guarded([&] {
        if (!out)
            return d4e::abi_fail(D4E_ERR_INVALID, "null pointer");
        *out = nullptr;
        const d4e_server_opts o = opts ? *opts : d4e_server_opts{};
        auto s = std::make_unique<d4e_server>();
        s->srv = std::make_unique<d4e::Server>(o);
        *out = s.release();
        return D4E_OK;
    });
}

int d4e_server_submit(d4e_server *s, const d4e_instance *inst, uint32_t mode, uint64_t tag) {
    return d4e::abi_guarded([&] {
        if (!s || !inst)
            return d4e::abi_fail(D4E_ERR_INVALID, "null pointer");
        s->srv->submit(*inst, mode, tag);
        return D4E_OK;
    });
}

int d4e_server_poll(d4e_server *s, d4e_result *out, uint32_t max, uint32_t *n) {
    return d4e::abi_guarded([&] {
        if (!s || !n || (!out && max))
            return d4e::abi_fail(D4E_ERR_INVALID, "null pointer");
        *n = s->srv->poll(out, max);
        return D4E_OK;
    });
}

int d4e_server_drain(d4e_server *s, double timeout_s) {
    return d4e::abi_guarded([&] {
        if (!s)
            return d4e::abi_fail(D4E_ERR_INVALID, "null pointer");
        if (!s->srv->drain(timeout_s))
            return d4e::abi_fail(D4E_ERR_STATE, "drain timed out");
        return D4E_OK;
    });
}

int d4e_server_stats_get(d4e_server *s, d4e_server_stats *st) {
    return d4e::abi_guarded([&] {
        if (!s || !st)
            return d4e::abi_fail(D4E_ERR_INVALID, "null pointer");
        *st = s->srv->stats();
        return D4E_OK;
    });
}

void d4e_server_destroy(d4e_server *s) { delete s; }

}  // extern "C"
