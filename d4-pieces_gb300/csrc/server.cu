// server.cu -- serving loop: continuous batching of tiling requests on one GPU.
//
// Two lanes, each a native worker thread with its own engines (packed 64-bit
// keys for requests that fit them, the general 128-bit encoding for the
// rest) on its own CUDA stream:
//   fast lane -- every request starts here, with a per-row frontier limit
//                of kFastStates; high stream priority.
//   slow lane -- requests whose frontier outgrew the fast lane restart here
//                from their first row; its k_expand grid leaves one CTA slot
//                per SM free, so fast-lane kernels run beside it, and while
//                the fast lane has work each slow-lane row step waits (up
//                to kSlowYieldMs) for it to go idle, so short requests get
//                the GPU first.  A slow-lane k_expand started while the fast
//                lane was idle is preempted when a request arrives: its
//                warps take no new chunk (a flag in mapped host memory), the
//                launch ends within about one chunk, and the row resumes
//                once the fast lane is idle again (or kSlowYieldMs later).
//                Requests here differ in row cost by orders of magnitude:
//                the heavy ones sit out some row steps (see plan_share), so
//                the lighter ones are not paced by the heaviest row.
// A heavy request therefore never holds up the rows of the light ones, and
// both lanes' launches overlap on the device.  Each lane loop admits queued
// requests in arrival order while the projected device bytes of everything
// admitted (both lanes) stay within the budget, advances every admitted
// request by one board row (one k_expand + k_compact pair per engine for
// all of them), and hands out the requests that finished.  A request that
// arrives while others run joins at their next row.  A restarted request
// repeats exactly what it did in the fast lane, so every result is the one
// the request gets alone.
//
// No counterpart in the reference: its SearcherFactory (src/searcher.cpp:86-107)
// runs a fixed job list, one CudaSearcher per job.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
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

// Instance ids of the packed-key engines: 14 bits, so up to 16384 requests
// per lane on the device at once; requests whose window and counter bits
// exceed 49 use the general engine.
constexpr uint32_t kServerIdBits = 14;

// Fast-lane limit on one row's distinct states (about 6 MB of frontier and
// table per request).
constexpr uint64_t kFastStates = 1ull << 17;

// Longest wait of a slow-lane row step for the fast lane to go idle
// (D4E_SLOW_YIELD_MS overrides; 0 = no wait).  Measured on the mix: at 60
// req/s the served p50 went 5.9 -> 3.7 ms and p99 526 -> 428 ms, at 2000
// req/s 293 -> 344 puzzles/s (no wait vs 10 ms).
constexpr double kSlowYieldMs = 10.0;

// Slow-lane launch plan: chunks per resident warp (the default plan aims at
// 8), so that a preempted k_expand ends within a few percent of its length.
constexpr uint32_t kSlowChunksPerWarp = 32;

// Slow-lane sharing: requests whose next row is projected at more than this
// many times the cheapest running one's sit out some row steps.
constexpr double kShareRatio = 8.0;

// A slow-lane row step whose running requests are each projected at no
// more than this many device bytes (rows of about a million states) does
// not wait for the fast lane: its kernels are short
// (D4E_LIGHT_STEP_MB overrides; 0 = every step waits).
constexpr double kLightStepBytes = 64.0 * (1 << 20);

// Time of the steps without the heavy requests per step with them
// (D4E_SLOW_SHARE overrides; 0 = no sharing).
double server_share() {
    const char *v = std::getenv("D4E_SLOW_SHARE");
    return v ? std::max(0.0, std::atof(v)) : 1.0;
}

bool server_preempt() {
    const char *v = std::getenv("D4E_PREEMPT");
    return !(v && std::strcmp(v, "0") == 0);
}

bool server_autotune() {
    const char *v = std::getenv("D4E_SERVER_AUTOTUNE");
    return v && std::strcmp(v, "1") == 0;
}

struct Request {
    uint32_t width = 0, height = 0, n_pieces = 0, sym = 0, mode = 0;
    std::vector<uint8_t> rows;
    std::vector<uint64_t> shapes;
    std::vector<uint32_t> counts;
    uint64_t tag = 0;
    Clock::time_point t_submit, t_admit;
    bool moved = false;     // restarted in the slow lane
    uint32_t nomem_retries = 0;
};

// A request that ran out of device memory while others shared the device
// restarts in the slow lane (at most this many times) instead of failing.
constexpr uint32_t kNoMemRetries = 2;

}  // namespace

class Server {
public:
    explicit Server(const d4e_server_opts &o) : opts_(o) {
        if (!opts_.max_active)
            opts_.max_active = 4096;
        opts_.max_active = std::min<uint32_t>(opts_.max_active, 1u << kServerIdBits);
        int n = 0;
        cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (opts_.device < 0 || opts_.device >= n)
            throw Error(kErrInvalid, "no such CUDA device");
        cuda_check(cudaSetDevice(opts_.device), "cudaSetDevice");
        size_t total_b = 0;
        device_available_bytes(opts_.device, &total_b);
        const uint64_t cap = (uint64_t)((double)total_b * 0.9);
        budget_ = opts_.memory_budget ? opts_.memory_budget
                                      : std::min<uint64_t>(150ull << 30, cap);
        int occ = 0;
        cuda_check(expand_max_blocks_per_sm(true, &occ), "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        if (const char *v = std::getenv("D4E_SLOW_YIELD_MS"))
            slow_yield_ms_ = std::atof(v);
        if (server_preempt() && slow_yield_ms_ > 0) {
            void *h = nullptr;
            cuda_check(cudaHostAlloc(&h, sizeof(unsigned int), cudaHostAllocMapped), "cudaHostAlloc");
            preempt_h_.reset(static_cast<unsigned int *>(h));
            *preempt_h_ = 0;
            cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void **>(&preempt_d_), h, 0),
                       "cudaHostGetDevicePointer");
        }
        for (int l = 0; l < 2; l++) {
            Lane &ln = lane_[l];
            EngineOpts eo;
            eo.device = opts_.device;
            eo.isolate_failures = true;
            eo.memory_budget = budget_;
            eo.high_priority = l == 0;
            // Launch plans are measured only when asked (D4E_SERVER_AUTOTUNE=1):
            // the trials run inside the first large request of each board
            // width and key encoding, which then waits for them.
            eo.autotune = server_autotune();
            if (l == 1 && occ > 1)
                eo.expand_ctas_per_sm = occ - 1;
            if (l == 1 && preempt_d_) {
                eo.preempt_flag = preempt_d_;
                eo.preempt_gate = [this](bool preempted) { return slow_gate(preempted); };
                eo.chunks_per_warp = kSlowChunksPerWarp;
            }
            EngineOpts e64 = eo;
            e64.k64_inst_bits = kServerIdBits;
            ln.eng[0] = std::make_unique<Engine>(e64);
            EngineOpts e128 = eo;
            e128.key_mode = KeyMode::K128;
            ln.eng[1] = std::make_unique<Engine>(e128);
        }
        if (const char *v = std::getenv("D4E_LIGHT_STEP_MB"))
            light_step_bytes_ = std::atof(v) * (1 << 20);
        if (const char *v = std::getenv("D4E_FAST_STATES"))
            fast_states_ = std::max<uint64_t>(1, std::strtoull(v, nullptr, 10));
        for (int l = 0; l < 2; l++)
            lane_[l].worker = std::thread([this, l] { loop(l); });
    }

    ~Server() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        for (auto &ln : lane_)
            ln.cv.notify_all();
        yield_cv_.notify_all();
        for (auto &ln : lane_)
            if (ln.worker.joinable())
                ln.worker.join();
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
            lane_[0].queue.push_back(std::move(r));
            st_.submitted++;
            set_fast_busy(true);
        }
        lane_[0].cv.notify_all();
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
    struct Lane {
        std::unique_ptr<Engine> eng[2];
        std::thread worker;
        std::condition_variable cv;
        std::deque<Request> queue;                            // guarded by mu_
        std::unordered_map<uint32_t, Request> running[2];     // worker-owned
        size_t n_running = 0;                                 // guarded by mu_
        double projected = 0;                                 // guarded by mu_
        double avg_peak = 0;                                  // worker-owned
        uint64_t n_peaks = 0;
        // Slow-lane sharing: time of the last row step that ran every
        // request, and of the steps without the heavy ones since.
        double last_full_ms = 0, owed_ms = 0;
    };

    // Bytes charged for a request not yet started: solve-one requests are
    // bounded by their sample width, fast-lane requests by the lane limit;
    // slow-lane counting requests are charged the average peak of the ones
    // finished so far.
    double initial_projection(int l, const Request &r) const {
        const double per_state = 16.0 + 16.0 / 0.5;   // record + table slot at load 0.5
        const double floor_b = 1.0 * 1024 * 1024;
        double p = l == 0 ? (double)fast_states_ * per_state : lane_[l].avg_peak;
        if (r.mode == D4E_MODE_SOLVE_ONE && opts_.beam)
            p = std::min(p, (double)opts_.beam * 64.0 * per_state);
        return std::max(floor_b, p);
    }

    uint64_t lane_limit(int l) const {
        if (l == 1)
            return opts_.max_states;
        return opts_.max_states ? std::min(opts_.max_states, fast_states_) : fast_states_;
    }

    void loop(int l) {
        Lane &ln = lane_[l];
        try {
            cuda_check(cudaSetDevice(opts_.device), "cudaSetDevice");
            for (;;) {
                const auto ta = Clock::now();
                admit(l);
                {
                    std::lock_guard<std::mutex> lk(mu_);
                    st_.lane_admit_ms[l] += ms_between(ta, Clock::now());
                }
                bool sit_out[2] = {false, false};   // engine whose every request sits out
                bool held_any = false;
                if (l == 1) {
                    if (share_ > 0)
                        held_any = plan_share(ln, sit_out);
                    bool heavy = false;
                    for (int e = 0; e < 2; e++)
                        if (ln.eng[e]->has_active() && !sit_out[e])
                            heavy |= heavy_step(ln, e);
                    if (slow_yield_ms_ > 0) {
                        // Short requests first: while the fast lane has work,
                        // the slow lane holds a heavy row step back (at most
                        // slow_yield_ms_ per step), so fast-lane rows get the
                        // whole GPU; heavy requests progress in the gaps.  A
                        // step that starts with the fast lane idle may be
                        // preempted.
                        std::unique_lock<std::mutex> lk(mu_);
                        const auto ready = [&] { return stop_ || fast_idle(); };
                        const bool idle =
                            heavy ? yield_cv_.wait_for(
                                        lk, std::chrono::duration<double, std::milli>(slow_yield_ms_),
                                        ready)
                                  : ready();
                        slow_preemptible_ = idle && !stop_;
                    }
                }
                bool busy = false;
                double step_ms = 0;
                for (int e = 0; e < 2; e++) {
                    if (!ln.eng[e]->has_active())
                        continue;
                    busy = true;
                    if (sit_out[e])
                        continue;
                    const auto t0 = Clock::now();
                    const Totals before = ln.eng[e]->totals();
                    const uint64_t restarts0 = before.restarts;
                    const size_t n_run = ln.running[e].size();
                    const StepStats s = ln.eng[e]->step();
                    const auto t1 = Clock::now();
                    step_ms += ms_between(t0, t1);
                    collect(l, e);
                    const auto t2 = Clock::now();
                    const Totals &after = ln.eng[e]->totals();
                    std::lock_guard<std::mutex> lk(mu_);
                    st_.lane_collect_ms[l] += ms_between(t1, t2);
                    st_.lane_upload_ms[l] += after.upload_ms - before.upload_ms;
                    st_.lane_solve_one_ms[l] += (after.keep_ms - before.keep_ms) +
                                                (after.trace_ms - before.trace_ms);
                    st_.lane_retries[l] += after.retries - before.retries;
                    st_.lane_phase_ms[l][0] += after.ph_select_ms - before.ph_select_ms;
                    st_.lane_phase_ms[l][1] += after.ph_table_ms - before.ph_table_ms;
                    st_.lane_phase_ms[l][2] += after.ph_expand_ms - before.ph_expand_ms;
                    st_.lane_phase_ms[l][3] += after.ph_post_ms - before.ph_post_ms;
                    st_.lane_phase_ms[l][4] += after.ph_compact_ms - before.ph_compact_ms;
                    st_.lane_phase_ms[l][5] += after.ph_tail_ms - before.ph_tail_ms;
                    st_.steps++;
                    st_.states_out += s.n_out;
                    st_.busy_ms += ms_between(t0, t1);
                    st_.lane_steps[l]++;
                    st_.lane_busy_ms[l] += ms_between(t0, t1);
                    st_.lane_kernel_ms[l] += s.expand_ms + s.compact_ms;
                    st_.lane_inst_rows[l] += n_run - s.paused;
                    st_.restarts += ln.eng[e]->totals().restarts - restarts0;
                    st_.preemptions += after.preemptions - before.preemptions;
                    st_.paused += s.paused;
                }
                if (l == 1 && busy) {
                    if (held_any) {
                        ln.owed_ms += step_ms;
                    } else {
                        ln.last_full_ms = step_ms;
                        ln.owed_ms = 0;
                    }
                }
                if (l == 0)
                    yield_cv_.notify_all();
                double proj = 0;
                for (int e = 0; e < 2; e++)
                    for (const auto &[id, r] : ln.running[e])
                        proj += (double)ln.eng[e]->projected_bytes(id);
                std::unique_lock<std::mutex> lk(mu_);
                ln.projected = proj;
                if (stop_)
                    return;
                if (!busy && ln.queue.empty()) {
                    if (l == 0)
                        set_fast_busy(false);
                    ln.cv.wait(lk, [&] { return stop_ || !ln.queue.empty(); });
                }
                if (stop_)
                    return;
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

    // Admission: arrival order, while the projected bytes of the requests on
    // the device (both lanes) plus the candidate fit the budget (a lane with
    // nothing running always takes one) and fewer than max_active run.
    void admit(int l) {
        Lane &ln = lane_[l];
        std::vector<Request> take;
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (ln.queue.empty())
                return;
            double proj = lane_[0].projected + lane_[1].projected;
            size_t active = ln.n_running;
            const size_t cap = l == 0 ? opts_.max_active : std::max<size_t>(16, opts_.max_active / 16);
            while (!ln.queue.empty() && active < cap) {
                const double p = initial_projection(l, ln.queue.front());
                if (active > 0 && proj + p > (double)budget_)
                    break;
                take.push_back(std::move(ln.queue.front()));
                ln.queue.pop_front();
                proj += p;
                ln.projected += p;
                active++;
            }
            ln.n_running = active;
            st_.peak_projected = std::max<uint64_t>(st_.peak_projected, (uint64_t)proj);
        }
        for (Request &r : take) {
            if (!r.moved)
                r.t_admit = Clock::now();
            InstanceSpec sp;
            sp.width = r.width;
            sp.height = r.height;
            sp.rows = r.rows.data();
            sp.shapes = r.shapes.data();
            sp.counts = r.counts.data();
            sp.n_pieces = r.n_pieces;
            sp.sym = r.sym;
            sp.mode = r.mode == D4E_MODE_SOLVE_ONE ? Mode::SolveOne : Mode::Count;
            sp.max_states = lane_limit(l);
            sp.beam = opts_.beam;
            int e = 0;
            uint32_t id = 0;
            try {
                try {
                    id = ln.eng[0]->add(sp);
                } catch (const Error &err) {
                    if (err.code != kErrUnsupported ||
                        std::string(err.what()).find("packed key") == std::string::npos)
                        throw;
                    e = 1;
                    id = ln.eng[1]->add(sp);
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
                res.latency_ms = ms_between(r.t_submit, Clock::now());
                std::lock_guard<std::mutex> lk(mu_);
                ln.n_running--;
                results_.push_back(res);
                st_.failed++;
                done_cv_.notify_all();
                continue;
            }
            ln.running[e].emplace(id, std::move(r));
            std::lock_guard<std::mutex> lk(mu_);
            st_.admitted++;
            st_.peak_active = std::max<uint64_t>(st_.peak_active,
                                                 lane_[0].n_running + lane_[1].n_running);
        }
    }

    // Sharing in the slow lane: one row step advances every running request
    // of both engines (one after the other), and requests that outgrew the
    // fast lane differ in row cost by orders of magnitude.  While some
    // running requests' next rows are projected at more than kShareRatio
    // times the cheapest one's (over both engines), those heavy ones sit out
    // row steps until the steps without them have taken as long as the last
    // step with them: the others move at their own pace, and the heavy ones
    // keep about half of the lane's time.  An engine whose every request
    // sits out is not stepped (sit_out).  Returns whether any request sits
    // out the next step.
    bool plan_share(Lane &ln, bool sit_out[2]) {
        uint64_t cheapest = UINT64_MAX;
        for (int e = 0; e < 2; e++)
            for (const auto &[id, r] : ln.running[e])
                cheapest = std::min<uint64_t>(
                    cheapest, std::max<uint64_t>(ln.eng[e]->projected_bytes(id), 1));
        const bool light_turn = ln.owed_ms < share_ * ln.last_full_ms;
        bool any = false;
        for (int e = 0; e < 2; e++) {
            Engine &eng = *ln.eng[e];
            bool all = !ln.running[e].empty();
            for (const auto &[id, r] : ln.running[e]) {
                const bool hold = light_turn && (double)eng.projected_bytes(id) >
                                                    kShareRatio * (double)cheapest;
                eng.set_hold(id, hold);
                any |= hold;
                all &= hold;
            }
            sit_out[e] = all;
        }
        return any;
    }

    // Whether more than one request is on the device.
    bool shared_device() {
        std::lock_guard<std::mutex> lk(mu_);
        return lane_[0].n_running + lane_[1].n_running > 1;
    }

    // Whether an engine's next row step runs a request projected above the
    // light-step bytes (requests sitting the step out do not count).
    bool heavy_step(Lane &ln, int e) {
        Engine &eng = *ln.eng[e];
        for (const auto &[id, r] : ln.running[e])
            if (!eng.held(id) && (double)eng.projected_bytes(id) > light_step_bytes_)
                return true;
        return false;
    }

    // Guarded by mu_.
    bool fast_idle() const { return lane_[0].n_running == 0 && lane_[0].queue.empty(); }

    // The preemption flag the slow lane's k_expand polls: set while the fast
    // lane has requests (guarded by mu_).
    void set_fast_busy(bool busy) {
        if (preempt_h_)
            __atomic_store_n(preempt_h_.get(), busy ? 1u : 0u, __ATOMIC_RELEASE);
    }

    // Called by the slow lane's engines before each k_expand launch: whether
    // the launch may be preempted.  After a preemption it first waits for the
    // fast lane to go idle (at most slow_yield_ms_); a fast lane still busy
    // then gets no second preemption of the same row.
    bool slow_gate(bool preempted) {
        std::unique_lock<std::mutex> lk(mu_);
        if (!preempted)
            return slow_preemptible_ && !stop_;
        const bool idle = yield_cv_.wait_for(
            lk, std::chrono::duration<double, std::milli>(slow_yield_ms_),
            [&] { return stop_ || fast_idle(); });
        return idle && !stop_;
    }

    void collect(int l, int e) {
        Lane &ln = lane_[l];
        Engine &eng = *ln.eng[e];
        std::vector<uint32_t> fin;
        for (const auto &[id, r] : ln.running[e])
            if (eng.done(id))
                fin.push_back(id);
        if (fin.empty())
            return;
        eng.sync_results();
        const auto now = Clock::now();
        std::vector<d4e_result> out;
        std::vector<Request> moved;
        for (uint32_t id : fin) {
            Request &r = ln.running[e].at(id);
            // Outgrew the fast lane (and not the caller's own limit):
            // restart in the slow lane.  Out of device memory beside other
            // requests: restart there too (a bounded number of times), since
            // alone it may fit.
            const bool outgrew = l == 0 && eng.status(id) == kErrUnsupported &&
                                 eng.error(id).rfind("frontier limit exceeded", 0) == 0 &&
                                 (opts_.max_states == 0 || opts_.max_states > fast_states_);
            const bool crowded = eng.status(id) == kErrNoMem && r.nomem_retries < kNoMemRetries &&
                                 shared_device();
            if (outgrew || crowded) {
                if (crowded)
                    r.nomem_retries++;
                r.moved = true;
                moved.push_back(std::move(r));
            } else {
                d4e_result res;
                engine_result(eng, id, r.mode, &res);
                res.tag = r.tag;
                res.queued_ms = ms_between(r.t_submit, r.t_admit);
                res.latency_ms = ms_between(r.t_submit, now);
                if (r.mode == D4E_MODE_COUNT && res.status == 0) {
                    const double peak = (double)eng.peak_bytes(id);
                    ln.avg_peak = ln.n_peaks ? 0.95 * ln.avg_peak + 0.05 * peak : peak;
                    ln.n_peaks++;
                }
                out.push_back(res);
            }
            ln.running[e].erase(id);
            eng.release(id);
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            ln.n_running -= fin.size();
            for (const d4e_result &res : out) {
                results_.push_back(res);
                if (res.status)
                    st_.failed++;
                else
                    st_.completed++;
            }
            for (Request &r : moved)
                lane_[1].queue.push_back(std::move(r));
            st_.moved += moved.size();
        }
        if (!moved.empty())
            lane_[1].cv.notify_all();
        done_cv_.notify_all();
    }

    d4e_server_opts opts_;
    uint64_t budget_ = 0;
    struct FreeHost {
        void operator()(unsigned int *p) const { cudaFreeHost(p); }
    };
    // Preemption flag (mapped host memory); outlives the lanes' engines.
    std::unique_ptr<unsigned int, FreeHost> preempt_h_;
    Lane lane_[2];
    std::mutex mu_;
    std::condition_variable done_cv_;
    std::condition_variable yield_cv_;   // fast lane stepped (slow lane may go)
    double slow_yield_ms_ = kSlowYieldMs;
    bool slow_preemptible_ = false;          // guarded by mu_
    double share_ = server_share();          // slow-lane sharing (0: off)
    double light_step_bytes_ = kLightStepBytes;   // D4E_LIGHT_STEP_MB
    unsigned int *preempt_d_ = nullptr;      // device address of the preemption flag
    uint64_t fast_states_ = kFastStates;   // fast-lane row limit (D4E_FAST_STATES overrides)
    std::deque<d4e_result> results_;
    d4e_server_stats st_{};
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
