// engine.cu -- host runtime of the GB300 row-by-row polyomino tiling engine.
#include "engine.h"

#include <algorithm>
#include <chrono>
#include <tuple>
#include <mutex>
#include <map>
#include <memory>
#include <functional>
#include <cstdlib>
#include <cstring>

#include "kernels.h"

namespace d4e {

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        const int code = e == cudaErrorMemoryAllocation ? kErrNoMem : kErrCuda;
        throw Error(code, std::string(what) + ": " + cudaGetErrorName(e) + ": " +
                              cudaGetErrorString(e));
    }
}

namespace {
thread_local cudaMemPool_t *tl_pool_ref = nullptr;

// Idle engine pools, at most one per device: an engine that ends hands its
// pool (with the device memory it has mapped) to the next engine created on
// that device, so back-to-back batches do not map their memory again.
std::mutex g_pool_mu;
std::vector<std::pair<int, cudaMemPool_t>> g_idle_pools;

cudaMemPool_t take_idle_pool(int device) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (size_t i = 0; i < g_idle_pools.size(); i++)
        if (g_idle_pools[i].first == device) {
            const cudaMemPool_t p = g_idle_pools[i].second;
            g_idle_pools.erase(g_idle_pools.begin() + i);
            return p;
        }
    return nullptr;
}

void give_idle_pool(int device, cudaMemPool_t pool) {
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        bool have = false;
        for (auto &e : g_idle_pools)
            have |= e.first == device;
        if (!have) {
            g_idle_pools.emplace_back(device, pool);
            return;
        }
    }
    cudaMemPoolDestroy(pool);
}
}  // namespace

void release_idle_pools() {
    std::vector<std::pair<int, cudaMemPool_t>> pools;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        pools.swap(g_idle_pools);
    }
    for (auto &e : pools) {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(e.first);
        cudaMemPoolDestroy(e.second);
        if (prev >= 0)
            cudaSetDevice(prev);
    }
}

cudaError_t engine_malloc_async(void **p, size_t bytes, cudaStream_t s) {
    if (tl_pool_ref && *tl_pool_ref)
        return cudaMallocFromPoolAsync(p, bytes, *tl_pool_ref, s);
    return cudaMallocAsync(p, bytes, s);
}

template <class T>
void DevBuf<T>::reserve(size_t n, cudaStream_t stream, size_t keep) {
    if (n <= cap)
        return;
    size_t nc = std::max(n, cap + cap / 2);
    if (p && !keep) {
        // Nothing to carry over: give the old block back first, so that the
        // pool can hand its memory to the new one.
        cuda_check(cudaFreeAsync(p, s), "cudaFreeAsync");
        p = nullptr;
        cap = 0;
    }
    T *np = nullptr;
    if (engine_malloc_async(reinterpret_cast<void **>(&np), nc * sizeof(T), stream) !=
        cudaSuccess) {
        // Geometric growth did not fit: take exactly what is needed.
        cudaGetLastError();
        nc = n;
        if (engine_malloc_async(reinterpret_cast<void **>(&np), nc * sizeof(T), stream) !=
            cudaSuccess) {
            // The pools' free blocks may be too scattered for one large
            // block: once the stream's frees have happened, return every
            // unused block to the driver (this engine's pool and the idle
            // ones) and try once more.
            cudaGetLastError();
            cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
            cudaMemPool_t pool = nullptr;
            if (tl_pool_ref && *tl_pool_ref)
                pool = *tl_pool_ref;
            else {
                int dev = 0;
                cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
                cuda_check(cudaDeviceGetDefaultMemPool(&pool, dev), "cudaDeviceGetDefaultMemPool");
            }
            cuda_check(cudaMemPoolTrimTo(pool, 0), "cudaMemPoolTrimTo");
            release_idle_pools();
            cuda_check(engine_malloc_async(reinterpret_cast<void **>(&np), nc * sizeof(T), stream),
                       ("cudaMallocAsync of " + std::to_string(nc * sizeof(T)) + " bytes").c_str());
        }
    }
    if (p) {
        cuda_check(cudaMemcpyAsync(np, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, stream),
                   "cudaMemcpyAsync");
        cuda_check(cudaFreeAsync(p, s), "cudaFreeAsync");
    }
    p = np;
    cap = nc;
    s = stream;
}

size_t device_available_bytes(int device, size_t *total) {
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    cudaMemPool_t pool;
    if (tl_pool_ref && *tl_pool_ref)
        pool = *tl_pool_ref;
    else
        cuda_check(cudaDeviceGetDefaultMemPool(&pool, device), "cudaDeviceGetDefaultMemPool");
    uint64_t reserved = 0, used = 0;
    cuda_check(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved),
               "cudaMemPoolGetAttribute");
    cuda_check(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used),
               "cudaMemPoolGetAttribute");
    if (total)
        *total = total_b;
    return free_b + (reserved > used ? reserved - used : 0);
}

template struct DevBuf<Plc>;
template struct DevBuf<InstDesc>;
template struct DevBuf<unsigned int>;
template struct DevBuf<unsigned long long>;
template struct DevBuf<Seg>;
template struct DevBuf<ulonglong2>;
template struct DevBuf<PathNode>;
template struct DevBuf<unsigned char>;
template struct DevBuf<CopyRange>;
template struct DevBuf<TraceJob>;
template struct DevBuf<LevelPtr>;
template struct DevBuf<TraceOut>;
template struct DevBuf<TraceChain>;
template struct DevBuf<TraceSeg>;

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev)
            cuda_check(cudaSetDevice(dev), "cudaSetDevice");
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev)
            cudaSetDevice(prev);
    }
};

// Memory pool of the engine whose method runs on this thread: engine
// buffers come from the engine's own stream-ordered pool, so that engines on
// other streams (the serving lanes) never wait on each other's frees.
// Device + pool of one engine method call.
struct EngineScope {
    DeviceGuard dev;
    cudaMemPool_t *prev;
    EngineScope(int device, cudaMemPool_t *pool) : dev(device), prev(tl_pool_ref) {
        tl_pool_ref = pool;
    }
    ~EngineScope() { tl_pool_ref = prev; }
};

uint64_t round_up(uint64_t v, uint64_t m) { return (v + m - 1) / m * m; }

// Placement + filter table bytes of one k_expand launch's instances: about
// a third of the 129 MB L2, leaving the rest to the hash table's hot lines.
constexpr uint64_t kGroupTableBytes = 48ull << 20;

// Rows the autotuner measures on: big enough to fill the GPU, small enough
// that a dozen trial runs cost little.
constexpr uint64_t kTuneMinStates = 1ull << 21;
constexpr uint64_t kTuneMaxStates = 1ull << 25;

// k_expand prefetches children's table lines into L2 when the launch's
// table is at most this large: it shortens inserts into tables a few times
// the L2 (8x10 case: 165 -> 148 ms per enumeration) but costs HBM bandwidth
// on tables of many GB (the 8x15 case's rows of 1-6 GB lost 4-7 %).
constexpr uint64_t kPrefetchTableBytes = 512ull << 20;

// A candidate plan replaces the current one only when it is this much
// faster (trial timings vary by a few percent).
constexpr double kTuneGain = 0.97;

uint32_t bit_length(uint64_t v) {
    uint32_t b = 0;
    while (v) {
        b++;
        v >>= 1;
    }
    return b;
}

}  // namespace

Engine::Engine(const EngineOpts &opts) : opts_(opts) {
    int n = 0;
    cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (opts_.device < 0 || opts_.device >= n)
        throw Error(kErrInvalid, "no such CUDA device");
    EngineScope g(opts_.device, &pool_);
    cuda_check(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, opts_.device),
               "cudaDeviceGetAttribute");
    pool_ = take_idle_pool(opts_.device);
    if (!pool_) {
        // The engine's own pool; freed blocks stay in it for the next
        // growth instead of going back to the driver at every sync.
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = opts_.device;
        cuda_check(cudaMemPoolCreate(&pool_, &props), "cudaMemPoolCreate");
        uint64_t keep_all = ~0ull;
        cuda_check(cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep_all),
                   "cudaMemPoolSetAttribute");
    }
    int prio_least = 0, prio_greatest = 0;
    cuda_check(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest),
               "cudaDeviceGetStreamPriorityRange");
    cuda_check(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking,
                                            opts_.high_priority ? prio_greatest : prio_least),
               "cudaStreamCreate");
    for (auto &e : ev_)
        cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    for (auto &e : ev_run_)
        cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    misc_.reserve(4, stream_);
    nraw_.reserve(2, stream_);
    if (opts_.chunk_states < 32)
        opts_.chunk_states = 32;
    tune_.chunk_cap = opts_.chunk_states;
    tune_.load = opts_.target_load;
    tune_.ctas_per_sm = opts_.expand_ctas_per_sm;
    if (opts_.chunks_per_warp)
        tune_.chunks_per_warp = opts_.chunks_per_warp;
    if (opts_.k64_inst_bits) {
        if (opts_.k64_inst_bits > 23 || opts_.keep_levels)
            throw Error(kErrInvalid, "k64_inst_bits must be 1..23 (and no keep_levels)");
        k64_ = true;
        inst_off_ = 63 - opts_.k64_inst_bits;
        inst_mask_ = (1ull << opts_.k64_inst_bits) - 1ull;
        mode_fixed_ = true;
    }
}

Engine::~Engine() {
    EngineScope g(opts_.device, &pool_);
    if (stream_)
        cudaStreamSynchronize(stream_);
    for (auto &c : chunks_) {
        if (c.keys)
            cudaFreeAsync(c.keys, stream_);
        if (c.cnts)
            cudaFreeAsync(c.cnts, stream_);
    }
    if (stream_)
        cudaStreamSynchronize(stream_);
    ranges_.release();
    keep_max_.release();
    jobs_.release();
    lvlptr_.release();
    trace_out_.release();
    chain_.release();
    tsegs_.release();
    bkt_recs_.release();
    bkt_cnt_.release();
    dtab_.release();
    for (auto p : lvl_keys_)
        cudaFree(p);
    for (auto p : lvl_cnts_)
        if (p)
            cudaFree(p);
    for (auto &e : ev_)
        if (e)
            cudaEventDestroy(e);
    for (auto &e : ev_run_)
        if (e)
            cudaEventDestroy(e);
    plc_.release();
    filt_.release();
    part_ctr_.release();
    insts_.release();
    inst_unique_.release();
    cursor_.release();
    results_.release();
    final_states_.release();
    misc_.release();
    nraw_.release();
    segs_.release();
    for (int i = 0; i < 2; i++) {
        keys_[i].release();
        cnts_[i].release();
    }
    table_.release();
    if (stream_) {
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
    if (pool_)
        give_idle_pool(opts_.device, pool_);
}

void Engine::ensure_inst_capacity(size_t n) {
    // Each buffer grows on its own (a growth may fall back to the exact size).
    const size_t old = inst_.size();
    insts_.reserve(n, stream_, old);
    inst_unique_.reserve(n, stream_, 0);
    cursor_.reserve(n, stream_, 0);
    results_.reserve(n, stream_, old);
    final_states_.reserve(n, stream_, old);
}

uint32_t Engine::add(const InstanceSpec &sp) {
    EngineScope g(opts_.device, &pool_);
    if (sp.width < 1 || sp.width > (uint32_t)kMaxWidth)
        throw Error(kErrInvalid, "board width must be 1..8");
    if (sp.height < 1 || sp.height > (uint32_t)kMaxHeight)
        throw Error(kErrInvalid, "board height must be 1..64");
    if (!sp.rows || (!sp.shapes && sp.n_pieces) || (!sp.counts && sp.n_pieces))
        throw Error(kErrInvalid, "null pointer in instance");
    for (uint32_t r = 0; r < sp.height; r++)
        if (sp.rows[r] >> sp.width)
            throw Error(kErrInvalid, "board row has cells beyond the width");
    if (opts_.keep_levels && !inst_.empty())
        throw Error(kErrState, "an engine keeping levels holds one instance");
    if (inst_.size() >= kMaxInstances)
        throw Error(kErrUnsupported, "too many instances");

    if ((sp.mode == Mode::SolveOne || sp.mode == Mode::List) && opts_.keep_levels)
        throw Error(kErrInvalid, "solve-one and list instances need an engine without keep_levels");

    Inst in;
    const std::string err = build_piece_lib(sp.shapes, sp.counts, sp.n_pieces, sp.sym, sp.width,
                                            in.lib);
    if (!err.empty())
        throw Error(err.find("more than") != std::string::npos ? kErrUnsupported : kErrInvalid,
                    err);
    const bool reuse = !free_ids_.empty();
    const uint32_t id = reuse ? free_ids_.back() : (uint32_t)inst_.size();
    const bool fixed_layout = opts_.k64_inst_bits != 0;
    if (mode_fixed_ && k64_ && (n_active_ > 0 || fixed_layout) &&
        (in.lib.dyn_bits + in.lib.used_bits > inst_off_ || id > inst_mask_))
        throw Error(kErrUnsupported, "instance does not fit the engine's packed key layout");
    in.mode = sp.mode;
    in.limit = sp.max_states;
    in.beam = sp.mode == Mode::SolveOne ? sp.beam : 0;
    in.width = sp.width;
    in.height = sp.height;
    InstDesc &d = in.desc;
    d.width = sp.width;
    d.height = sp.height;
    d.win_rows = 64 / sp.width;
    d.n_plc = (uint32_t)in.lib.plc.size();
    d.plc_off = (uint32_t)plc_total_;
    d.filt_off = (uint32_t)filt_total_;
    d.fwords = in.lib.fwords;
    for (int c = 0; c < kMaxWidth; c++) {
        d.f0_off[c] = in.lib.f0_off[c];
        d.f1_off[c] = in.lib.f1_off[c];
        d.f2_off[c] = in.lib.f2_off[c];
    }
    filt_total_ += in.lib.filters.size();
    d.n_types = (uint32_t)in.lib.fields.size();
    d.dyn_bits = in.lib.dyn_bits;
    d.used_bits = in.lib.used_bits;
    plc_total_ += d.n_plc;
    for (int c = 0; c < kMaxWidth; c++) {
        d.col_off[c] = in.lib.col_off[c];
        d.col_len[c] = in.lib.col_len[c];
    }
    for (uint32_t t = 0; t < d.n_types; t++)
        d.types[t] = in.lib.fields[t];
    std::memset(d.rows, 0, sizeof(d.rows));
    for (uint32_t r = 0; r < sp.height; r++)
        d.rows[r] = sp.rows[r];
    unsigned long long w0 = 0;
    for (uint32_t r = 0; r < std::min(d.win_rows, sp.height); r++)
        w0 |= (unsigned long long)sp.rows[r] << (r * sp.width);
    in.root_window = w0;

    d.flags = sp.mode == Mode::SolveOne ? kInstWitness : 0u;
    d.limit = (uint32_t)std::min<uint64_t>(sp.max_states, 0xFFFFFFFFull);
    if (reuse) {
        free_ids_.pop_back();
        inst_[id] = std::move(in);
    } else {
        ensure_inst_capacity(id + 1);
        inst_.push_back(std::move(in));
    }
    pending_.push_back(id);
    pending_upload_.push_back(id);
    return id;
}

void Engine::release(uint32_t id) {
    Inst &in = inst_.at(id);
    if (!in.done)
        throw Error(kErrState, "instance has not finished");
    if (!in.result_ready)
        sync_results();
    drop_levels(in);
    in = Inst{};
    in.done = true;
    in.result_ready = true;
    in.status = kErrState;
    in.error = "instance released";
    free_ids_.push_back(id);
}

void Engine::fail_instance(uint32_t id, int code, const std::string &msg) {
    Inst &in = inst_[id];
    in.status = code;
    in.error = msg;
    in.active = false;
    in.done = true;
    in.result = 0;
    in.result_ready = true;
    in.seg_len = 0;
    drop_levels(in);
    n_active_--;
    tot_.failed++;
}

uint64_t Engine::frontier_bytes(int buf) const {
    return (uint64_t)keys_[buf].cap * sizeof(ulonglong2) +
           (uint64_t)cnts_[buf].cap * sizeof(unsigned long long);
}

double Engine::memory_limit(double device_avail) const {
    // Bytes available to the next frontier and the table: what the device
    // has, or what the budget leaves next to the current frontier.
    if (!opts_.memory_budget)
        return device_avail;
    const double b = (double)opts_.memory_budget - (double)frontier_bytes(cur_) -
                     (double)lvl_bytes_;
    return std::min(device_avail, b);
}

void Engine::fix_key_mode() {
    // The encoding is chosen while no state is resident (first step, or any
    // step after every instance has finished), from the instances waiting to
    // start; later additions must fit it (checked in add()).
    if (opts_.k64_inst_bits || (mode_fixed_ && (n_active_ > 0 || pending_.empty())))
        return;
    uint32_t need = 0, max_id = 0;
    for (uint32_t id : pending_) {
        need = std::max(need, inst_[id].lib.dyn_bits + inst_[id].lib.used_bits);
        max_id = std::max(max_id, id);
    }
    const uint32_t ibits = bit_length(max_id);
    const bool fits = need + ibits <= 63;
    if (opts_.key_mode == KeyMode::K64 && !fits)
        throw Error(kErrUnsupported, "packed 64-bit keys do not fit these instances");
    k64_ = opts_.key_mode == KeyMode::K64 || (opts_.key_mode == KeyMode::Auto && fits);
    inst_off_ = need;
    inst_mask_ = ibits ? ((1ull << ibits) - 1ull) : 0ull;
    mode_fixed_ = true;
}

void Engine::flush_uploads() {
    if (pending_upload_.empty())
        return;
    // Descriptors of newly added instances, one copy per run of consecutive
    // ids (ids are appended in order unless released ids are reused).
    std::vector<InstDesc> descs;
    descs.reserve(pending_upload_.size());
    for (uint32_t id : pending_upload_)
        descs.push_back(inst_[id].desc);
    for (size_t i = 0; i < pending_upload_.size();) {
        size_t j = i + 1;
        while (j < pending_upload_.size() && pending_upload_[j] == pending_upload_[j - 1] + 1)
            j++;
        const uint32_t lo = pending_upload_[i];
        cuda_check(cudaMemcpyAsync(insts_.p + lo, descs.data() + i, (j - i) * sizeof(InstDesc),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload descriptors");
        cuda_check(cudaMemsetAsync(results_.p + lo, 0, (j - i) * sizeof(unsigned long long),
                                   stream_),
                   "memset");
        cuda_check(cudaMemsetAsync(final_states_.p + lo, 0, (j - i) * sizeof(unsigned int),
                                   stream_),
                   "memset");
        i = j;
    }
    tot_.h2d_bytes += descs.size() * sizeof(InstDesc);
    // Placement tables are packed back to back in order of addition.
    std::vector<Plc> plc;
    plc.reserve(plc_total_ - plc_uploaded_);
    for (uint32_t id : pending_upload_) {
        const auto &v = inst_[id].lib.plc;
        plc.insert(plc.end(), v.begin(), v.end());
    }
    plc_.reserve(std::max<uint64_t>(plc_total_, 1), stream_, plc_uploaded_);
    if (!plc.empty())
        cuda_check(cudaMemcpyAsync(plc_.p + plc_uploaded_, plc.data(), plc.size() * sizeof(Plc),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload placements");
    tot_.h2d_bytes += plc.size() * sizeof(Plc);
    plc_uploaded_ = plc_total_;
    std::vector<unsigned long long> filt;
    filt.reserve(filt_total_ - filt_uploaded_);
    for (uint32_t id : pending_upload_) {
        const auto &v = inst_[id].lib.filters;
        filt.insert(filt.end(), v.begin(), v.end());
    }
    filt_.reserve(std::max<uint64_t>(filt_total_, 1), stream_, filt_uploaded_);
    if (!filt.empty())
        cuda_check(cudaMemcpyAsync(filt_.p + filt_uploaded_, filt.data(),
                                   filt.size() * sizeof(unsigned long long),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload filters");
    tot_.h2d_bytes += filt.size() * sizeof(unsigned long long);
    filt_uploaded_ = filt_total_;
    // The host staging vectors die here: make sure the copies have read them.
    cuda_check(cudaStreamSynchronize(stream_), "upload tables");
    pending_upload_.clear();
}

uint64_t Engine::projected_bytes(uint32_t id) const {
    const Inst &in = inst_.at(id);
    if (in.done)
        return 0;
    const double per_state = (k64_ ? 16.0 : 24.0) + (double)(slot_units() * 16) / tune_.load;
    const double est = (double)std::max<uint64_t>(in.seg_len, 1) * in.growth;
    return (uint64_t)(est * per_state + (double)in.seg_len * (k64_ ? 16.0 : 24.0));
}

uint64_t Engine::peak_bytes(uint32_t id) const {
    const Inst &in = inst_.at(id);
    uint64_t peak = 1;
    for (uint64_t v : in.level_sizes)
        peak = std::max(peak, v);
    const double per_state = (k64_ ? 16.0 : 24.0) + (double)(slot_units() * 16) / tune_.load;
    return (uint64_t)((double)peak * per_state);
}

uint64_t Engine::next_size_estimate(uint32_t id) const {
    const Inst &in = inst_.at(id);
    if (in.done)
        return 0;
    return (uint64_t)((double)std::max<uint64_t>(in.seg_len, 1) * growth_);
}

// Per-row constants of one instance's segment, in the engine's key encoding.
Seg Engine::seg_for(uint32_t id, uint32_t row) const {
    const Inst &in = inst_[id];
    const uint32_t R = in.desc.win_rows, W = in.width;
    Seg s{};
    s.inst = id;
    s.row = row;
    const uint32_t src = row + R;
    const unsigned long long in_row = src < in.height ? in.desc.rows[src] : 0u;
    s.in_shift = in_row << ((R - 1) * W);
    const uint32_t dyn_rows = W ? in.lib.dyn_bits / W : 0;
    unsigned long long hi = 0;
    for (uint32_t i = dyn_rows; i < R; i++) {
        const uint32_t r = row + i;
        if (r < in.height)
            hi |= (unsigned long long)in.desc.rows[r] << (i * W);
    }
    s.hi_board = hi;
    s.tag = k64_ ? (kMarker | ((unsigned long long)id << inst_off_))
                 : (kMarker | ((unsigned long long)id << kInstShift128));
    return s;
}

ulonglong2 Engine::root_record(uint32_t id) const {
    const Inst &in = inst_[id];
    if (k64_) {
        const unsigned long long dynmask = (1ull << in.lib.dyn_bits) - 1ull;
        return make_ulonglong2((in.root_window & dynmask) | kMarker |
                                   ((unsigned long long)id << inst_off_),
                               1ull);
    }
    return make_ulonglong2(in.root_window, kMarker | ((unsigned long long)id << kInstShift128));
}

uint64_t Engine::table_limit() {
    // Most table slots the device (or the memory budget) can hold next to
    // the current frontier, each paired with room for load * rec_bytes of
    // next frontier, 10% of the device kept back; whole regions.
    const uint64_t slot_bytes = slot_units() * sizeof(ulonglong2);
    size_t total_b = 0;
    const size_t free_b = device_available_bytes(opts_.device, &total_b);
    const double rec_bytes = k64_ ? 16.0 : 24.0;
    const double avail = memory_limit((double)table_.cap * sizeof(ulonglong2) + (double)free_b -
                                      0.1 * (double)total_b);
    const uint64_t limit =
        avail > 0 ? (uint64_t)(avail / ((double)slot_bytes + tune_.load * rec_bytes)) : 0;
    return std::max<uint64_t>(limit / kRegionAlign * kRegionAlign, kRegionAlign);
}

// Whether every instance of a launch keeps its copy counters within 32 bits
// (k_expand then works on them in 32-bit words; D4E_U32=0 never).
bool Engine::counters_fit_u32(const std::vector<Seg> &segs) const {
    static const bool off = [] {
        const char *v = std::getenv("D4E_U32");
        return v && std::strcmp(v, "0") == 0;
    }();
    if (off)
        return false;
    for (const Seg &sg : segs)
        if (inst_[sg.inst].desc.used_bits > 32)
            return false;
    return true;
}

// Whether some instance of a launch has filters of more than one word.
bool Engine::multi_word_filters(const std::vector<Seg> &segs) const {
    for (const Seg &sg : segs)
        if (inst_[sg.inst].desc.fwords > 1)
            return true;
    return false;
}

// Placements to stage in shared memory for a launch over `segs`: the
// instance's whole table when the launch holds one instance and it fits
// (D4E_STAGE_PLC=0 reads it through L1 instead).
uint32_t Engine::stage_plc(const std::vector<Seg> &segs) const {
    static const bool off = [] {
        const char *v = std::getenv("D4E_STAGE_PLC");
        return v && std::strcmp(v, "0") == 0;
    }();
    if (off || segs.size() != 1)
        return 0;
    const uint32_t np = inst_[segs[0].inst].desc.n_plc;
    return expand_stage_bytes(np) <= kStageMaxBytes ? np : 0;
}

int Engine::expand_occupancy() {
    int &occ = k64_ ? occ64_ : occ128_;
    if (!occ) {
        cuda_check(expand_max_blocks_per_sm(k64_, &occ),
                   "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        occ = std::max(occ, 1);
    }
    return opts_.expand_ctas_per_sm > 0 ? std::min(occ, opts_.expand_ctas_per_sm) : occ;
}

namespace {
using HostClock = std::chrono::steady_clock;
double host_ms_since(HostClock::time_point t0) {
    return std::chrono::duration<double, std::milli>(HostClock::now() - t0).count();
}
}  // namespace

StepStats Engine::step() {
    const auto t_step = HostClock::now();
    StepStats st = step_impl();
    tot_.step_wall_ms += host_ms_since(t_step);
    return st;
}

StepStats Engine::step_impl() {
    EngineScope g(opts_.device, &pool_);
    StepStats st;
    fix_key_mode();
    if (tot_.steps == 0 && !run_started_) {
        cuda_check(cudaEventRecord(ev_run_[0], stream_), "cudaEventRecord");
        run_started_ = true;
    }
    const auto t_up = HostClock::now();
    flush_uploads();

    // Inject root states of newly added instances as new frontier segments.
    if (!pending_.empty()) {
        std::vector<ulonglong2> rk;
        std::vector<unsigned long long> rc;
        for (uint32_t id : pending_) {
            Inst &in = inst_[id];
            in.seg_begin = n_cur_ + rk.size();
            in.seg_len = 1;
            in.active = true;
            n_active_++;
            active_.push_back(id);
            rk.push_back(root_record(id));
            rc.push_back(1ull);
        }
        keys_[cur_].reserve(n_cur_ + rk.size(), stream_, n_cur_);
        cuda_check(cudaMemcpyAsync(keys_[cur_].p + n_cur_, rk.data(), rk.size() * sizeof(ulonglong2),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload roots");
        tot_.h2d_bytes += rk.size() * sizeof(ulonglong2);
        if (!k64_) {
            cnts_[cur_].reserve(n_cur_ + rk.size(), stream_, n_cur_);
            cuda_check(cudaMemcpyAsync(cnts_[cur_].p + n_cur_, rc.data(),
                                       rc.size() * sizeof(unsigned long long),
                                       cudaMemcpyHostToDevice, stream_),
                       "upload roots");
            tot_.h2d_bytes += rc.size() * sizeof(unsigned long long);
        }
        if (opts_.keep_levels) {
            ulonglong2 *k = nullptr;
            unsigned long long *c = nullptr;
            cuda_check(cudaMalloc(&k, sizeof(ulonglong2)), "cudaMalloc");
            cuda_check(cudaMemcpyAsync(k, rk.data(), sizeof(ulonglong2), cudaMemcpyHostToDevice,
                                       stream_),
                       "upload root");
            if (!k64_) {
                cuda_check(cudaMalloc(&c, sizeof(unsigned long long)), "cudaMalloc");
                cuda_check(cudaMemcpyAsync(c, rc.data(), sizeof(unsigned long long),
                                           cudaMemcpyHostToDevice, stream_),
                           "upload root");
            }
            lvl_keys_.push_back(k);
            lvl_cnts_.push_back(c);
            lvl_n_.push_back(1);
        }
        // rk / rc are pageable: wait until the copies have read them.
        cuda_check(cudaStreamSynchronize(stream_), "upload roots");
        n_cur_ += rk.size();
        std::vector<uint32_t> roots;
        for (uint32_t id : pending_)
            if (inst_[id].mode == Mode::SolveOne || inst_[id].mode == Mode::List)
                roots.push_back(id);
        pending_.clear();
        keep_levels_of(roots);   // level 0 of solve-one and list instances
    }
    tot_.upload_ms += host_ms_since(t_up);
    if (n_active_ == 0)
        return st;

    auto t_phase = HostClock::now();
    auto phase = [&](double &acc) {
        const auto now = HostClock::now();
        acc += std::chrono::duration<double, std::milli>(now - t_phase).count();
        t_phase = now;
    };
    // Active instances in frontier order.
    std::sort(active_.begin(), active_.end(),
              [&](uint32_t a, uint32_t b) { return inst_[a].seg_begin < inst_[b].seg_begin; });
    const int occ = expand_occupancy();
    const uint64_t slots = (uint64_t)sms_ * (uint64_t)occ;
    const size_t n_inst = inst_.size();
    h_unique_.assign(n_inst, 0);
    h_cursor_.assign(n_inst, 0ull);
    st.n_in = n_cur_;

    // Which instances run this row.  The next frontier must hold the
    // projected children of the running instances plus the unchanged
    // segments of the paused ones, next to the current frontier and a hash
    // table; instances that do not fit wait (their states are carried over
    // unchanged) and run once memory frees up.  Older instances go first and
    // the oldest always runs.
    const uint64_t slot_bytes = slot_units() * sizeof(ulonglong2);
    const double rec_bytes = k64_ ? 16.0 : 24.0;
    const int nxt_buf = 1 - cur_;
    double mem = 0;
    {
        size_t total_b = 0;
        const size_t free_b = device_available_bytes(opts_.device, &total_b);
        mem = memory_limit((double)free_b + (double)table_.cap * sizeof(ulonglong2) +
                           (double)frontier_bytes(nxt_buf) - 0.1 * (double)total_b);
    }
    std::vector<uint32_t> order(active_);
    std::sort(order.begin(), order.end());
    std::vector<uint32_t> run, paused;
    double paused_bytes = 0, run_front = 0, run_table = 0;
    bool any_free = false;
    for (uint32_t id : order) {
        paused_bytes += (double)inst_[id].seg_len * rec_bytes;
        any_free |= !inst_[id].held;
    }
    for (uint32_t id : order) {
        const Inst &in = inst_[id];
        if (in.held && any_free) {
            paused.push_back(id);
            continue;
        }
        const double est = (double)std::max<uint64_t>(in.seg_len, 1) * in.growth;
        const double f = est * rec_bytes, t = est / tune_.load * (double)slot_bytes;
        const double seg_b = (double)in.seg_len * rec_bytes;
        const double need = run_front + f + (paused_bytes - seg_b) + std::max(run_table, t);
        if (run.empty() || need <= mem) {
            run.push_back(id);
            run_front += f;
            paused_bytes -= seg_b;
            run_table = std::max(run_table, t);
        } else {
            paused.push_back(id);
        }
    }
    std::sort(run.begin(), run.end(),
              [&](uint32_t a, uint32_t b) { return inst_[a].seg_begin < inst_[b].seg_begin; });
    st.paused = (uint32_t)paused.size();
    st.n_in = 0;
    for (uint32_t id : run)
        st.n_in += inst_[id].seg_len;

    // Split the running instances into groups, each one k_expand + k_compact
    // pair: a group's estimated children must fit the table budget, and its
    // placement and filter tables (read at every walk step) must stay well
    // inside L2, so that batches of thousands of instances run as a few
    // cache-resident launches rather than one launch that misses L2 on
    // every table read.  Usually one group holds them all.
    const double table_mem = std::max(mem - run_front - paused_bytes, run_table);
    const uint64_t budget_slots = (uint64_t)(table_mem / (double)slot_bytes);
    std::vector<std::vector<uint32_t>> groups(1);
    {
        double acc = 0, acc_tab = 0;
        for (uint32_t id : run) {
            const Inst &in = inst_[id];
            const double e = (double)std::max<uint64_t>(in.seg_len, 1) * in.growth /
                             tune_.load;
            const double tab = (double)(in.lib.plc.size() * sizeof(Plc) +
                                        in.lib.filters.size() * sizeof(unsigned long long) +
                                        sizeof(InstDesc));
            if (!groups.back().empty() &&
                (acc + e > (double)budget_slots || acc_tab + tab > (double)kGroupTableBytes)) {
                groups.emplace_back();
                acc = 0;
                acc_tab = 0;
            }
            groups.back().push_back(id);
            acc += e;
            acc_tab += tab;
        }
    }

    uint64_t off = 0;                                     // next-frontier fill
    std::vector<std::pair<uint32_t, uint64_t>> nseg;      // (id, begin)
    std::vector<uint32_t> finishing;
    const int nxt = 1 - cur_;
    // Groups are processed from a work list: a group whose children overflow
    // the largest table the device can hold is split in half and both halves
    // are redone.
    std::vector<std::vector<uint32_t>> work(groups.rbegin(), groups.rend());
    phase(tot_.ph_select_ms);
    while (!work.empty()) {
        const std::vector<uint32_t> grp = std::move(work.back());
        work.pop_back();
        uint64_t n_grp = 0;
        double est = 0;
        for (uint32_t id : grp) {
            n_grp += inst_[id].seg_len;
            est += (double)std::max<uint64_t>(inst_[id].seg_len, 1) * inst_[id].growth;
        }
        // Small frontiers (fewer states than a quarter of the resident lanes)
        // are split: each state's walk is cut by its first placement into
        // `fan` work items (the longest placement list of a column), so a
        // handful of states still fills the GPU; when even that leaves most
        // lanes idle (a first row: one state whose fills run to ~1e6) by its
        // first two placements, fan^2 items -- unless the step as a whole
        // is large (16x the resident lanes): then the engine is busy (a
        // server lane under load) and its small groups, new arrivals mostly,
        // must not flood the GPU with mostly empty items.  Larger frontiers
        // already fill the GPU, and warps fetch chunks independently with
        // in-warp work donation.
        // The split is chosen per instance (Seg::levels): in a large group
        // (a batch), an instance whose states each expect far more children
        // than a lane's share of the launch -- a first row, or a few states
        // of a wide board -- is split too, so that its walks do not keep a
        // handful of lanes busy long after the rest of the GPU has finished.
        // fan = the instance's longest placement list of a column.
        const uint64_t lanes = slots * 256;
        const bool small_grp = n_grp * 4 < lanes;
        static const bool split_heavy = [] {   // D4E_SPLIT_HEAVY=0: the group rule only
            const char *v = std::getenv("D4E_SPLIT_HEAVY");
            return !(v && std::strcmp(v, "0") == 0);
        }();
        std::vector<uint32_t> fan_of(grp.size(), 0), lv_of(grp.size(), 0);
        bool any_split = false;
        uint64_t items = 0;
        {
            const double share = 16.0 * std::max(64.0, est / (double)lanes);
            for (size_t k = 0; k < grp.size(); k++) {
                const Inst &in = inst_[grp[k]];
                uint32_t f = 0;
                for (int c = 0; c < kMaxWidth; c++)
                    f = std::max<uint32_t>(f, in.desc.col_len[c]);
                uint32_t lv = 0;
                if (f > 1) {
                    if (small_grp)
                        lv = n_grp * f * 4 < lanes && n_cur_ < lanes * 16 ? 2 : 1;
                    else if (split_heavy && (in.row == 0 || in.growth > share))
                        lv = in.row > 0 && in.growth / f > share ? 2 : 1;
                }
                lv = std::min(lv, opts_.max_split_levels);
                fan_of[k] = lv ? f : 0;
                lv_of[k] = lv;
                any_split |= lv > 0;
                const uint64_t per = lv == 2 ? (uint64_t)f * f : lv == 1 ? f : 1;
                items += in.seg_len * per;
            }
        }
        // Launch plan: warps take chunks independently, about
        // `chunks_per_warp` chunks per resident warp, within [32, chunk_cap]
        // items; the grid is `ctas` CTAs per SM.
        // Each instance inserts into its own table region, sized from its
        // growth estimate at the plan's load and made of whole compaction
        // tiles (so every k_compact tile belongs to one instance); at least
        // 2^20 slots for the group.  total = 0: the group does not fit the
        // memory the table may take and must be split.
        const uint64_t limit = table_limit();
        std::vector<uint64_t> region(grp.size());
        auto layout = [&](double load) -> uint64_t {
            uint64_t tot = 0;
            for (size_t k = 0; k < grp.size(); k++) {
                const Inst &in = inst_[grp[k]];
                const double want =
                    (double)std::max<uint64_t>(in.seg_len, 1) * in.growth / load;
                // A first row's fan-out is unknown: at least 64K slots.
                uint64_t r = std::max<uint64_t>((uint64_t)want, in.min_region);
                if (in.row == 0)
                    r = std::max<uint64_t>(r, 1ull << 16);
                region[k] = round_up(std::max<uint64_t>(r, kRegionAlign), kRegionAlign);
                tot += region[k];
            }
            if (tot < (1ull << 20)) {
                const uint64_t scale = ((1ull << 20) + tot - 1) / tot;
                tot = 0;
                for (auto &r : region) {
                    r *= scale;
                    tot += r;
                }
            }
            if (tot > limit) {
                if (grp.size() > 1)
                    return 0;
                region[0] = limit / kRegionAlign * kRegionAlign;
                tot = region[0];
            }
            return tot;
        };
        // Launch plan: warps take chunks independently, about
        // `chunks_per_warp` chunks per resident warp, within [32, chunk_cap]
        // items; the grid is `ctas` CTAs per SM.
        std::vector<Seg> segs;
        uint64_t chunk = 0, n_chunks = 0;
        int grid = 0;
        auto plan = [&](const Tuning &t) -> uint64_t {
            const uint64_t tot = layout(t.load);
            if (!tot)
                return 0;
            const int ctas = t.ctas_per_sm > 0 ? std::min(t.ctas_per_sm, occ) : occ;
            const uint64_t warps = (uint64_t)sms_ * (uint64_t)ctas * 8;
            const uint64_t cpw = t.chunks_per_warp;
            chunk = (items + cpw * warps - 1) / (cpw * warps);
            chunk = std::min<uint64_t>(std::max<uint64_t>(round_up(chunk, 32), 32), t.chunk_cap);
            segs.clear();
            n_chunks = 0;
            uint64_t tb = 0;
            uint64_t item_off = 0;
            for (size_t k = 0; k < grp.size(); k++) {
                const uint32_t id = grp[k];
                const Inst &in = inst_[id];
                Seg s = seg_for(id, in.row);
                const uint64_t f = fan_of[k];
                const uint64_t per = lv_of[k] == 2 ? f * f : lv_of[k] == 1 ? f : 1;
                s.rec = in.seg_begin;
                s.begin = item_off;
                s.len = in.seg_len * per;
                s.fan = fan_of[k];
                s.levels = lv_of[k];
                item_off += s.len;
                s.chunk_base = n_chunks;
                s.tbase = tb;
                s.tcap = region[k];
                tb += region[k];
                n_chunks += (s.len + chunk - 1) / chunk;
                segs.push_back(s);
            }
            segs_.reserve(segs.size(), stream_);
            cuda_check(cudaMemcpyAsync(segs_.p, segs.data(), segs.size() * sizeof(Seg),
                                       cudaMemcpyHostToDevice, stream_),
                       "upload segments");
            tot_.h2d_bytes += segs.size() * sizeof(Seg);
            grid = (int)std::min<uint64_t>(n_chunks, (uint64_t)sms_ * (uint64_t)ctas);
            return tot;
        };
        if (opts_.autotune && !tune_.set && !any_split && n_grp >= kTuneMinStates &&
            n_grp <= kTuneMaxStates)
            autotune(grp, est, occ, plan, segs, chunk, n_chunks, grid);
        const uint64_t cap = plan(tune_);
        if (!cap) {
            // The group's tables do not fit: split it.
            const size_t half = grp.size() / 2;
            work.emplace_back(grp.begin() + half, grp.end());
            work.emplace_back(grp.begin(), grp.begin() + half);
            tot_.splits++;
            continue;
        }
        // Large packed-key rows: partitioned de-duplication (children
        // appended into hash buckets, each bucket merged in shared memory)
        // instead of random inserts into a table far larger than L2.
        bool part = false;
        uint64_t n_bkt = 0, bkt_cap = 0;
        const bool want_part = opts_.dedup == EngineOpts::Dedup::Partitioned;
        if (want_part && k64_ && raw_ratio_ > 0.0) {
            n_bkt = std::max<uint64_t>(1, (uint64_t)(est * 1.25 / kBucketTarget) + 1);
            const double est_raw = (double)n_grp * raw_ratio_ * 1.25;
            bkt_cap = round_up((uint64_t)(est_raw / (double)n_bkt * 1.5) + 256, 64);
            const double bytes = (double)n_bkt * (double)bkt_cap * 16.0 +
                                 (double)n_bkt * kBucketSlots * 16.0 + (double)n_bkt * 4.0 +
                                 est * 16.0;
            part = bytes <= (double)limit * (16.0 + 16.0 * tune_.load);
        }
        unsigned long long h_raw = 0;
        float part_ms = 0.f, merge_ms = 0.f;
        if (part) {
            if (!merge_ready_) {
                cuda_check(bucket_merge_prepare(), "cudaFuncSetAttribute");
                merge_ready_ = true;
            }
            bkt_recs_.reserve(n_bkt * bkt_cap, stream_);
            bkt_cnt_.reserve(n_bkt, stream_);
            dtab_.reserve(n_bkt * kBucketSlots, stream_);
            cuda_check(cudaMemsetAsync(bkt_cnt_.p, 0, n_bkt * sizeof(unsigned int), stream_),
                       "memset");
            cuda_check(cudaMemsetAsync(inst_unique_.p, 0, n_inst * sizeof(unsigned int), stream_),
                       "memset");
            cuda_check(cudaMemsetAsync(misc_.p, 0, 4 * sizeof(unsigned int), stream_), "memset");
            cuda_check(cudaMemsetAsync(nraw_.p, 0, 2 * sizeof(unsigned long long), stream_),
                       "memset");
            phase(tot_.ph_table_ms);
            ExpandArgs a{};
            a.segs = segs_.p;
            a.n_segs = (uint32_t)segs.size();
            a.n_chunks = n_chunks;
            a.chunk_states = chunk;
            a.insts = insts_.p;
            a.plc = plc_.p;
            a.filt = filt_.p;
            a.recs = keys_[cur_].p;
            a.cnts = cnts_[cur_].p;
            a.table = table_.p;
            a.cap = 0;
            a.inst_unique = inst_unique_.p;
            a.n_raw = nraw_.p;
            a.status = misc_.p;
            a.work = nraw_.p + 1;
            a.max_probe = opts_.max_probe;
            a.append = 1;
            a.bkt_recs = bkt_recs_.p;
            a.bkt_cnt = bkt_cnt_.p;
            a.n_bkt = n_bkt;
            a.bkt_cap = bkt_cap;
            cuda_check(cudaEventRecord(ev_[0], stream_), "cudaEventRecord");
            launch_expand(k64_, a, grid, stream_);
            cuda_check(cudaGetLastError(), "k_expand launch");
            cuda_check(cudaEventRecord(ev_[1], stream_), "cudaEventRecord");
            tot_.expand_launches++;
            MergeArgs m{};
            m.bkt_recs = bkt_recs_.p;
            m.bkt_cnt = bkt_cnt_.p;
            m.n_bkt = n_bkt;
            m.bkt_cap = bkt_cap;
            m.dtab = reinterpret_cast<Slot16 *>(dtab_.p);
            m.insts = insts_.p;
            m.inst_off = inst_off_;
            m.inst_mask = inst_mask_;
            m.inst_unique = inst_unique_.p;
            m.status = misc_.p;
            launch_bucket_merge(m, sms_ * 3, stream_);
            cuda_check(cudaGetLastError(), "k_bucket_merge launch");
            cuda_check(cudaEventRecord(ev_[2], stream_), "cudaEventRecord");
            tot_.other_launches++;
            unsigned int h_status = 0;
            cuda_check(cudaMemcpyAsync(&h_status, misc_.p, sizeof(unsigned int),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read status");
            cuda_check(cudaMemcpyAsync(&h_raw, nraw_.p, sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read raw");
            h_grp_unique_.resize(n_inst);
            cuda_check(cudaMemcpyAsync(h_grp_unique_.data(), inst_unique_.p,
                                       n_inst * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                       stream_),
                       "read unique");
            cuda_check(cudaStreamSynchronize(stream_), "k_expand + k_bucket_merge");
            phase(tot_.ph_expand_ms);
            cudaEventElapsedTime(&part_ms, ev_[0], ev_[1]);
            cudaEventElapsedTime(&merge_ms, ev_[1], ev_[2]);
            st.expand_ms += part_ms;
            tot_.merge_ms += merge_ms;
            st.compact_ms += merge_ms;
            if (h_raw && n_grp)
                raw_ratio_ = (double)h_raw / (double)n_grp;
            if (h_status & kStatusBucketOverflow) {
                // A bucket (or its on-chip table) was too small: redo the row
                // with the direct table.
                part = false;
                tot_.partition_fallbacks++;
                st.retries++;
                tot_.retries++;
            } else {
                tot_.partitioned++;
            }
        }
        const uint64_t units = cap * slot_units();
        if (!part) {
        if (table_.cap < units) {
            table_.release();
            table_clean_ = 0;
            try {
                table_.reserve(units, stream_);
            } catch (const Error &e) {
                // The device could not give the table the memory its limit
                // promised: split the group, or fail a lone instance.
                if (e.code != kErrNoMem || !opts_.isolate_failures)
                    throw;
                cudaGetLastError();
                if (grp.size() > 1) {
                    const size_t half = grp.size() / 2;
                    work.emplace_back(grp.begin() + half, grp.end());
                    work.emplace_back(grp.begin(), grp.begin() + half);
                    tot_.splits++;
                } else {
                    fail_instance(grp[0], kErrNoMem,
                                  "row does not fit the device: a table of " +
                                      std::to_string(units * sizeof(ulonglong2)) + " bytes");
                    st.failed++;
                }
                continue;
            }
        }
        if (table_clean_ < units) {
            cuda_check(cudaMemsetAsync(table_.p + table_clean_, 0,
                                       (units - table_clean_) * sizeof(ulonglong2), stream_),
                       "memset table");
            table_clean_ = units;
        }
        cuda_check(cudaMemsetAsync(inst_unique_.p, 0, n_inst * sizeof(unsigned int), stream_),
                   "memset");
        cuda_check(cudaMemsetAsync(misc_.p, 0, 4 * sizeof(unsigned int), stream_), "memset");
        cuda_check(cudaMemsetAsync(nraw_.p, 0, 2 * sizeof(unsigned long long), stream_), "memset");
        phase(tot_.ph_table_ms);
        ExpandArgs a{};
        a.segs = segs_.p;
        a.n_segs = (uint32_t)segs.size();
        a.n_chunks = n_chunks;
        a.chunk_states = chunk;
        a.insts = insts_.p;
        a.plc = plc_.p;
        a.filt = filt_.p;
        a.recs = keys_[cur_].p;
        a.cnts = cnts_[cur_].p;
        a.table = table_.p;
        a.cap = cap;
        a.inst_unique = inst_unique_.p;
        a.n_raw = nraw_.p;
        a.status = misc_.p;
        a.work = nraw_.p + 1;
        a.max_probe = opts_.max_probe;
        a.prefetch = units * sizeof(ulonglong2) <= kPrefetchTableBytes ? 1u : 0u;
        a.stage_plc = stage_plc(segs);
        a.u32 = counters_fit_u32(segs) ? 1u : 0u;
        a.single_word = multi_word_filters(segs) ? 0u : 1u;
        // Multi-instance rows of an engine that is never preempted claim
        // chunks by SM partition (ExpandArgs::parts; D4E_CLAIM_PARTS=0: one
        // global counter).
        {
            static const bool parts_on = [] {
                const char *v = std::getenv("D4E_CLAIM_PARTS");
                return !(v && std::strcmp(v, "0") == 0);
            }();
            if (parts_on && k64_ && segs.size() > 1 && !opts_.preempt_flag) {
                part_ctr_.reserve(sms_, stream_);
                cuda_check(cudaMemsetAsync(part_ctr_.p, 0, sms_ * sizeof(unsigned long long),
                                           stream_),
                           "memset");
                a.parts = (uint32_t)sms_;
                a.part_step = (n_chunks + (uint64_t)sms_ - 1) / (uint64_t)sms_;
                a.part_ctr = part_ctr_.p;
            }
        }
        // A launch that honours the preemption flag may end with chunks not
        // yet taken (the work counter below n_chunks): launch again, with
        // the counters kept, until the row is done.
        const bool can_preempt = opts_.preempt_flag && opts_.preempt_gate;
        for (bool preempted = false;;) {
            a.preempt = can_preempt && opts_.preempt_gate(preempted) ? opts_.preempt_flag
                                                                      : nullptr;
            cuda_check(cudaEventRecord(ev_[0], stream_), "cudaEventRecord");
            launch_expand(k64_, a, grid, stream_);
            cuda_check(cudaGetLastError(), "k_expand launch");
            cuda_check(cudaEventRecord(ev_[1], stream_), "cudaEventRecord");
            tot_.expand_launches++;
            if (!a.preempt)
                break;
            unsigned long long h_taken = 0;
            cuda_check(cudaMemcpyAsync(&h_taken, a.work, sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read work counter");
            cuda_check(cudaStreamSynchronize(stream_), "k_expand");
            tot_.d2h_bytes += sizeof(unsigned long long);
            if (h_taken >= n_chunks)
                break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
            st.expand_ms += ms;
            tot_.preemptions++;
            preempted = true;
        }
        cuda_check(cudaMemcpyAsync(&h_raw, nraw_.p, sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, stream_),
                   "read raw");
        h_grp_unique_.resize(n_inst);
        cuda_check(cudaMemcpyAsync(h_grp_unique_.data(), inst_unique_.p,
                                   n_inst * sizeof(unsigned int), cudaMemcpyDeviceToHost, stream_),
                   "read unique");
        cuda_check(cudaStreamSynchronize(stream_), "k_expand");
        phase(tot_.ph_expand_ms);
        {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
            st.expand_ms += ms;
        }
        if (h_raw && n_grp)
            raw_ratio_ = (double)h_raw / (double)n_grp;
        }
        tot_.d2h_bytes += sizeof(unsigned long long) + n_inst * sizeof(unsigned int);
        // The table k_compact reads: the merged bucket tables, or the
        // instances' regions.
        void *ctab = part ? (void *)dtab_.p : (void *)table_.p;
        const uint64_t ccap = part ? n_bkt * kBucketSlots : cap;
        st.groups++;
        st.n_raw += h_raw;
        st.table_cap = std::max<uint64_t>(st.table_cap, cap);

        // Instances whose region overflowed are redone, alone, with 4x the
        // region (a lone instance at least raw / load); their partial
        // children are dropped by this group's compaction.
        std::vector<char> redo(grp.size(), 0);
        std::vector<uint32_t> retry;
        for (size_t k = 0; k < grp.size(); k++) {
            const uint32_t id = grp[k];
            if (!(h_grp_unique_[id] & kUniqueOverflow)) {
                h_unique_[id] = h_grp_unique_[id];
                continue;
            }
            redo[k] = 1;
            h_unique_[id] = 0;
            h_cursor_[id] = kCursorDrop;
            st.retries++;
            tot_.retries++;
            Inst &in = inst_[id];
            if (region[k] >= limit / kRegionAlign * kRegionAlign) {
                if (!opts_.isolate_failures)
                    throw Error(kErrNoMem, "hash table cannot grow: device memory exhausted");
                fail_instance(id, kErrNoMem,
                              "row does not fit the device: more than " +
                                  std::to_string(region[k]) + " table slots");
                st.failed++;
                continue;
            }
            // Small regions grow fast (a wrong first guess costs a relaunch).
            uint64_t grow = region[k] * (region[k] < (1ull << 18) ? 32 : 4);
            if (grp.size() == 1)
                grow = std::max<uint64_t>(grow, (uint64_t)((double)h_raw / tune_.load));
            in.min_region = grow;
            retry.push_back(id);
        }
        uint64_t uniq = 0;
        for (size_t k = 0; k < grp.size(); k++)
            if (!redo[k])
                uniq += h_unique_[grp[k]];
        if (opts_.max_frontier && st.n_out + uniq > opts_.max_frontier) {
            cuda_check(cudaMemsetAsync(table_.p, 0, cap * slot_units() * sizeof(ulonglong2),
                                       stream_),
                       "memset table");
            cuda_check(cudaStreamSynchronize(stream_), "memset table");
            throw Error(kErrUnsupported, "frontier limit exceeded: " +
                                             std::to_string(st.n_out + uniq) + " states");
        }

        // This group's next segments follow the previous groups' ones.
        const uint64_t off0 = off;
        const size_t nseg0 = nseg.size();
        for (size_t k = 0; k < grp.size(); k++) {
            const uint32_t id = grp[k];
            if (redo[k])
                continue;
            const Inst &in = inst_[id];
            const uint64_t u = h_unique_[id];
            if (in.limit && u > in.limit) {
                // Over its own frontier limit: the instance fails, its
                // children are dropped by the compaction.
                h_cursor_[id] = kCursorDrop;
                fail_instance(id, kErrUnsupported,
                              "frontier limit exceeded: " + std::to_string(u) + " states");
                st.failed++;
                continue;
            }
            st.n_out += u;
            if (in.row + 1 == in.height && !opts_.keep_levels && in.mode == Mode::Count) {
                h_cursor_[id] = kCursorFinal;
                finishing.push_back(id);
            } else {
                h_cursor_[id] = off;
                nseg.push_back({id, off});
                off += u;
            }
        }
        // The next frontier must hold the group's distinct states.  When the
        // device cannot hold them (the rows' growth outran the estimate that
        // admitted them), the group's largest instances fail alone with
        // D4E_ERR_NOMEM -- their children are dropped by the compaction --
        // until the rest fit.
        for (;;) {
            try {
                keys_[nxt].reserve(std::max<uint64_t>(off, 1), stream_, off0);
                if (!k64_)
                    cnts_[nxt].reserve(std::max<uint64_t>(off, 1), stream_, off0);
                break;
            } catch (const Error &e) {
                if (e.code != kErrNoMem || !opts_.isolate_failures || nseg.size() == nseg0)
                    throw;
                cudaGetLastError();
                size_t big = nseg0;
                for (size_t q = nseg0; q < nseg.size(); q++)
                    if (h_unique_[nseg[q].first] > h_unique_[nseg[big].first])
                        big = q;
                const uint32_t id = nseg[big].first;
                const uint64_t u = h_unique_[id];
                h_cursor_[id] = kCursorDrop;
                fail_instance(id, kErrNoMem,
                              "row does not fit the device: " + std::to_string(u) +
                                  " distinct states in the next frontier");
                st.failed++;
                st.n_out -= u;
                nseg.erase(nseg.begin() + (std::ptrdiff_t)big);
                off = off0;
                for (size_t q = nseg0; q < nseg.size(); q++) {
                    nseg[q].second = off;
                    h_cursor_[nseg[q].first] = off;
                    off += h_unique_[nseg[q].first];
                }
            }
        }
        cuda_check(cudaMemcpyAsync(cursor_.p, h_cursor_.data(),
                                   n_inst * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                                   stream_),
                   "upload cursors");
        tot_.h2d_bytes += n_inst * sizeof(unsigned long long);
        // Solve-one instances over their sample width keep a hash-chosen
        // subset of about `beam` states (the same subset alone or batched).
        std::vector<uint32_t> sampled;
        for (size_t k = 0; k < grp.size(); k++) {
            Inst &in = inst_[grp[k]];
            if (!redo[k] && in.mode == Mode::SolveOne && in.beam && !in.done &&
                h_unique_[grp[k]] > in.beam)
                sampled.push_back(grp[k]);
        }
        if (!sampled.empty()) {
            h_keep_max_.assign(n_inst, ~0ull);
            for (uint32_t id : sampled) {
                const double frac = (double)inst_[id].beam / (double)h_unique_[id];
                h_keep_max_[id] = (unsigned long long)std::ldexp(frac, 64);
                inst_[id].sampled = true;
            }
            keep_max_.reserve(n_inst, stream_);
            cuda_check(cudaMemcpyAsync(keep_max_.p, h_keep_max_.data(),
                                       n_inst * sizeof(unsigned long long),
                                       cudaMemcpyHostToDevice, stream_),
                       "upload sample thresholds");
            tot_.h2d_bytes += n_inst * sizeof(unsigned long long);
        }
        CompactArgs c;
        c.table = ctab;
        c.cap = ccap;
        c.cursor = cursor_.p;
        c.out_recs = keys_[nxt].p;
        c.out_cnts = cnts_[nxt].p;
        c.results = results_.p;
        c.final_states = final_states_.p;
        c.inst_off = inst_off_;
        c.inst_mask = inst_mask_;
        c.keep_max = sampled.empty() ? nullptr : keep_max_.p;
        c.status = misc_.p;
        c.stages = tune_.compact_stages;
        const int cgrid = compact_grid(ccap, sms_, tune_.compact_ctas);
        phase(tot_.ph_post_ms);
        cuda_check(cudaEventRecord(ev_[2], stream_), "cudaEventRecord");
        launch_compact(k64_, c, cgrid, stream_);
        cuda_check(cudaGetLastError(), "k_compact launch");
        cuda_check(cudaEventRecord(ev_[3], stream_), "cudaEventRecord");
        tot_.compact_launches++;
        tot_.compact_slots += ccap;
        unsigned int c_status = 0;
        cuda_check(cudaMemcpyAsync(&c_status, misc_.p, sizeof(unsigned int),
                                   cudaMemcpyDeviceToHost, stream_),
                   "read status");
        cuda_check(cudaStreamSynchronize(stream_), "k_compact");
        if (c_status & kStatusCompactStall)
            throw Error(kErrCuda, "k_compact: a staged table tile did not arrive");
        phase(tot_.ph_compact_ms);
        float cms = 0.f;
        cudaEventElapsedTime(&cms, ev_[2], ev_[3]);
        st.compact_ms += cms;
        // Table growth of the next row follows the distinct children the
        // table had to hold (before sampling).
        std::vector<double> table_growth(grp.size(), 0.0);
        for (size_t k = 0; k < grp.size(); k++) {
            const Inst &in = inst_[grp[k]];
            if (in.seg_len)
                table_growth[k] = (double)h_unique_[grp[k]] / (double)in.seg_len;
        }
        if (!sampled.empty()) {
            // Kept states per sampled instance = cursor advance.
            std::vector<unsigned long long> cend(n_inst);
            cuda_check(cudaMemcpyAsync(cend.data(), cursor_.p, n_inst * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read cursors");
            cuda_check(cudaStreamSynchronize(stream_), "read cursors");
            tot_.d2h_bytes += n_inst * sizeof(unsigned long long);
            for (uint32_t id : sampled)
                h_unique_[id] = (unsigned int)(cend[id] - h_cursor_[id]);
        }
        // Per-instance growth estimates for the next row.
        for (size_t k = 0; k < grp.size(); k++) {
            Inst &in = inst_[grp[k]];
            if (redo[k] || in.done)
                continue;
            in.min_region = 0;
            if (in.seg_len)
                in.growth = std::clamp(table_growth[k] * 1.25, 1.0, 256.0);
        }
        if (!retry.empty())
            work.push_back(std::move(retry));
        phase(tot_.ph_post_ms);
    }
    // Paused instances: their states move unchanged to the next frontier.
    std::vector<std::pair<uint32_t, uint64_t>> moved;   // (id, new begin)
    if (!paused.empty()) {
        // Room for the carried states; when the device cannot give it, the
        // largest waiting instances fail alone (D4E_ERR_NOMEM) until the
        // rest fit.
        for (;;) {
            uint64_t need = off;
            for (uint32_t id : paused)
                need += inst_[id].seg_len;
            try {
                keys_[nxt].reserve(std::max<uint64_t>(need, 1), stream_, off);
                if (!k64_)
                    cnts_[nxt].reserve(std::max<uint64_t>(need, 1), stream_, off);
                break;
            } catch (const Error &e) {
                if (e.code != kErrNoMem || !opts_.isolate_failures)
                    throw;
                cudaGetLastError();
                auto big = std::max_element(paused.begin(), paused.end(),
                                            [&](uint32_t a, uint32_t b) {
                                                return inst_[a].seg_len < inst_[b].seg_len;
                                            });
                fail_instance(*big, kErrNoMem,
                              "waiting row does not fit the device next to the running ones: " +
                                  std::to_string(inst_[*big].seg_len) + " states");
                st.failed++;
                paused.erase(big);
            }
        }
        for (uint32_t id : paused) {
            const Inst &in = inst_[id];
            if (in.seg_len) {
                cuda_check(cudaMemcpyAsync(keys_[nxt].p + off, keys_[cur_].p + in.seg_begin,
                                           in.seg_len * sizeof(ulonglong2),
                                           cudaMemcpyDeviceToDevice, stream_),
                           "carry paused states");
                if (!k64_)
                    cuda_check(cudaMemcpyAsync(cnts_[nxt].p + off, cnts_[cur_].p + in.seg_begin,
                                               in.seg_len * sizeof(unsigned long long),
                                               cudaMemcpyDeviceToDevice, stream_),
                               "carry paused states");
            }
            moved.push_back({id, off});
            off += in.seg_len;
        }
    }
    if (opts_.keep_levels) {
        ulonglong2 *k = nullptr;
        unsigned long long *cn = nullptr;
        const uint64_t n = std::max<uint64_t>(off, 1);
        cuda_check(cudaMalloc(&k, n * sizeof(ulonglong2)), "cudaMalloc");
        if (!k64_)
            cuda_check(cudaMalloc(&cn, n * sizeof(unsigned long long)), "cudaMalloc");
        if (off) {
            cuda_check(cudaMemcpyAsync(k, keys_[nxt].p, off * sizeof(ulonglong2),
                                       cudaMemcpyDeviceToDevice, stream_),
                       "keep level");
            if (!k64_)
                cuda_check(cudaMemcpyAsync(cn, cnts_[nxt].p, off * sizeof(unsigned long long),
                                           cudaMemcpyDeviceToDevice, stream_),
                           "keep level");
        }
        lvl_keys_.push_back(k);
        lvl_cnts_.push_back(cn);
        lvl_n_.push_back(off);
    }
    cuda_check(cudaEventRecord(ev_run_[1], stream_), "cudaEventRecord");
    cuda_check(cudaStreamSynchronize(stream_), "row end");
    float rms = 0.f;
    cudaEventElapsedTime(&rms, ev_run_[0], ev_run_[1]);
    tot_.run_ms = rms;

    // Advance the instances.
    std::vector<uint32_t> still;
    still.reserve(active_.size());
    std::vector<uint32_t> keep_now, to_trace, to_total, ended;
    for (const auto &[id, begin] : nseg) {
        Inst &in = inst_[id];
        in.seg_begin = begin;
        in.seg_len = h_unique_[id];
        in.level_sizes.push_back(in.seg_len);
        in.row++;
        if (in.mode == Mode::SolveOne || in.mode == Mode::List) {
            if (in.seg_len == 0) {
                ended.push_back(id);
            } else {
                keep_now.push_back(id);
                if (in.row == in.height)
                    (in.mode == Mode::SolveOne ? to_trace : to_total).push_back(id);
                else
                    still.push_back(id);
            }
            continue;
        }
        if (in.mode == Mode::Sets && in.row == in.height && in.seg_len) {
            // The final row's states are the tiling piece multisets: read
            // them back and decode each used-copy counter per piece type.
            std::vector<ulonglong2> rec(in.seg_len);
            std::vector<unsigned long long> cn;
            cuda_check(cudaMemcpyAsync(rec.data(), keys_[nxt].p + begin,
                                       in.seg_len * sizeof(ulonglong2), cudaMemcpyDeviceToHost,
                                       stream_),
                       "read final states");
            if (!k64_) {
                cn.resize(in.seg_len);
                cuda_check(cudaMemcpyAsync(cn.data(), cnts_[nxt].p + begin,
                                           in.seg_len * sizeof(unsigned long long),
                                           cudaMemcpyDeviceToHost, stream_),
                           "read final states");
            }
            cuda_check(cudaStreamSynchronize(stream_), "read final states");
            tot_.d2h_bytes += in.seg_len * (k64_ ? 16 : 24);
            const unsigned long long usedmask =
                in.lib.used_bits ? ((1ull << in.lib.used_bits) - 1ull) : 0ull;
            // Sort key: the copy counters repacked type-major (type 0 most
            // significant), so numeric order is the lexicographic order of
            // the copies; the counters take used_bits <= 40 bits in all.
            const auto &fields = in.lib.fields;
            const size_t nt = fields.size();
            std::vector<std::pair<unsigned long long, unsigned long long>> ks(in.seg_len);
            unsigned long long sum = 0;
            for (uint64_t k = 0; k < in.seg_len; k++) {
                const unsigned long long used =
                    k64_ ? (rec[k].x >> in.lib.dyn_bits) & usedmask : rec[k].y & kUsedMask128;
                unsigned long long key = 0;
                for (const TypeField &f : fields)
                    if (f.fm)
                        key = (key << __builtin_popcountll(f.fm)) |
                              ((used & f.fm) >> __builtin_ctzll(f.fm));
                ks[k] = {key, k64_ ? rec[k].y : cn[k]};
                sum += ks[k].second;
            }
            std::sort(ks.begin(), ks.end());
            PieceSets &out = in.sets;
            out.n_types = (uint32_t)nt;
            out.copies.assign(in.seg_len * nt, 0);
            out.tilings.resize(in.seg_len);
            for (uint64_t k = 0; k < in.seg_len; k++) {
                unsigned long long key = ks[k].first;
                for (size_t t = nt; t-- > 0;)
                    if (fields[t].fm) {
                        const int b = __builtin_popcountll(fields[t].fm);
                        out.copies[k * nt + t] = (uint8_t)(key & ((1ull << b) - 1ull));
                        key >>= b;
                    }
                out.tilings[k] = ks[k].second;
            }
            in.active = false;
            in.done = true;
            n_active_--;
            in.result = sum;
            in.result_ready = true;
            in.seg_len = 0;
            continue;
        }
        if (in.row == in.height || in.seg_len == 0) {
            in.active = false;
            in.done = true;
            n_active_--;
            unsigned long long sum = 0;
            if (opts_.keep_levels && in.row == in.height && in.seg_len) {
                // Final level: sum the counts of the stored states.
                if (k64_) {
                    std::vector<ulonglong2> rec(in.seg_len);
                    cuda_check(cudaMemcpyAsync(rec.data(), lvl_keys_.back(),
                                               in.seg_len * sizeof(ulonglong2),
                                               cudaMemcpyDeviceToHost, stream_),
                               "read final level");
                    cuda_check(cudaStreamSynchronize(stream_), "read final level");
                    for (const auto &r : rec)
                        sum += r.y;
                } else {
                    std::vector<unsigned long long> cn(in.seg_len);
                    cuda_check(cudaMemcpyAsync(cn.data(), lvl_cnts_.back(),
                                               in.seg_len * sizeof(unsigned long long),
                                               cudaMemcpyDeviceToHost, stream_),
                               "read final level");
                    cuda_check(cudaStreamSynchronize(stream_), "read final level");
                    for (auto v : cn)
                        sum += v;
                }
                tot_.d2h_bytes += in.seg_len * (k64_ ? 16 : 8);
            }
            in.result = sum;
            in.result_ready = true;
            in.seg_len = 0;
        } else {
            still.push_back(id);
        }
    }
    for (uint32_t id : finishing) {
        Inst &in = inst_[id];
        in.level_sizes.push_back(h_unique_[id]);
        in.row++;
        in.active = false;
        in.done = true;
        in.seg_len = 0;
        n_active_--;
        unfetched_.push_back(id);
    }
    for (const auto &[id, begin] : moved) {
        inst_[id].seg_begin = begin;
        still.push_back(id);
    }
    active_.swap(still);
    n_cur_ = off;
    cur_ = nxt;
    // Solve-one: keep the new levels, trace the instances that completed
    // their last row, and retry exhausted sampled attempts wider.
    const auto t_keep = HostClock::now();
    keep_levels_of(keep_now);
    const auto t_trace = HostClock::now();
    tot_.keep_ms += host_ms_since(t_keep);
    trace_solutions(to_trace);
    total_lists(to_total);
    tot_.trace_ms += host_ms_since(t_trace);
    for (uint32_t id : ended) {
        if (inst_[id].sampled)
            restart(id);
        else
            finish_solve_one(id, false);
    }
    if (st.n_in)
        growth_ = std::clamp((double)st.n_out / (double)st.n_in * 1.25, 1.0, 256.0);

    phase(tot_.ph_tail_ms);
    tot_.steps++;
    tot_.states_in += st.n_in;
    tot_.states_raw += st.n_raw;
    tot_.states_out += st.n_out;
    tot_.expand_ms += st.expand_ms;
    tot_.compact_ms += st.compact_ms;
    tot_.peak_frontier = std::max<uint64_t>(tot_.peak_frontier, st.n_out);
    tot_.paused += st.paused;
    return st;
}

namespace {

// Tuned launch parameters per (key encoding, board width, device), shared
// by every engine of the process.
struct TuneKey {
    bool k64;
    uint32_t width;
    int device;
    bool operator<(const TuneKey &o) const {
        return std::tie(k64, width, device) < std::tie(o.k64, o.width, o.device);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, Tuning> g_tune_cache;

}  // namespace

void autotune_clear() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.clear();
}

void Engine::autotune(const std::vector<uint32_t> &grp, double est, int occ,
                      const std::function<uint64_t(const Tuning &)> &plan,
                      const std::vector<Seg> &segs, const uint64_t &chunk,
                      const uint64_t &n_chunks, const int &grid) {
    // Replaces the reference's launch-sizing model (KSizing::optimize /
    // KParams::fom, src/kernel.cu:99-236) with measurement: the row about to
    // run is expanded and compacted (children discarded) under candidate
    // launch plans, and the fastest is kept -- first the CTAs per SM, then
    // the chunk sizing, then the table load factor.
    const TuneKey key{k64_, inst_[grp[0]].width, opts_.device};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            tune_ = it->second;
            return;
        }
    }
    const auto t0 = HostClock::now();
    const size_t n_inst = inst_.size();
    std::vector<unsigned long long> drop(n_inst, kCursorDrop);
    cuda_check(cudaMemcpyAsync(cursor_.p, drop.data(), n_inst * sizeof(unsigned long long),
                               cudaMemcpyHostToDevice, stream_),
               "upload cursors");
    (void)est;
    double last_compact_ms = 0;   // k_compact part of the last trial
    auto trial = [&](const Tuning &t) -> double {
        const uint64_t cap = plan(t);
        if (!cap)
            return 1e30;
        const uint64_t units = cap * slot_units();
        if (table_.cap < units) {
            table_.release();
            table_clean_ = 0;
            table_.reserve(units, stream_);
        }
        if (table_clean_ < units) {
            cuda_check(cudaMemsetAsync(table_.p + table_clean_, 0,
                                       (units - table_clean_) * sizeof(ulonglong2), stream_),
                       "memset table");
            table_clean_ = units;
        }
        cuda_check(cudaMemsetAsync(inst_unique_.p, 0, n_inst * sizeof(unsigned int), stream_),
                   "memset");
        cuda_check(cudaMemsetAsync(misc_.p, 0, 4 * sizeof(unsigned int), stream_), "memset");
        cuda_check(cudaMemsetAsync(nraw_.p, 0, 2 * sizeof(unsigned long long), stream_), "memset");
        ExpandArgs a{};
        a.segs = segs_.p;
        a.n_segs = (uint32_t)segs.size();
        a.n_chunks = n_chunks;
        a.chunk_states = chunk;
        a.insts = insts_.p;
        a.plc = plc_.p;
        a.filt = filt_.p;
        a.recs = keys_[cur_].p;
        a.cnts = cnts_[cur_].p;
        a.table = table_.p;
        a.cap = cap;
        a.inst_unique = inst_unique_.p;
        a.n_raw = nraw_.p;
        a.status = misc_.p;
        a.work = nraw_.p + 1;
        a.max_probe = opts_.max_probe;
        a.prefetch = units * sizeof(ulonglong2) <= kPrefetchTableBytes ? 1u : 0u;
        a.stage_plc = stage_plc(segs);
        a.u32 = counters_fit_u32(segs) ? 1u : 0u;
        a.single_word = multi_word_filters(segs) ? 0u : 1u;
        CompactArgs c{};
        c.table = table_.p;
        c.cap = cap;
        c.cursor = cursor_.p;   // every instance dropped: scan and clear only
        c.out_recs = keys_[1 - cur_].p;
        c.out_cnts = cnts_[1 - cur_].p;
        c.results = results_.p;
        c.final_states = final_states_.p;
        c.inst_off = inst_off_;
        c.inst_mask = inst_mask_;
        c.keep_max = nullptr;
        c.status = misc_.p;
        c.stages = t.compact_stages;
        const int cgrid = compact_grid(cap, sms_, t.compact_ctas);
        cuda_check(cudaEventRecord(ev_[0], stream_), "cudaEventRecord");
        launch_expand(k64_, a, grid, stream_);
        cuda_check(cudaEventRecord(ev_[2], stream_), "cudaEventRecord");
        launch_compact(k64_, c, cgrid, stream_);
        cuda_check(cudaGetLastError(), "autotune launch");
        cuda_check(cudaEventRecord(ev_[1], stream_), "cudaEventRecord");
        unsigned int stt = 0;
        cuda_check(cudaMemcpyAsync(&stt, misc_.p, sizeof(stt), cudaMemcpyDeviceToHost, stream_),
                   "read status");
        cuda_check(cudaStreamSynchronize(stream_), "autotune trial");
        tot_.other_launches += 2;
        float ms = 0.f, cms = 0.f;
        cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
        cudaEventElapsedTime(&cms, ev_[2], ev_[1]);
        last_compact_ms = cms;
        for (uint32_t id : grp)
            inst_[id].min_region = 0;
        if (stt & kStatusCompactStall)
            throw Error(kErrCuda, "k_compact: a staged table tile did not arrive");
        return (stt & kStatusTableOverflow) ? 1e30 : (double)ms;
    };
    Tuning best = tune_;
    best.ctas_per_sm = occ;
    trial(best);                       // warm-up
    double best_ms = trial(best);
    auto consider = [&](Tuning t) {
        const double ms = trial(t);
        if (ms < best_ms * kTuneGain) {
            best_ms = ms;
            best = t;
        }
    };
    for (int c = occ - 1; c >= std::max(1, occ - 2); c--) {
        Tuning t = best;
        t.ctas_per_sm = c;
        consider(t);
    }
    const Tuning base = best;
    for (uint32_t cpw : {4u, 16u}) {
        Tuning t = base;
        t.chunks_per_warp = cpw;
        consider(t);
    }
    const Tuning base2 = best;
    for (uint64_t cap : {256ull, 512ull, 2048ull}) {
        Tuning t = base2;
        t.chunk_cap = cap;
        consider(t);
    }
    const Tuning base3 = best;
    for (double load : {0.35, 0.7}) {
        Tuning t = base3;
        t.load = load;
        consider(t);
    }
    // The dedup tile plan (k_compact blocks per SM x ring depth), chosen by
    // the compaction's own time, a few percent of the trial's.
    {
        trial(best);
        double best_cms = last_compact_ms;
        const Tuning base4 = best;
        for (const auto &[ctas, stages] : {std::pair<int, uint32_t>{2, 2},
                                           std::pair<int, uint32_t>{1, 6}}) {
            if (!compact_plan_ok(ctas, stages))
                continue;
            Tuning t = base4;
            t.compact_ctas = ctas;
            t.compact_stages = stages;
            if (trial(t) < 1e29 && last_compact_ms < best_cms * kTuneGain) {
                best_cms = last_compact_ms;
                best.compact_ctas = ctas;
                best.compact_stages = stages;
            }
        }
    }
    best.set = true;
    tune_ = best;
    tot_.tune_ms += host_ms_since(t0);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = best;
}

void Engine::keep_levels_of(const std::vector<uint32_t> &ids) {
    // One pool block per call for the current segments of `ids`, filled by
    // one range-copy launch.
    uint64_t total = 0;
    for (uint32_t id : ids)
        total += inst_[id].seg_len;
    if (ids.empty() || total == 0)
        return;
    LvlChunk ch;
    cuda_check(engine_malloc_async(reinterpret_cast<void **>(&ch.keys),
                                   total * sizeof(ulonglong2), stream_),
               "cudaMallocAsync");
    ch.bytes = total * sizeof(ulonglong2);
    if (!k64_) {
        cuda_check(engine_malloc_async(reinterpret_cast<void **>(&ch.cnts),
                                       total * sizeof(unsigned long long), stream_),
                   "cudaMallocAsync");
        ch.bytes += total * sizeof(unsigned long long);
    }
    uint32_t ci;
    if (!free_chunks_.empty()) {
        ci = free_chunks_.back();
        free_chunks_.pop_back();
    } else {
        ci = (uint32_t)chunks_.size();
        chunks_.emplace_back();
    }
    std::vector<CopyRange> rg;
    rg.reserve(ids.size());
    uint64_t dst = 0;
    for (uint32_t id : ids) {
        Inst &in = inst_[id];
        if (!in.seg_len)
            continue;
        rg.push_back({in.seg_begin, dst, in.seg_len});
        in.levels.push_back({ci, dst, in.seg_len});
        ch.refs++;
        dst += in.seg_len;
    }
    chunks_[ci] = ch;
    lvl_bytes_ += ch.bytes;
    ranges_.reserve(rg.size(), stream_);
    cuda_check(cudaMemcpyAsync(ranges_.p, rg.data(), rg.size() * sizeof(CopyRange),
                               cudaMemcpyHostToDevice, stream_),
               "upload ranges");
    tot_.h2d_bytes += rg.size() * sizeof(CopyRange);
    const int grid = (int)std::min<uint64_t>((rg.size() + 7) / 8, (uint64_t)sms_ * 8);
    launch_copy_ranges(keys_[cur_].p, k64_ ? nullptr : cnts_[cur_].p, ch.keys, ch.cnts, ranges_.p,
                       (uint32_t)rg.size(), grid, stream_);
    cuda_check(cudaGetLastError(), "k_copy_ranges launch");
    tot_.other_launches++;
    // rg is pageable: the upload must have read it before it goes away.
    cuda_check(cudaStreamSynchronize(stream_), "keep levels");
}

void Engine::drop_levels(Inst &in) {
    for (const LevelRef &l : in.levels) {
        LvlChunk &c = chunks_[l.chunk];
        if (--c.refs == 0) {
            if (c.keys)
                cudaFreeAsync(c.keys, stream_);
            if (c.cnts)
                cudaFreeAsync(c.cnts, stream_);
            lvl_bytes_ -= c.bytes;
            c = LvlChunk{};
            free_chunks_.push_back(l.chunk);
        }
    }
    in.levels.clear();
}

void Engine::finish_solve_one(uint32_t id, bool found) {
    Inst &in = inst_[id];
    in.found = found;
    in.result = found ? 1 : 0;
    in.result_ready = true;
    in.active = false;
    in.done = true;
    in.seg_len = 0;
    drop_levels(in);
    n_active_--;
}

void Engine::total_lists(const std::vector<uint32_t> &ids) {
    // A list instance's tilings: the counts of its final level, which stays
    // kept (with every other level) for solutions().
    for (uint32_t id : ids) {
        Inst &in = inst_[id];
        const LevelRef &l = in.levels.back();
        const LvlChunk &c = chunks_[l.chunk];
        unsigned long long sum = 0;
        if (k64_) {
            std::vector<ulonglong2> rec(l.len);
            cuda_check(cudaMemcpyAsync(rec.data(), c.keys + l.first, l.len * sizeof(ulonglong2),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read final level");
            cuda_check(cudaStreamSynchronize(stream_), "read final level");
            for (const auto &r : rec)
                sum += r.y;
        } else {
            std::vector<unsigned long long> cn(l.len);
            cuda_check(cudaMemcpyAsync(cn.data(), c.cnts + l.first,
                                       l.len * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                       stream_),
                       "read final level");
            cuda_check(cudaStreamSynchronize(stream_), "read final level");
            for (auto v : cn)
                sum += v;
        }
        tot_.d2h_bytes += l.len * (k64_ ? 16 : 8);
        in.result = sum;
        in.result_ready = true;
        in.active = false;
        in.done = true;
        in.seg_len = 0;
        n_active_--;
    }
}

void Engine::restart(uint32_t id) {
    // The sampled attempt ended without a tiling: start again from the
    // root with a 16x wider sample (exact from 2^24 states on).
    Inst &in = inst_[id];
    drop_levels(in);
    in.row = 0;
    in.seg_len = 0;
    in.level_sizes.clear();
    in.sampled = false;
    in.growth = 256.0;
    in.beam = in.beam >= (1ull << 20) ? 0 : in.beam * 16;
    in.active = false;
    n_active_--;
    pending_.push_back(id);
    tot_.restarts++;
}

void Engine::trace_solutions(const std::vector<uint32_t> &ids) {
    if (ids.empty())
        return;
    std::vector<TraceJob> jobs;
    std::vector<LevelPtr> lp;
    for (uint32_t id : ids) {
        const Inst &in = inst_[id];
        if (in.levels.size() != (size_t)in.height + 1)
            throw Error(kErrState, "solve-one level store incomplete");
        TraceJob j{};
        j.inst = id;
        j.height = in.height;
        j.lvl = (uint32_t)lp.size();
        j.tag = seg_for(id, 0).tag;
        jobs.push_back(j);
        for (const LevelRef &l : in.levels) {
            const LvlChunk &c = chunks_[l.chunk];
            lp.push_back({c.keys + l.first, c.cnts ? c.cnts + l.first : nullptr, l.len});
        }
    }
    // Flattened passes: the final level of every job (passes 0 and 1),
    // then level H - s of every job with H >= s, for s = 1, 2, ...
    uint32_t hmax = 0;
    for (const TraceJob &j : jobs)
        hmax = std::max(hmax, j.height);
    std::vector<TraceSeg> segs;
    std::vector<std::pair<size_t, unsigned long long>> pass_at;   // (first seg, records)
    for (uint32_t s = 0; s <= hmax; s++) {
        const size_t first = segs.size();
        unsigned long long base = 0;
        for (uint32_t k = 0; k < jobs.size(); k++) {
            if (jobs[k].height < s)
                continue;
            const uint32_t r = jobs[k].height - s;
            const unsigned long long len = lp[jobs[k].lvl + r].len;
            if (!len)
                continue;
            segs.push_back({k, r, base, len});
            base += len;
        }
        pass_at.push_back({first, base});
    }
    jobs_.reserve(jobs.size(), stream_);
    lvlptr_.reserve(lp.size(), stream_);
    trace_out_.reserve(jobs.size(), stream_);
    chain_.reserve(jobs.size(), stream_);
    tsegs_.reserve(std::max<size_t>(segs.size(), 1), stream_);
    cuda_check(cudaMemcpyAsync(jobs_.p, jobs.data(), jobs.size() * sizeof(TraceJob),
                               cudaMemcpyHostToDevice, stream_),
               "upload trace jobs");
    cuda_check(cudaMemcpyAsync(lvlptr_.p, lp.data(), lp.size() * sizeof(LevelPtr),
                               cudaMemcpyHostToDevice, stream_),
               "upload level pointers");
    if (!segs.empty())
        cuda_check(cudaMemcpyAsync(tsegs_.p, segs.data(), segs.size() * sizeof(TraceSeg),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload trace segments");
    cuda_check(cudaMemsetAsync(chain_.p, 0, jobs.size() * sizeof(TraceChain), stream_), "memset");
    tot_.h2d_bytes += jobs.size() * sizeof(TraceJob) + lp.size() * sizeof(LevelPtr) +
                      segs.size() * sizeof(TraceSeg);
    auto pass = [&](int kind, uint32_t s) {
        const size_t first = pass_at[s].first;
        const size_t nseg = (s + 1 < pass_at.size() ? pass_at[s + 1].first : segs.size()) - first;
        const unsigned long long total = pass_at[s].second;
        const int grid = (int)std::min<unsigned long long>((total + 255) / 256,
                                                           (unsigned long long)sms_ * 8);
        launch_trace_pass(k64_, kind, lvlptr_.p, jobs_.p, tsegs_.p + first, (uint32_t)nseg, total,
                          chain_.p, std::max(grid, 1), stream_);
        cuda_check(cudaGetLastError(), "k_trace_pass launch");
        tot_.other_launches++;
    };
    pass(0, 0);
    pass(1, 0);
    for (uint32_t s = 1; s <= hmax; s++)
        pass(2, s);
    const int grid = (int)std::min<uint64_t>((jobs.size() + 7) / 8, (uint64_t)sms_ * 8);
    launch_trace_fill(k64_, insts_.p, plc_.p, lvlptr_.p, jobs_.p, (uint32_t)jobs.size(), chain_.p,
                      trace_out_.p, grid, stream_);
    cuda_check(cudaGetLastError(), "k_trace_fill launch");
    tot_.other_launches++;
    std::vector<TraceOut> out(jobs.size());
    cuda_check(cudaMemcpyAsync(out.data(), trace_out_.p, out.size() * sizeof(TraceOut),
                               cudaMemcpyDeviceToHost, stream_),
               "read trace");
    cuda_check(cudaStreamSynchronize(stream_), "k_trace");
    tot_.d2h_bytes += out.size() * sizeof(TraceOut);
    for (size_t k = 0; k < ids.size(); k++) {
        const uint32_t id = ids[k];
        Inst &in = inst_[id];
        const TraceOut &o = out[k];
        if (o.status != 0) {
            in.active = true;   // fail_instance retires an active instance
            fail_instance(id, kErrState,
                          o.status == 1 ? "solve-one trace: witness without parent"
                                        : "solve-one trace: no fill between kept states");
            continue;
        }
        const uint32_t W = in.width, H = in.height, cells = W * H;
        in.tgrid.assign(cells, -1);
        in.sgrid.assign(cells, -1);
        int step = 0;
        for (uint32_t r = 0; r < H; r++)
            for (uint32_t q = 0; q < o.nfill[r]; q++, step++) {
                const uint32_t pi = o.plc[r][q];
                for (uint64_t bits = in.lib.plc[pi].mask; bits; bits &= bits - 1) {
                    const uint32_t cell = r * W + (uint32_t)__builtin_ctzll(bits);
                    if (cell < cells) {
                        in.tgrid[cell] = (int8_t)in.lib.plc_type[pi];
                        in.sgrid[cell] = (int16_t)step;
                    }
                }
            }
        finish_solve_one(id, true);
    }
}

bool Engine::solution(uint32_t id, int8_t *type_grid, int16_t *step_grid) {
    const Inst &in = inst_.at(id);
    if (in.mode != Mode::SolveOne)
        throw Error(kErrState, "not a solve-one instance");
    if (!in.done)
        throw Error(kErrState, "instance has not finished");
    if (in.status)
        throw Error(in.status, in.error);
    if (!in.found)
        return false;
    if (type_grid)
        std::memcpy(type_grid, in.tgrid.data(), in.tgrid.size());
    if (step_grid)
        std::memcpy(step_grid, in.sgrid.data(), in.sgrid.size() * sizeof(int16_t));
    return true;
}

uint64_t Engine::bucket_count(uint32_t id, uint32_t pattern) {
    EngineScope g(opts_.device, &pool_);
    const Inst &in = inst_.at(id);
    if (!in.active)
        return 0;
    const unsigned long long rowmask = (1ull << in.width) - 1ull;
    if (k64_ && in.lib.dyn_bits < in.width)
        // Single-row pieces only: the current row is the board's, for every state.
        return (in.desc.rows[in.row] & rowmask) == (pattern & rowmask) ? in.seg_len : 0;
    cuda_check(cudaMemsetAsync(nraw_.p, 0, sizeof(unsigned long long), stream_), "memset");
    launch_count_pattern(keys_[cur_].p + in.seg_begin, in.seg_len, rowmask, pattern & rowmask,
                         nraw_.p, sms_ * 4, stream_);
    tot_.other_launches++;
    unsigned long long n = 0;
    cuda_check(cudaMemcpyAsync(&n, nraw_.p, sizeof(n), cudaMemcpyDeviceToHost, stream_),
               "read count");
    cuda_check(cudaStreamSynchronize(stream_), "k_count_pattern");
    return n;
}

void Engine::sync_results() {
    if (unfetched_.empty())
        return;
    EngineScope g(opts_.device, &pool_);
    const uint32_t lo = *std::min_element(unfetched_.begin(), unfetched_.end());
    const uint32_t hi = *std::max_element(unfetched_.begin(), unfetched_.end()) + 1;
    std::vector<unsigned long long> r(hi - lo);
    cuda_check(cudaMemcpyAsync(r.data(), results_.p + lo, r.size() * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, stream_),
               "read results");
    tot_.d2h_bytes += r.size() * sizeof(unsigned long long);
    cuda_check(cudaStreamSynchronize(stream_), "read results");
    for (uint32_t id : unfetched_) {
        inst_[id].result = r[id - lo];
        inst_[id].result_ready = true;
    }
    unfetched_.clear();
}

void Engine::run() {
    while (has_active())
        step();
    sync_results();
}

uint64_t Engine::count(uint32_t id) {
    Inst &in = inst_.at(id);
    if (!in.done)
        throw Error(kErrState, "instance has not finished");
    if (in.status)
        throw Error(in.status, in.error);
    if (!in.result_ready)
        sync_results();
    return in.result;
}

uint64_t Engine::solutions(uint32_t id, uint64_t max, int8_t *type_grids, int16_t *step_grids,
                           bool single) {
    EngineScope g(opts_.device, &pool_);
    Inst &in = inst_.at(id);
    if (!opts_.keep_levels && in.mode != Mode::List)
        throw Error(kErrState,
                    "solutions need an engine created with keep_levels, or a list instance");
    if (!in.done)
        throw Error(kErrState, "instance has not finished");
    const uint32_t H = in.height;
    if (in.row < H || count(id) == 0 || max == 0)
        return 0;
    // The instance's levels: the engine's level store (keep_levels), or the
    // rows kept for this list instance.
    std::vector<ulonglong2 *> lk(H + 1, nullptr);
    std::vector<uint64_t> ln(H + 1, 0);
    if (opts_.keep_levels) {
        if (lvl_n_.size() != (size_t)H + 1)
            throw Error(kErrState, "level store incomplete");
        for (uint32_t r = 0; r <= H; r++) {
            lk[r] = lvl_keys_[r];
            ln[r] = lvl_n_[r];
        }
    } else {
        if (in.levels.size() != (size_t)H + 1)
            throw Error(kErrState, "list level store incomplete");
        for (uint32_t r = 0; r <= H; r++) {
            const LevelRef &l = in.levels[r];
            lk[r] = chunks_[l.chunk].keys + l.first;
            ln[r] = l.len;
        }
    }

    // Backward pass: live[r] = states of level r with a child in live[r + 1].
    std::vector<ulonglong2 *> live(H + 1, nullptr);
    std::vector<uint64_t> live_n(H + 1, 0);
    live[H] = lk[H];
    live_n[H] = ln[H];
    DevBuf<unsigned char> alive;
    DevBuf<unsigned long long> nsel;
    nsel.reserve(1, stream_);
    std::vector<ulonglong2 *> owned;
    auto build_set = [&](const ulonglong2 *recs, uint64_t n) -> uint64_t {
        uint64_t cap = round_up(std::max<uint64_t>(n * 2, 1024), 1024);
        for (;;) {
            const uint64_t units = cap * slot_units();
            if (table_.cap < units) {
                table_.release();
                table_clean_ = 0;
                table_.reserve(units, stream_);
            }
            cuda_check(cudaMemsetAsync(table_.p, 0, units * sizeof(ulonglong2), stream_),
                       "memset");
            cuda_check(cudaMemsetAsync(misc_.p, 0, sizeof(unsigned int), stream_), "memset");
            KeySetArgs t{ table_.p, cap, misc_.p, opts_.max_probe };
            launch_keyset_insert(k64_, t, recs, n, sms_ * 4, stream_);
            unsigned int stt = 0;
            cuda_check(cudaMemcpyAsync(&stt, misc_.p, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                       stream_),
                       "read status");
            cuda_check(cudaStreamSynchronize(stream_), "k_keyset_insert");
            if (!(stt & kStatusTableOverflow))
                return cap;
            cap *= 4;
        }
    };
    auto probe_args = [&](uint32_t r, uint64_t cap) {
        const Seg s = seg_for(id, r);
        ProbeArgs p;
        p.insts = insts_.p;
        p.plc = plc_.p;
        p.inst = id;
        p.row = r;
        p.in_shift = s.in_shift;
        p.hi_board = s.hi_board;
        p.tag = s.tag;
        p.table = table_.p;
        p.cap = cap;
        p.max_probe = opts_.max_probe;
        return p;
    };
    for (int r = (int)H - 1; r >= 0; r--) {
        const uint64_t cap = build_set(live[r + 1], live_n[r + 1]);
        const uint64_t n = ln[r];
        alive.reserve(std::max<uint64_t>(n, 1), stream_);
        launch_mark_alive(k64_, probe_args((uint32_t)r, cap), lk[r], n, alive.p, sms_ * 4,
                          stream_);
        ulonglong2 *out = nullptr;
        cuda_check(cudaMalloc(&out, std::max<uint64_t>(n, 1) * sizeof(ulonglong2)), "cudaMalloc");
        owned.push_back(out);
        cuda_check(cudaMemsetAsync(nsel.p, 0, sizeof(unsigned long long), stream_), "memset");
        launch_select(lk[r], alive.p, n, out, nsel.p, sms_ * 4, stream_);
        unsigned long long ns = 0;
        cuda_check(cudaMemcpyAsync(&ns, nsel.p, sizeof(ns), cudaMemcpyDeviceToHost, stream_),
                   "read select");
        cuda_check(cudaStreamSynchronize(stream_), "select");
        live[r] = out;
        live_n[r] = ns;
    }

    // Forward pass: extend partial tilings row by row through live states.
    const uint32_t max_nodes = (uint32_t)std::min<uint64_t>(single ? 1 : max, 1u << 26);
    std::vector<std::vector<PathNode>> levels(H + 1);
    PathNode root{};
    {
        ulonglong2 rk;
        cuda_check(cudaMemcpyAsync(&rk, lk[0], sizeof(rk), cudaMemcpyDeviceToHost, stream_),
                   "read root");
        cuda_check(cudaStreamSynchronize(stream_), "read root");
        root.k0 = rk.x;
        root.k1 = k64_ ? 0ull : rk.y;
        root.parent = ~0u;
        root.nfill = 0;
    }
    levels[0].push_back(root);
    DevBuf<PathNode> din, dout;
    DevBuf<unsigned int> dn;
    dn.reserve(2, stream_);
    for (uint32_t r = 0; r < H; r++) {
        const uint64_t cap = build_set(live[r + 1], live_n[r + 1]);
        const uint32_t n = (uint32_t)levels[r].size();
        din.reserve(n, stream_);
        dout.reserve(max_nodes, stream_);
        cuda_check(cudaMemcpyAsync(din.p, levels[r].data(), n * sizeof(PathNode),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload nodes");
        cuda_check(cudaMemsetAsync(dn.p, 0, 2 * sizeof(unsigned int), stream_), "memset");
        launch_extend_paths(k64_, probe_args(r, cap), din.p, n, dout.p, dn.p, max_nodes, dn.p + 1,
                            sms_ * 4, stream_);
        unsigned int hn[2] = {0, 0};
        cuda_check(cudaMemcpyAsync(hn, dn.p, sizeof(hn), cudaMemcpyDeviceToHost, stream_),
                   "read nodes");
        cuda_check(cudaStreamSynchronize(stream_), "extend paths");
        const uint32_t got = std::min(hn[0], max_nodes);
        levels[r + 1].resize(got);
        if (got) {
            cuda_check(cudaMemcpyAsync(levels[r + 1].data(), dout.p, got * sizeof(PathNode),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read nodes");
            cuda_check(cudaStreamSynchronize(stream_), "read nodes");
        }
    }
    for (auto p : owned)
        cudaFree(p);
    table_clean_ = 0;   // the table now holds membership sets

    // Leaves -> grids.  Steps are numbered in anchor order (row-major), the
    // order in which the reference's solver places them.
    const uint32_t W = in.width, cells = W * H;
    const auto &lib = in.lib;
    uint64_t produced = 0;
    for (const PathNode &leaf : levels[H]) {
        if (produced >= max)
            break;
        std::vector<const PathNode *> chain(H);
        const PathNode *nd = &leaf;
        for (int r = (int)H; r >= 1; r--) {
            chain[r - 1] = nd;
            nd = r >= 2 ? &levels[r - 1][nd->parent] : nullptr;
        }
        int8_t *tg = type_grids ? type_grids + produced * cells : nullptr;
        int16_t *sg = step_grids ? step_grids + produced * cells : nullptr;
        for (uint32_t cidx = 0; cidx < cells; cidx++) {
            if (tg)
                tg[cidx] = -1;
            if (sg)
                sg[cidx] = -1;
        }
        int step = 0;
        for (uint32_t r = 0; r < H; r++) {
            const PathNode *pn = chain[r];
            for (uint32_t d = 0; d < pn->nfill; d++, step++) {
                const uint32_t pi = pn->plc[d];
                const uint64_t m = lib.plc[pi].mask;
                for (uint64_t bits = m; bits; bits &= bits - 1) {
                    const int b = __builtin_ctzll(bits);
                    const uint32_t cell = r * W + (uint32_t)b;
                    if (cell < cells) {
                        if (tg)
                            tg[cell] = (int8_t)lib.plc_type[pi];
                        if (sg)
                            sg[cell] = (int16_t)step;
                    }
                }
            }
        }
        produced++;
    }
    return produced;
}


void Engine::list_solutions(const std::vector<uint32_t> &ids, uint64_t max_per,
                            std::vector<TilingList> &out) {
    EngineScope g(opts_.device, &pool_);
    out.assign(ids.size(), TilingList{});
    struct Job {
        uint32_t id;
        size_t k;       // index into ids / out
        uint32_t H;
        uint64_t cap;   // tilings to list (partial tilings kept per level)
        std::vector<const ulonglong2 *> lk;   // kept levels
        std::vector<uint64_t> ln;
        std::vector<const ulonglong2 *> live; // states of each level on a tiling
        std::vector<uint64_t> live_n;
        std::vector<std::vector<PathNode>> nodes;   // partial tilings per level
    };
    std::vector<Job> js;
    for (size_t k = 0; k < ids.size(); k++) {
        const uint32_t id = ids[k];
        Inst &in = inst_.at(id);
        if (in.mode != Mode::List)
            throw Error(kErrState, "not a list instance");
        if (!in.done)
            throw Error(kErrState, "instance has not finished");
        if (in.status || in.row < in.height || max_per == 0 || count(id) == 0)
            continue;
        if (in.levels.size() != (size_t)in.height + 1)
            throw Error(kErrState, "list level store incomplete");
        Job j;
        j.id = id;
        j.k = k;
        j.H = in.height;
        j.cap = std::min<uint64_t>(std::min<uint64_t>(max_per, count(id)), 1u << 26);
        for (const LevelRef &l : in.levels) {
            j.lk.push_back(chunks_[l.chunk].keys + l.first);
            j.ln.push_back(l.len);
        }
        j.live.assign(j.H + 1, nullptr);
        j.live_n.assign(j.H + 1, 0);
        j.live[j.H] = j.lk[j.H];
        j.live_n[j.H] = j.ln[j.H];
        j.nodes.resize(j.H + 1);
        js.push_back(std::move(j));
    }
    if (js.empty())
        return;
    uint32_t hmax = 0;
    for (const Job &j : js)
        hmax = std::max(hmax, j.H);

    DevBuf<ListJob> djobs;
    DevBuf<unsigned long long> dcnt;
    DevBuf<unsigned int> dn;
    std::vector<std::unique_ptr<DevBuf<ulonglong2>>> owned;   // live-state buffers
    auto fill_probe = [&](ListJob &lj, const Job &j, uint32_t row) {
        const Seg sg = seg_for(j.id, row);
        lj.inst = j.id;
        lj.row = row;
        lj.in_shift = sg.in_shift;
        lj.hi_board = sg.hi_board;
        lj.tag = sg.tag;
    };
    auto upload_jobs = [&](std::vector<ListJob> &v) -> uint32_t {
        uint32_t b = 0;
        for (ListJob &lj : v) {
            lj.blk_base = b;
            b += list_blocks(lj.n);
        }
        djobs.reserve(v.size(), stream_);
        cuda_check(cudaMemcpyAsync(djobs.p, v.data(), v.size() * sizeof(ListJob),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload list jobs");
        tot_.h2d_bytes += v.size() * sizeof(ListJob);
        return b;
    };
    // Membership set of the given levels' records (all instances in one
    // table: keys carry their instance); returns its capacity.
    auto build_set = [&](const std::vector<std::pair<const ulonglong2 *, uint64_t>> &rg) {
        uint64_t tot = 0;
        std::vector<ListJob> v;
        for (const auto &[recs, n] : rg) {
            tot += n;
            ListJob lj{};
            lj.recs = recs;
            lj.n = n;
            v.push_back(lj);
        }
        uint64_t cap = round_up(std::max<uint64_t>(tot * 2, 1024), 1024);
        for (;;) {
            const uint64_t units = cap * slot_units();
            if (table_.cap < units) {
                table_.release();
                table_clean_ = 0;
                table_.reserve(units, stream_);
            }
            cuda_check(cudaMemsetAsync(table_.p, 0, units * sizeof(ulonglong2), stream_),
                       "memset");
            cuda_check(cudaMemsetAsync(misc_.p, 0, sizeof(unsigned int), stream_), "memset");
            const uint32_t blocks = upload_jobs(v);
            KeySetArgs t{table_.p, cap, misc_.p, opts_.max_probe};
            launch_keyset_insert_jobs(k64_, t, djobs.p, (uint32_t)v.size(), blocks, stream_);
            cuda_check(cudaGetLastError(), "k_keyset_insert_jobs launch");
            tot_.other_launches++;
            unsigned int stt = 0;
            cuda_check(cudaMemcpyAsync(&stt, misc_.p, sizeof(unsigned int),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read status");
            cuda_check(cudaStreamSynchronize(stream_), "k_keyset_insert_jobs");
            if (!(stt & kStatusTableOverflow))
                return cap;
            cap *= 4;
        }
    };
    auto probe_base = [&](uint64_t cap) {
        ProbeArgs p{};
        p.insts = insts_.p;
        p.plc = plc_.p;
        p.table = table_.p;
        p.cap = cap;
        p.max_probe = opts_.max_probe;
        return p;
    };

    // Backward pass, aligned at the instances' last rows: step t marks level
    // H - 1 - t of every instance taller than t, keeping the states with a
    // child among the next level's live states.
    for (uint32_t t = 0; t < hmax; t++) {
        std::vector<size_t> act;
        std::vector<std::pair<const ulonglong2 *, uint64_t>> rg;
        for (size_t q = 0; q < js.size(); q++)
            if (js[q].H > t) {
                act.push_back(q);
                const uint32_t r = js[q].H - 1 - t;
                rg.push_back({js[q].live[r + 1], js[q].live_n[r + 1]});
            }
        const uint64_t cap = build_set(rg);
        std::vector<ListJob> v;
        uint64_t off = 0;
        for (size_t q : act) {
            const Job &j = js[q];
            const uint32_t r = j.H - 1 - t;
            ListJob lj{};
            lj.recs = j.lk[r];
            lj.n = j.ln[r];
            lj.out_off = off;
            lj.out_cap = j.ln[r];
            fill_probe(lj, j, r);
            off += j.ln[r];
            v.push_back(lj);
        }
        owned.push_back(std::make_unique<DevBuf<ulonglong2>>());
        DevBuf<ulonglong2> &dst = *owned.back();
        dst.reserve(std::max<uint64_t>(off, 1), stream_);
        dcnt.reserve(act.size(), stream_);
        cuda_check(cudaMemsetAsync(dcnt.p, 0, act.size() * sizeof(unsigned long long), stream_),
                   "memset");
        const uint32_t blocks = upload_jobs(v);
        launch_mark_select_jobs(k64_, probe_base(cap), djobs.p, (uint32_t)v.size(), blocks, dst.p,
                                dcnt.p, stream_);
        cuda_check(cudaGetLastError(), "k_mark_select_jobs launch");
        tot_.other_launches++;
        std::vector<unsigned long long> cn(act.size());
        cuda_check(cudaMemcpyAsync(cn.data(), dcnt.p, cn.size() * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, stream_),
                   "read live counts");
        cuda_check(cudaStreamSynchronize(stream_), "k_mark_select_jobs");
        for (size_t a = 0; a < act.size(); a++) {
            Job &j = js[act[a]];
            const uint32_t r = j.H - 1 - t;
            j.live[r] = dst.p + v[a].out_off;
            j.live_n[r] = cn[a];
        }
    }

    // Forward pass, aligned at the first row: partial tilings of every
    // instance taller than r extended by one row through live states.
    DevBuf<PathNode> din, dout;
    {
        std::vector<PathNode> roots(js.size());
        for (size_t q = 0; q < js.size(); q++) {
            ulonglong2 rk;
            cuda_check(cudaMemcpyAsync(&rk, js[q].lk[0], sizeof(rk), cudaMemcpyDeviceToHost,
                                       stream_),
                       "read root");
            cuda_check(cudaStreamSynchronize(stream_), "read root");
            PathNode &nd = roots[q];
            nd = PathNode{};
            nd.k0 = rk.x;
            nd.k1 = k64_ ? 0ull : rk.y;
            nd.parent = ~0u;
            nd.nfill = 0;
            js[q].nodes[0].push_back(nd);
        }
        din.reserve(roots.size(), stream_);
        cuda_check(cudaMemcpyAsync(din.p, roots.data(), roots.size() * sizeof(PathNode),
                                   cudaMemcpyHostToDevice, stream_),
                   "upload roots");
        cuda_check(cudaStreamSynchronize(stream_), "upload roots");
    }
    // Node offsets of each instance in din (level r).
    std::vector<uint64_t> in_off(js.size());
    for (size_t q = 0; q < js.size(); q++)
        in_off[q] = q;
    for (uint32_t r = 0; r < hmax; r++) {
        std::vector<size_t> act;
        std::vector<std::pair<const ulonglong2 *, uint64_t>> rg;
        for (size_t q = 0; q < js.size(); q++)
            if (js[q].H > r && !js[q].nodes[r].empty()) {
                act.push_back(q);
                rg.push_back({js[q].live[r + 1], js[q].live_n[r + 1]});
            }
        if (act.empty())
            break;
        const uint64_t cap = build_set(rg);
        std::vector<ListJob> v;
        uint64_t off = 0;
        for (size_t q : act) {
            const Job &j = js[q];
            ListJob lj{};
            lj.nodes = din.p + in_off[q];
            lj.n = j.nodes[r].size();
            lj.out_off = off;
            lj.out_cap = j.cap;
            fill_probe(lj, j, r);
            off += j.cap;
            v.push_back(lj);
        }
        dout.reserve(std::max<uint64_t>(off, 1), stream_);
        dn.reserve(act.size(), stream_);
        cuda_check(cudaMemsetAsync(dn.p, 0, act.size() * sizeof(unsigned int), stream_), "memset");
        cuda_check(cudaMemsetAsync(misc_.p, 0, sizeof(unsigned int), stream_), "memset");
        const uint32_t blocks = upload_jobs(v);
        launch_extend_paths_jobs(k64_, probe_base(cap), djobs.p, (uint32_t)v.size(), blocks,
                                 dout.p, dn.p, misc_.p, stream_);
        cuda_check(cudaGetLastError(), "k_extend_paths_jobs launch");
        tot_.other_launches++;
        std::vector<unsigned int> cn(act.size());
        cuda_check(cudaMemcpyAsync(cn.data(), dn.p, cn.size() * sizeof(unsigned int),
                                   cudaMemcpyDeviceToHost, stream_),
                   "read nodes");
        cuda_check(cudaStreamSynchronize(stream_), "k_extend_paths_jobs");
        // The new partial tilings: one read of the whole output when it is
        // small, else each instance's part.
        const bool bulk = off * sizeof(PathNode) <= (64ull << 20);
        std::vector<PathNode> host(bulk ? off : 0);
        if (bulk) {
            cuda_check(cudaMemcpyAsync(host.data(), dout.p, off * sizeof(PathNode),
                                       cudaMemcpyDeviceToHost, stream_),
                       "read nodes");
            tot_.d2h_bytes += off * sizeof(PathNode);
        }
        for (size_t a = 0; a < act.size(); a++) {
            Job &j = js[act[a]];
            const uint64_t got = std::min<uint64_t>(cn[a], j.cap);
            j.nodes[r + 1].resize(got);
            if (!bulk && got) {
                cuda_check(cudaMemcpyAsync(j.nodes[r + 1].data(), dout.p + v[a].out_off,
                                           got * sizeof(PathNode), cudaMemcpyDeviceToHost,
                                           stream_),
                           "read nodes");
                tot_.d2h_bytes += got * sizeof(PathNode);
            }
            in_off[act[a]] = v[a].out_off;
        }
        cuda_check(cudaStreamSynchronize(stream_), "read nodes");
        if (bulk)
            for (size_t a = 0; a < act.size(); a++) {
                Job &j = js[act[a]];
                std::copy(host.begin() + (std::ptrdiff_t)v[a].out_off,
                          host.begin() + (std::ptrdiff_t)(v[a].out_off + j.nodes[r + 1].size()),
                          j.nodes[r + 1].begin());
            }
        std::swap(din.p, dout.p);
        std::swap(din.cap, dout.cap);
        std::swap(din.s, dout.s);
    }
    owned.clear();
    table_clean_ = 0;   // the table now holds membership sets

    // Leaves -> grids, as solutions() writes them.
    for (Job &j : js) {
        const Inst &in = inst_[j.id];
        const uint32_t W = in.width, H = j.H, cells = W * H;
        const auto &lib = in.lib;
        TilingList &tl = out[j.k];
        const auto &leaves = j.nodes[H];
        const uint64_t n = std::min<uint64_t>(leaves.size(), j.cap);
        tl.n = n;
        tl.types.assign(n * cells, -1);
        tl.steps.assign(n * cells, -1);
        for (uint64_t q = 0; q < n; q++) {
            std::vector<const PathNode *> chain(H);
            const PathNode *nd = &leaves[q];
            for (int r = (int)H; r >= 1; r--) {
                chain[r - 1] = nd;
                nd = r >= 2 ? &j.nodes[r - 1][nd->parent] : nullptr;
            }
            int8_t *tg = tl.types.data() + q * cells;
            int16_t *sg = tl.steps.data() + q * cells;
            int step = 0;
            for (uint32_t r = 0; r < H; r++) {
                const PathNode *pn = chain[r];
                for (uint32_t d = 0; d < pn->nfill; d++, step++) {
                    const uint32_t pi = pn->plc[d];
                    for (uint64_t bits = lib.plc[pi].mask; bits; bits &= bits - 1) {
                        const uint32_t cell = r * W + (uint32_t)__builtin_ctzll(bits);
                        if (cell < cells) {
                            tg[cell] = (int8_t)lib.plc_type[pi];
                            sg[cell] = (int16_t)step;
                        }
                    }
                }
            }
        }
    }
}

}  // namespace d4e
