// rmq_serve.cu — the range-minimum query server (include/rmq_gb300_serve.h).
//
// State: an arena (one cudaMalloc of the HBM budget, first-fit free list,
// 256-byte granules) holding every resident array's values, coarse levels and
// argmin arrays; a table of registered arrays (resident or evicted); a FIFO of
// pending requests; S slots, each a stream with pinned and device staging
// for one batch.
//
// Dispatcher thread (continuous batching): reaps finished slots (copies
// results into the requests' host buffers, unpins arrays, wakes waiters),
// marks admitted arrays ready when their build event completes, and whenever
// a slot is free packs the pending requests whose arrays are ready (FIFO, up
// to max_batch_queries) into it and launches: one H2D of descriptors, work
// units and queries, one query kernel (the batched per-warp kernel, one
// descriptor per request), one D2H of the results, event.  Requests arriving while batches run are
// admitted into the next free slot, so up to S batches overlap on the device
// with builds of newly admitted arrays on their own stream.
//
// Admission: an array is placed in the arena when registered or, after an
// eviction, when a request needs it; if it does not fit, idle arrays (built,
// no batch in flight) are evicted least recently used first.  Generated
// arrays are re-admitted by regenerating their values from the seed, host
// arrays by re-uploading.  No device-side waits: all synchronisation is host
// polling of CUDA events.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>
#if defined(__linux__)
#include <sys/prctl.h>
#endif

#include "../../include/rmq_gb300_batch.h"
#include "../../include/rmq_gb300_serve.h"
#include "rmq_arena.h"
#include "rmq_internal.h"

namespace {

using Clock = std::chrono::steady_clock;
using rmq::Arena;

struct ServedArray {
    uint64_t n = 0, seed = 0;
    const float* host = nullptr;
    rmq::Layout lay;
    uint64_t bytes = 0, val_bytes = 0, lvl_bytes = 0;
    bool resident = false, ready = false, admitted_before = false;
    uint64_t off = 0;  // arena byte offset
    int pins = 0;
    uint64_t last_use = 0;
    cudaEvent_t built = nullptr;
};

struct Request {
    uint64_t array = 0;
    const uint32_t* h_lr = nullptr;
    uint64_t q = 0;
    uint32_t* h_idx = nullptr;
    float* h_min = nullptr;
    // Page-locked request buffers: their device-side addresses, through which
    // the kernel reads the queries and writes the results in place.
    bool direct = false;
    const uint32_t* d_lr = nullptr;
    uint32_t* d_idx = nullptr;
    float* d_min = nullptr;
    Clock::time_point t_submit, t_done;
    int status = RMQ_OK;
    bool done = false;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    // One upload and one download per batch: in = descs | q_off | unit_off |
    // io | owner of each 32-query unit | the staged requests' queries (sized
    // by the batch); out = invalid-query count per request | the staged
    // requests' argmin | their minima.  Requests with page-locked buffers
    // are read and written in place and take no staging.
    uint8_t* h_in = nullptr;   // pinned
    uint8_t* h_out = nullptr;  // pinned
    uint8_t* d_in = nullptr;
    uint8_t* d_out = nullptr;
    uint64_t snq = 0;          // staged queries of the batch in flight
    uint32_t nr = 0;
    std::vector<uint64_t> reqs;
    std::vector<Request*> rptr;     // stable element pointers (taken under the lock)
    std::vector<uint64_t> req_off;  // staged query offset of each staged request
    bool busy = false;
};

// Bytes of a batch's header for nr requests, rounded to 16 (the owner table
// follows), of its owner table for `units` work units (the staged queries
// follow), and of the invalid-query counts at the head of the download.
size_t header_bytes(uint32_t nr) {
    const size_t b = size_t(nr) * sizeof(rmq::ArrayDesc) + 2 * size_t(nr + 1) * sizeof(uint64_t) +
                     size_t(nr) * sizeof(rmq::ServeIO);
    return (b + 15) & ~size_t(15);
}
size_t owner_bytes(uint64_t units) { return (units * sizeof(uint32_t) + 15) & ~size_t(15); }
size_t bad_bytes(uint32_t nr) { return (size_t(nr) * sizeof(uint32_t) + 15) & ~size_t(15); }

// The device-side address of page-locked host memory [p, p + bytes), or null
// when that range is not wholly page-locked and mapped (or p is null).
void* mapped_range(const void* p, size_t bytes, size_t align) {
    if (p == nullptr || bytes == 0 || (reinterpret_cast<uintptr_t>(p) & (align - 1)) != 0) return nullptr;
    cudaPointerAttributes a0, a1;
    const char* last = static_cast<const char*>(p) + bytes - 1;
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || a0.devicePointer == nullptr ||
        a1.devicePointer != static_cast<char*>(a0.devicePointer) + (bytes - 1))
        return nullptr;
    return a0.devicePointer;
}

}  // namespace

struct rmq_server {
    rmq_server_config cfg;
    int device = 0;
    uint8_t* arena = nullptr;
    Arena alloc;
    std::vector<ServedArray> arrays;
    // Requests by id, kept until their waiter has collected the outcome (or
    // the server is destroyed); unordered_map keeps element addresses stable.
    std::unordered_map<uint64_t, Request> requests;
    uint64_t next_request = 0;
    std::deque<uint64_t> pending;
    std::vector<uint64_t> admitting;
    std::vector<Slot> slots;
    cudaStream_t build_stream = nullptr;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread dispatcher;
    bool stop = false;
    uint64_t use_clock = 0;
    uint64_t not_done = 0;
    uint32_t fail_batches = 0;  // injected launch failures still to come
    rmq_server_stats stats{};
};

namespace {

rmq::ArrayDesc describe(const ServedArray& a) {
    rmq::ArrayDesc d;
    std::memset(&d, 0, sizeof(d));
    d.val_off = a.off / 4;
    d.lvl_base = (a.off + a.val_bytes) / 4;
    d.idx_base = (a.off + a.val_bytes + a.lvl_bytes) / 4;
    d.num_levels = a.lay.num_levels;
    for (uint32_t k = 0; k < a.lay.num_levels; ++k) {
        d.size[k] = uint32_t(a.lay.size[k]);
        d.off[k] = k == 0 ? 0u : uint32_t(a.lay.offset[k]);
    }
    return d;
}

void evict(rmq_server* s, uint64_t id) {
    ServedArray& a = s->arrays[id];
    s->alloc.release(a.off, a.bytes);
    a.resident = false;
    a.ready = false;
    s->stats.evictions++;
    s->stats.resident_arrays--;
    s->stats.resident_bytes -= a.bytes;
}

// Places array id in the arena (evicting idle arrays, least recently used
// first) and enqueues its values and build on the build stream.  Holds mu.
bool admit(rmq_server* s, uint64_t id) {
    ServedArray& a = s->arrays[id];
    uint64_t off = 0;
    while (!s->alloc.alloc(a.bytes, &off)) {
        const uint64_t victim = rmq::lru_victim(s->arrays, id);
        if (victim == ~uint64_t(0)) return false;
        evict(s, victim);
    }
    a.off = off;
    a.resident = true;
    a.ready = false;
    a.last_use = ++s->use_clock;
    float* vals = reinterpret_cast<float*>(s->arena + a.off);
    float* lvl = reinterpret_cast<float*>(s->arena + a.off + a.val_bytes);
    uint32_t* idx = reinterpret_cast<uint32_t*>(s->arena + a.off + a.val_bytes + a.lvl_bytes);
    int st = RMQ_OK;
    if (a.host != nullptr) {
        st = cudaMemcpyAsync(vals, a.host, a.n * sizeof(float), cudaMemcpyHostToDevice, s->build_stream) ==
                     cudaSuccess ? RMQ_OK : RMQ_ERR_CUDA;
    } else {
        st = rmq_gen_values_device(vals, a.n, a.seed, reinterpret_cast<rmq_stream_t>(s->build_stream));
    }
    if (st == RMQ_OK && rmq::launch_build(a.lay, vals, lvl, idx, s->build_stream) != cudaSuccess) st = RMQ_ERR_CUDA;
    if (st == RMQ_OK && cudaEventRecord(a.built, s->build_stream) != cudaSuccess) st = RMQ_ERR_CUDA;
    if (st != RMQ_OK) {
        cudaGetLastError();
        s->alloc.release(a.off, a.bytes);
        a.resident = false;
        return false;
    }
    if (a.admitted_before) s->stats.readmissions++;
    a.admitted_before = true;
    s->stats.resident_arrays++;
    s->stats.resident_bytes += a.bytes;
    s->admitting.push_back(id);
    return true;
}

// Copies a finished slot's results out and completes its requests.  Called
// without mu held (the slot and its requests belong to the dispatcher).  With
// `failed` set (the batch's launch failed) every request of the slot gets
// that status and all-ones argmin / NaN minima instead of results; the status
// is set under mu together with `done`, so a waiter never sees one without
// the other.
void finish_slot(rmq_server* s, Slot& sl, int failed = RMQ_OK) {
    std::vector<int> status(sl.reqs.size(), failed);
    const uint32_t* bad = reinterpret_cast<const uint32_t*>(sl.h_out);
    const uint32_t* h_idx = reinterpret_cast<const uint32_t*>(sl.h_out + bad_bytes(sl.nr));
    const float* h_min = reinterpret_cast<const float*>(sl.h_out + bad_bytes(sl.nr) + sl.snq * sizeof(uint32_t));
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
        Request& r = *sl.rptr[i];
        if (failed != RMQ_OK) {
            for (uint64_t j = 0; j < r.q; ++j) {
                if (r.h_idx != nullptr) r.h_idx[j] = rmq::kNoPos;
                if (r.h_min != nullptr) r.h_min[j] = std::numeric_limits<float>::quiet_NaN();
            }
            continue;
        }
        if (bad[i] != 0) status[i] = RMQ_ERR_QUERY_RANGE;
        if (r.direct) continue;  // results already in place
        const uint64_t o = sl.req_off[i];
        if (r.h_idx != nullptr) std::memcpy(r.h_idx, h_idx + o, r.q * sizeof(uint32_t));
        if (r.h_min != nullptr) std::memcpy(r.h_min, h_min + o, r.q * sizeof(float));
    }
    const Clock::time_point now = Clock::now();
    std::lock_guard<std::mutex> lock(s->mu);
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
        Request& r = *sl.rptr[i];
        r.status = status[i];
        r.t_done = now;
        r.done = true;
        ServedArray& a = s->arrays[r.array];
        a.pins--;
        a.last_use = ++s->use_clock;
        s->stats.requests_done++;
        s->stats.queries_done += r.q;
        s->not_done--;
    }
    sl.reqs.clear();
    sl.rptr.clear();
    sl.busy = false;
    s->cv_done.notify_all();
}

// Packs ready pending requests into a free slot and launches the batch.
// Called with `lk` held; releases it while packing and launching.
bool launch_batch(rmq_server* s, Slot& sl, std::unique_lock<std::mutex>& lk) {
    rmq::NvtxRange nvtx_range("rmq_server_batch");
    const uint64_t max_q = s->cfg.max_batch_queries;
    const uint32_t max_r = s->cfg.max_batch_requests;
    uint64_t nq = 0;
    sl.reqs.clear();
    sl.rptr.clear();
    sl.req_off.clear();
    for (auto it = s->pending.begin(); it != s->pending.end() && sl.reqs.size() < max_r;) {
        Request& r = s->requests.at(*it);
        ServedArray& a = s->arrays[r.array];
        if (!a.resident && !admit(s, r.array)) {
            ++it;  // waits for memory to free up
            continue;
        }
        if (!a.ready) {
            ++it;  // still building
            continue;
        }
        if (nq + r.q > max_q) break;
        sl.reqs.push_back(*it);
        sl.rptr.push_back(&r);
        nq += r.q;
        a.pins++;
        it = s->pending.erase(it);
    }
    if (sl.reqs.empty()) return false;
    sl.busy = true;
    uint64_t busy = 0;
    for (const Slot& x : s->slots) busy += x.busy ? 1 : 0;
    if (busy > s->stats.max_batches_in_flight) s->stats.max_batches_in_flight = busy;
    if (sl.reqs.size() > s->stats.max_requests_per_batch) s->stats.max_requests_per_batch = sl.reqs.size();
    s->stats.batches++;
    const uint32_t nr = uint32_t(sl.reqs.size());
    std::vector<rmq::ArrayDesc> descs(nr);
    std::vector<const Request*> reqs(sl.rptr.begin(), sl.rptr.end());
    for (uint32_t i = 0; i < nr; ++i) descs[i] = describe(s->arrays[reqs[i]->array]);
    const bool inject = s->fail_batches > 0;
    if (inject) s->fail_batches--;
    lk.unlock();

    // Upload: descriptors | q_off[nr + 1] | unit_off[nr + 1] | io[nr] |
    // owner of each unit | the staged requests' queries.
    const size_t hdr = header_bytes(nr);
    rmq::ArrayDesc* hd = reinterpret_cast<rmq::ArrayDesc*>(sl.h_in);
    uint64_t* hq = reinterpret_cast<uint64_t*>(sl.h_in + size_t(nr) * sizeof(rmq::ArrayDesc));
    uint64_t* hu = hq + (nr + 1);
    rmq::ServeIO* hio = reinterpret_cast<rmq::ServeIO*>(hu + (nr + 1));
    std::memcpy(hd, descs.data(), nr * sizeof(rmq::ArrayDesc));
    hq[0] = 0;
    hu[0] = 0;
    for (uint32_t i = 0; i < nr; ++i) {
        hq[i + 1] = hq[i] + reqs[i]->q;
        hu[i + 1] = hu[i] + (reqs[i]->q + 31) / 32;
    }
    uint32_t* h_owner = reinterpret_cast<uint32_t*>(sl.h_in + hdr);
    const size_t qat = hdr + owner_bytes(hu[nr]);
    uint32_t* h_q = reinterpret_cast<uint32_t*>(sl.h_in + qat);
    // staged requests' queries and results are packed in request order
    uint64_t snq = 0;
    sl.req_off.assign(nr, 0);
    for (uint32_t i = 0; i < nr; ++i) {
        if (!reqs[i]->direct) {
            sl.req_off[i] = snq;
            snq += reqs[i]->q;
        }
    }
    const size_t bb = bad_bytes(nr);
    uint32_t* d_idx = reinterpret_cast<uint32_t*>(sl.d_out + bb);
    float* d_min = reinterpret_cast<float*>(sl.d_out + bb + snq * sizeof(uint32_t));
    for (uint32_t i = 0; i < nr; ++i) {
        for (uint64_t u = hu[i]; u < hu[i + 1]; ++u) h_owner[u] = i;
        const Request& r = *reqs[i];
        if (r.direct) {
            hio[i] = rmq::ServeIO{reinterpret_cast<const uint2*>(r.d_lr), r.d_idx, r.d_min};
        } else {
            const uint64_t o = sl.req_off[i];
            std::memcpy(h_q + 2 * o, r.h_lr, r.q * 2 * sizeof(uint32_t));
            hio[i] = rmq::ServeIO{reinterpret_cast<const uint2*>(sl.d_in + qat) + o,
                                  r.h_idx != nullptr ? d_idx + o : nullptr, r.h_min != nullptr ? d_min + o : nullptr};
        }
    }
    const rmq::ArrayDesc* dd = reinterpret_cast<const rmq::ArrayDesc*>(sl.d_in);
    const uint64_t* dq = reinterpret_cast<const uint64_t*>(sl.d_in + size_t(nr) * sizeof(rmq::ArrayDesc));
    const uint64_t* du = dq + (nr + 1);
    sl.snq = snq;
    sl.nr = nr;
    // An injected failure (rmq_server_fail_next_batches) stands in for a
    // failing upload: nothing is issued and the batch takes the error path.
    cudaError_t e = inject ? cudaErrorInvalidConfiguration
                           : cudaMemcpyAsync(sl.d_in, sl.h_in, qat + snq * 2 * sizeof(uint32_t),
                                             cudaMemcpyHostToDevice, sl.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_out, 0, bb, sl.stream);
    if (e == cudaSuccess) {
        rmq::ServeQueryArgs a;
        a.values = reinterpret_cast<const float*>(s->arena);
        a.descs = dd;
        a.owner = reinterpret_cast<const uint32_t*>(sl.d_in + hdr);
        a.unit_off = du;
        a.q_off = dq;
        a.total_units = hu[nr];
        a.lvl_val = reinterpret_cast<const float*>(s->arena);
        a.lvl_idx = reinterpret_cast<const uint32_t*>(s->arena);
        a.io = reinterpret_cast<const rmq::ServeIO*>(du + (nr + 1));
        a.bad = reinterpret_cast<uint32_t*>(sl.d_out);
        a.threads = s->cfg.query_threads;
        e = rmq::launch_serve_query(a, sl.stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.h_out, sl.d_out, bb + snq * 8, cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, sl.stream);
    if (e != cudaSuccess) {
        // Launch failure: the batch's requests complete with RMQ_ERR_CUDA.
        cudaGetLastError();
        cudaStreamSynchronize(sl.stream);
        finish_slot(s, sl, RMQ_ERR_CUDA);
        lk.lock();
        return true;
    }
    lk.lock();
    return true;
}

void dispatcher_main(rmq_server* s) {
    cudaSetDevice(s->device);
#if defined(__linux__)
    // The dispatcher polls in-flight batches every 4 us; with Linux's default
    // 50 us timer slack each of those waits would last ~55 us, and that delay
    // lands on every request's latency.
    prctl(PR_SET_TIMERSLACK, 1UL, 0UL, 0UL, 0UL);
#endif
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        bool progressed = false;
        for (Slot& sl : s->slots) {
            if (sl.busy && cudaEventQuery(sl.done) == cudaSuccess) {
                lk.unlock();
                finish_slot(s, sl);
                lk.lock();
                progressed = true;
            }
        }
        for (size_t i = 0; i < s->admitting.size();) {
            ServedArray& a = s->arrays[s->admitting[i]];
            if (cudaEventQuery(a.built) == cudaSuccess) {
                a.ready = true;
                s->admitting[i] = s->admitting.back();
                s->admitting.pop_back();
                progressed = true;
            } else {
                ++i;
            }
        }
        cudaGetLastError();  // cudaEventQuery's cudaErrorNotReady
        if (!s->pending.empty()) {
            for (Slot& sl : s->slots) {
                if (!sl.busy && !s->pending.empty()) {
                    if (!launch_batch(s, sl, lk)) break;
                    progressed = true;
                }
            }
        }
        bool any_busy = false;
        for (const Slot& sl : s->slots) any_busy |= sl.busy;
        if (s->stop && !any_busy && (s->pending.empty() || s->admitting.empty())) {
            // Stopping: requests that can never be admitted are failed.
            if (!s->pending.empty() && s->admitting.empty() && !progressed) {
                for (uint64_t rid : s->pending) {
                    Request& r = s->requests.at(rid);
                    r.status = RMQ_ERR_OOM;
                    r.done = true;
                    r.t_done = Clock::now();
                    s->not_done--;
                }
                s->pending.clear();
                s->cv_done.notify_all();
            }
            if (s->pending.empty()) break;
        }
        if (!progressed) s->cv_work.wait_for(lk, std::chrono::microseconds(any_busy || !s->admitting.empty() ? 4 : 200));
    }
}

int register_array(rmq_server* s, uint64_t n, uint64_t seed, const float* host, uint64_t* id) {
    if (s == nullptr || id == nullptr || n == 0) return RMQ_ERR_ARG;
    if (n > 0xFFFFFF00ull) return RMQ_ERR_UNSUPPORTED;
    ServedArray a;
    a.n = n;
    a.seed = seed;
    a.host = host;
    a.lay = rmq::plan_layout(n, s->cfg.scan_threshold, 3);
    a.val_bytes = rmq::arena_round_up(n * sizeof(float));
    const uint64_t lvl_entries = a.lay.num_levels > 1 ? a.lay.total : 0;
    a.lvl_bytes = rmq::arena_round_up(lvl_entries * sizeof(float));
    a.bytes = a.val_bytes + 2 * a.lvl_bytes;
    if (a.bytes > s->cfg.hbm_budget_bytes) return RMQ_ERR_OOM;
    if (cudaEventCreateWithFlags(&a.built, cudaEventDisableTiming) != cudaSuccess) return RMQ_ERR_CUDA;
    std::lock_guard<std::mutex> lock(s->mu);
    *id = s->arrays.size();
    s->arrays.push_back(a);
    s->stats.registrations++;
    admit(s, *id);  // if it does not fit now, a request admits it later
    s->cv_work.notify_one();
    return RMQ_OK;
}

}  // namespace

extern "C" {

void rmq_server_config_init(rmq_server_config* cfg) {
    if (cfg == nullptr) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->hbm_budget_bytes = uint64_t(64) << 30;
    cfg->slots = 4;
    cfg->max_batch_queries = uint64_t(1) << 21;
    cfg->max_batch_requests = 4096;
    cfg->scan_threshold = 64;
    cfg->query_threads = 256;
}

int rmq_server_create(const rmq_server_config* cfg_in, rmq_server** out) {
    if (out == nullptr) return RMQ_ERR_ARG;
    *out = nullptr;
    rmq_server_config cfg;
    rmq_server_config_init(&cfg);
    if (cfg_in != nullptr) {
        if (cfg_in->hbm_budget_bytes) cfg.hbm_budget_bytes = cfg_in->hbm_budget_bytes;
        if (cfg_in->slots) cfg.slots = cfg_in->slots;
        if (cfg_in->max_batch_queries) cfg.max_batch_queries = cfg_in->max_batch_queries;
        if (cfg_in->max_batch_requests) cfg.max_batch_requests = cfg_in->max_batch_requests;
        if (cfg_in->scan_threshold) cfg.scan_threshold = cfg_in->scan_threshold;
        if (cfg_in->query_threads) cfg.query_threads = cfg_in->query_threads;
    }
    if (cfg.scan_threshold < 8 || cfg.max_batch_queries < (uint64_t(1) << 16) || cfg.slots > 64 ||
        cfg.query_threads % 32 != 0 || cfg.query_threads > 512)
        return RMQ_ERR_ARG;
    rmq_server* s = new (std::nothrow) rmq_server();
    if (s == nullptr) return RMQ_ERR_OOM;
    s->cfg = cfg;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = cudaMalloc(&s->arena, cfg.hbm_budget_bytes);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->build_stream, cudaStreamNonBlocking);
    s->alloc.init(cfg.hbm_budget_bytes);
    s->slots.resize(cfg.slots);
    const uint64_t mq = cfg.max_batch_queries;
    const uint32_t mr = cfg.max_batch_requests;
    for (Slot& sl : s->slots) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        const size_t in_bytes = header_bytes(mr) + owner_bytes(mq / 32 + mr) + mq * 2 * sizeof(uint32_t);
        const size_t out_bytes = bad_bytes(mr) + mq * 8;
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_in, in_bytes);
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_out, out_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_in, in_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_out, out_bytes);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        rmq_server_destroy(s);
        return e == cudaErrorMemoryAllocation ? RMQ_ERR_OOM : RMQ_ERR_CUDA;
    }
    s->dispatcher = std::thread(dispatcher_main, s);
    *out = s;
    return RMQ_OK;
}

int rmq_server_register_generated(rmq_server* s, uint64_t n, uint64_t seed, uint64_t* array_id) {
    return register_array(s, n, seed, nullptr, array_id);
}

int rmq_server_register_host(rmq_server* s, const float* h_values, uint64_t n, uint64_t* array_id) {
    if (h_values == nullptr) return RMQ_ERR_ARG;
    return register_array(s, n, 0, h_values, array_id);
}

int rmq_server_submit(rmq_server* s, uint64_t array_id, const uint32_t* h_lr, uint64_t q, uint32_t* h_argmin,
                      float* h_min, uint64_t* request_id) {
    if (s == nullptr || request_id == nullptr || (h_argmin == nullptr && h_min == nullptr)) return RMQ_ERR_ARG;
    if (q == 0 || h_lr == nullptr || q > s->cfg.max_batch_queries) return RMQ_ERR_ARG;
    Request r;
    r.array = array_id;
    r.h_lr = h_lr;
    r.q = q;
    r.h_idx = h_argmin;
    r.h_min = h_min;
    // Page-locked, mapped request buffers are read and written in place by
    // the kernel (no staging copies); anything else is staged.
    r.d_lr = static_cast<const uint32_t*>(mapped_range(h_lr, q * 2 * sizeof(uint32_t), 8));
    r.d_idx = static_cast<uint32_t*>(mapped_range(h_argmin, q * sizeof(uint32_t), 4));
    r.d_min = static_cast<float*>(mapped_range(h_min, q * sizeof(float), 4));
    r.direct = r.d_lr != nullptr && (h_argmin == nullptr || r.d_idx != nullptr) &&
               (h_min == nullptr || r.d_min != nullptr);
    std::lock_guard<std::mutex> lock(s->mu);
    if (array_id >= s->arrays.size() || s->stop) return RMQ_ERR_ARG;
    if (r.direct) s->stats.direct_requests++;
    r.t_submit = Clock::now();
    *request_id = s->next_request++;
    s->requests.emplace(*request_id, r);
    s->pending.push_back(*request_id);
    s->not_done++;
    s->cv_work.notify_one();
    return RMQ_OK;
}

int rmq_server_wait(rmq_server* s, uint64_t request_id, int64_t timeout_ms, double* latency_us) {
    if (s == nullptr) return RMQ_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return RMQ_ERR_ARG;  // unknown, or already collected
    const Request& r = it->second;
    auto done = [&] { return r.done; };
    if (timeout_ms < 0) s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return RMQ_ERR_TIMEOUT;
    if (latency_us != nullptr)
        *latency_us = std::chrono::duration<double, std::micro>(r.t_done - r.t_submit).count();
    const int status = r.status;
    s->requests.erase(it);  // collected: the id is no longer valid
    return status;
}

int rmq_server_drain(rmq_server* s, int64_t timeout_ms) {
    if (s == nullptr) return RMQ_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&] { return s->not_done == 0; };
    if (timeout_ms < 0) s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return RMQ_ERR_TIMEOUT;
    return RMQ_OK;
}

int rmq_server_replay(rmq_server* s, const rmq_trace_event* ev, uint64_t count, const uint32_t* h_lr,
                      uint32_t* h_argmin, float* h_min, double* latency_us, double* wall_s) {
    if (s == nullptr || (count > 0 && ev == nullptr)) return RMQ_ERR_ARG;
    std::vector<uint64_t> rid(count, ~uint64_t(0));
    const Clock::time_point t0 = Clock::now();
    for (uint64_t i = 0; i < count; ++i) {
        const Clock::time_point due = t0 + std::chrono::duration_cast<Clock::duration>(
                                               std::chrono::duration<double>(ev[i].t_arrival_s));
        for (;;) {
            const Clock::time_point now = Clock::now();
            if (now >= due) break;
            if (due - now > std::chrono::microseconds(200)) std::this_thread::sleep_for(due - now - std::chrono::microseconds(100));
        }
        if (ev[i].kind == 1) {
            uint64_t id;
            rmq_server_register_generated(s, ev[i].n, ev[i].seed, &id);
        } else {
            uint64_t r;
            if (rmq_server_submit(s, ev[i].array_id, h_lr + 2 * ev[i].q_offset, ev[i].q,
                                  h_argmin != nullptr ? h_argmin + ev[i].q_offset : nullptr,
                                  h_min != nullptr ? h_min + ev[i].q_offset : nullptr, &r) == RMQ_OK)
                rid[i] = r;
        }
    }
    const int st = rmq_server_drain(s, -1);
    Clock::time_point first = Clock::time_point::max(), last = t0;
    std::lock_guard<std::mutex> lock(s->mu);
    for (uint64_t i = 0; i < count; ++i) {
        if (rid[i] == ~uint64_t(0)) {
            if (latency_us) latency_us[i] = -1.0;
            continue;
        }
        auto it = s->requests.find(rid[i]);
        if (it == s->requests.end()) {
            if (latency_us) latency_us[i] = -1.0;
            continue;
        }
        const Request& r = it->second;
        if (latency_us) latency_us[i] = std::chrono::duration<double, std::micro>(r.t_done - r.t_submit).count();
        if (r.t_submit < first) first = r.t_submit;
        if (r.t_done > last) last = r.t_done;
        s->requests.erase(it);  // the replay collects its own requests
    }
    if (wall_s) *wall_s = first == Clock::time_point::max() ? 0.0 : std::chrono::duration<double>(last - first).count();
    return st;
}

int rmq_serve_serial_loop(rmq_handle* const* handles, uint64_t num_handles, const rmq_trace_event* ev,
                          uint64_t count, const uint32_t* h_lr, uint32_t* h_argmin, float* h_min, double* wall_s) {
    if (handles == nullptr || (count > 0 && (ev == nullptr || h_lr == nullptr || h_argmin == nullptr)))
        return RMQ_ERR_ARG;
    const Clock::time_point t0 = Clock::now();
    int first_error = RMQ_OK;
    for (uint64_t i = 0; i < count; ++i) {
        if (ev[i].kind != 0) continue;
        if (ev[i].array_id >= num_handles || handles[ev[i].array_id] == nullptr) return RMQ_ERR_ARG;
        const uint64_t o = ev[i].q_offset;
        const int st = rmq_query_idx_host(handles[ev[i].array_id], h_lr + 2 * o, ev[i].q, h_argmin + o,
                                          h_min != nullptr ? h_min + o : nullptr);
        if (st != RMQ_OK && first_error == RMQ_OK) first_error = st;
    }
    if (wall_s != nullptr) *wall_s = std::chrono::duration<double>(Clock::now() - t0).count();
    return first_error;
}

int rmq_server_fail_next_batches(rmq_server* s, uint32_t count) {
    if (s == nullptr) return RMQ_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    s->fail_batches = count;
    return RMQ_OK;
}

int rmq_server_get_stats(rmq_server* s, rmq_server_stats* stats) {
    if (s == nullptr || stats == nullptr) return RMQ_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    *stats = s->stats;
    return RMQ_OK;
}

void rmq_server_destroy(rmq_server* s) {
    if (s == nullptr) return;
    if (s->dispatcher.joinable()) {
        {
            std::lock_guard<std::mutex> lock(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        s->dispatcher.join();
    }
    int prev = -1;
    if (cudaGetDevice(&prev) == cudaSuccess && prev != s->device) cudaSetDevice(s->device);
    else prev = -1;
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        cudaFreeHost(sl.h_in);
        cudaFreeHost(sl.h_out);
        cudaFree(sl.d_in);
        cudaFree(sl.d_out);
    }
    if (s->build_stream) {
        cudaStreamSynchronize(s->build_stream);
        cudaStreamDestroy(s->build_stream);
    }
    for (ServedArray& a : s->arrays)
        if (a.built) cudaEventDestroy(a.built);
    cudaFree(s->arena);
    cudaGetLastError();
    if (prev >= 0) cudaSetDevice(prev);
    delete s;
}

}  // extern "C"
