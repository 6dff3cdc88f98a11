// rmq_api.cu — implementation of the C ABI declared in include/rmq_gb300.h.
//
// Replaces the host drivers xxx_rmq (src/xxx.h:203-298) and
// hierarchical_vector_load (src/xxx.h:932-1040): those validate t, lay out the
// levels, allocate, build, time `reps` query launches with a device-wide sync
// after each, and return a host array.  Here the build and the queries are
// separate, stream-ordered calls; the handle owns the level buffers, the caller
// owns inputs and outputs, and every failure is a status code (the reference
// exits the process on a bad t, src/xxx.h:211-217).
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/rmq_gb300.h"
#include "rmq_internal.h"

using rmq::Layout;

struct rmq_handle {
    Layout lay;
    const float* d_values = nullptr;
    float* val_buf = nullptr;
    uint32_t* idx_buf = nullptr;
    uint64_t* idx_buf64 = nullptr;  // 64-bit handles
    unsigned* counters = nullptr;   // arrival counters of the single-launch build (after the levels)
    bool wide = false;
    uint32_t* err = nullptr;  // invalid-query counter (validate mode)
    int device = 0;
    int variant = RMQ_VARIANT_VL;
    int lanes = 8;
    int with_index = 1;
    int l2_persist = 0;
    int validate = 0;
    size_t persist_bytes = 0;
    float persist_hit_ratio = 1.f;
    float build_ms = 0.f;
    std::mutex validate_mu;

    // Staging of the host-buffer calls (rmq_query_host / rmq_query_idx_host),
    // created on the first such call.
    struct HostPipe {
        static constexpr int kBufs = 3;
        std::mutex mu;
        uint64_t chunk = 0;  // queries per staging buffer
        void* d_q[kBufs] = {};
        float* d_min[kBufs] = {};
        void* d_idx[kBufs] = {};
        cudaStream_t up = nullptr, run = nullptr, down = nullptr;
        cudaEvent_t ev_up[kBufs] = {}, ev_run[kBufs] = {}, ev_down[kBufs] = {};
    } pipe;
};

namespace {

// Variant defaults.  VL: the paper's chosen configuration (rf = 8, t = 32,
// scripts/static_data.py:251-253).  CL: the paper chose 16 lanes x 2 entries
// (rf = 32, t = 64, scripts/get_and_filter_data.py:11); for this CL kernel
// (lanes share whole 32-byte sectors, every lane walks each query's descent)
// the best measured on GB300 is the smallest tile, 2 lanes, with rf = 8 and
// t = 64 (n = q = 2^26: 16.1 G queries/s with argmin, against 10.7 at
// rf = 16 with 4 lanes and 9.4 at rf = 8 with 4 lanes).
constexpr int kClRfLog = 3;
constexpr uint64_t kClT = 64;
constexpr int kClLanes = 2;
constexpr int kVlRfLog = 3;
constexpr uint64_t kVlT = 32;
// AUTO resolves to VL with rf = 8: measured on GB300 it is the fastest
// work distribution at every batch size and array size tried (CL tiles
// repeat each query's descent arithmetic on every lane of the tile).

// Largest n of 32-bit handles: queries are uint32 pairs and the descent rounds
// r up by at most rf - 1 without overflowing 32 bits.  64-bit handles take up
// to 2^40 entries (4 TiB of values, far above any GPU's memory).
constexpr uint64_t kMaxN = 0xFFFFFF00ull;
constexpr uint64_t kMaxNWide = uint64_t(1) << 40;

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
        else prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return RMQ_OK;
    if (e == cudaErrorMemoryAllocation) return RMQ_ERR_OOM;
    return RMQ_ERR_CUDA;
}

int resolve_config(uint64_t n, const rmq_config* cfg_in, int* variant, int* rf_log,
                   uint64_t* t, int* lanes) {
    rmq_config cfg;
    if (cfg_in != nullptr) cfg = *cfg_in;
    else rmq_config_init(&cfg);
    int v = cfg.variant;
    if (v == RMQ_VARIANT_AUTO) v = RMQ_VARIANT_VL;
    // CL and its three ablated work distributions share the CL preconditions.
    const bool cl = v == RMQ_VARIANT_CL || v == RMQ_VARIANT_CL_NO_SHUFFLE || v == RMQ_VARIANT_CL_QUERY_PER_TILE ||
                    v == RMQ_VARIANT_CL_ATOMIC;
    // VL and its short-query form share the VL preconditions.
    const bool vl = v == RMQ_VARIANT_VL || v == RMQ_VARIANT_VL_SHORT;
    if (!cl && !vl) return RMQ_ERR_ARG;
    int r = cfg.rf_log != 0 ? cfg.rf_log : (cl ? kClRfLog : kVlRfLog);
    if (r < 3 || r > 5) return RMQ_ERR_ARG;
    uint64_t tt = cfg.scan_threshold != 0 ? cfg.scan_threshold : (cl ? kClT : kVlT);
    const uint64_t rf = uint64_t(1) << r;
    // The reference's own preconditions (src/xxx.h:211, src/xxx.h:938).
    if (cl && tt < 2 * rf) return RMQ_ERR_ARG;
    if (vl && tt < rf) return RMQ_ERR_ARG;
    // The atomic combine orders a lane's candidates inside a query with 24
    // bits of sector number: pieces of at most 2^27 entries.
    if (v == RMQ_VARIANT_CL_ATOMIC && tt >= (uint64_t(1) << 27)) return RMQ_ERR_UNSUPPORTED;
    int g = cfg.lanes != 0 ? cfg.lanes : kClLanes;
    if (g != 2 && g != 4 && g != 8 && g != 16 && g != 32) return RMQ_ERR_ARG;
    (void)n;
    *variant = v;
    *rf_log = r;
    *t = tt;
    *lanes = g;
    return RMQ_OK;
}

void fill_info(const Layout& lay, int variant, int lanes, rmq_info* info) {
    std::memset(info, 0, sizeof(*info));
    info->index_bits = 32;
    info->num_levels = lay.num_levels;
    info->rf_log = lay.rf_log;
    info->variant = variant;
    info->lanes = lanes;
    info->n = lay.n;
    info->scan_threshold = lay.t;
    for (uint32_t k = 0; k < lay.num_levels && k < 20; ++k) {
        info->level_size[k] = lay.size[k];
        info->level_offset[k] = k == 0 ? ~uint64_t(0) : lay.offset[k];
    }
}

}  // namespace

extern "C" {

void rmq_config_init(rmq_config* cfg) {
    if (cfg == nullptr) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->variant = RMQ_VARIANT_AUTO;
    cfg->with_index = 1;
}

int rmq_debug_bounds_violations(uint64_t* count) {
    if (count == nullptr) return RMQ_ERR_ARG;
    *count = 0;
#if RMQ_DEBUG_BOUNDS
    const unsigned int a = rmq::bounds_bad_query(), b = rmq::bounds_bad_batch();
    if (a == ~0u || b == ~0u) return RMQ_ERR_CUDA;
    *count = uint64_t(a) + b;
    return RMQ_OK;
#else
    return RMQ_ERR_UNSUPPORTED;
#endif
}

const char* rmq_strerror(int status) {
    switch (status) {
        case RMQ_OK: return "ok";
        case RMQ_ERR_ARG: return "invalid argument";
        case RMQ_ERR_CUDA: return "CUDA runtime error";
        case RMQ_ERR_OOM: return "device out of memory";
        case RMQ_ERR_QUERY_RANGE: return "query out of range (l > r or r >= n)";
        case RMQ_ERR_TIMEOUT: return "device-side wait timed out";
        case RMQ_ERR_NO_INDEX: return "handle was built without argmin arrays";
        case RMQ_ERR_UNSUPPORTED: return "unsupported size or configuration";
        default: return "unknown status";
    }
}

int rmq_plan_layout(uint64_t n, uint64_t scan_threshold, int32_t rf_log, int32_t variant,
                    rmq_info* info) {
    if (info == nullptr || n == 0) return RMQ_ERR_ARG;
    if (n > kMaxNWide) return RMQ_ERR_UNSUPPORTED;
    rmq_config cfg;
    rmq_config_init(&cfg);
    cfg.variant = variant;
    cfg.scan_threshold = scan_threshold;
    cfg.rf_log = rf_log;
    int v, r, g;
    uint64_t t;
    const int st = resolve_config(n, &cfg, &v, &r, &t, &g);
    if (st != RMQ_OK) return st;
    const Layout lay = rmq::plan_layout(n, t, uint32_t(r));
    fill_info(lay, v, g, info);
    if (n > kMaxN) info->index_bits = 64;
    return RMQ_OK;
}

int rmq_build(const float* d_values, uint64_t n, const rmq_config* cfg, rmq_stream_t stream,
              rmq_handle** out) {
    rmq::NvtxRange nvtx_range("rmq_build");
    if (out == nullptr) return RMQ_ERR_ARG;
    *out = nullptr;
    if (d_values == nullptr || n == 0) return RMQ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d_values) & 31u) != 0) return RMQ_ERR_ARG;
    if (n > kMaxNWide) return RMQ_ERR_UNSUPPORTED;
    int v, r, g;
    uint64_t t;
    int st = resolve_config(n, cfg, &v, &r, &t, &g);
    if (st != RMQ_OK) return st;
    const int bits = cfg != nullptr ? cfg->index_bits : 0;
    if (bits != 0 && bits != 32 && bits != 64) return RMQ_ERR_ARG;
    const bool wide = bits == 64 || n > kMaxN;
    if (bits == 32 && n > kMaxN) return RMQ_ERR_UNSUPPORTED;
    if (wide && v != RMQ_VARIANT_VL && v != RMQ_VARIANT_VL_SHORT) return RMQ_ERR_UNSUPPORTED;  // 64-bit: VL only

    rmq_handle* h = new (std::nothrow) rmq_handle();
    if (h == nullptr) return RMQ_ERR_OOM;
    if (cudaGetDevice(&h->device) != cudaSuccess) {
        delete h;
        return RMQ_ERR_CUDA;
    }
    h->lay = rmq::plan_layout(n, t, uint32_t(r));
    h->wide = wide;
    h->d_values = d_values;
    h->variant = v;
    h->lanes = g;
    h->with_index = cfg != nullptr ? (cfg->with_index != 0) : 1;
    h->l2_persist = cfg != nullptr ? cfg->l2_persist : 0;
    h->validate = cfg != nullptr ? cfg->validate : 0;

    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (h->lay.num_levels > 1) {
        // One allocation: level values, then argmin indices, so that a single
        // L2 access-policy window can cover both.
        const size_t idx_bytes = h->with_index ? (wide ? sizeof(uint64_t) : sizeof(uint32_t)) : 0;
        const size_t level_bytes = h->lay.total * (sizeof(float) + idx_bytes);
        const size_t counter_bytes = rmq::tail_counters(h->lay) * sizeof(unsigned);
        e = cudaMalloc(&h->val_buf, level_bytes + counter_bytes);
        if (e == cudaSuccess && h->with_index && !wide) h->idx_buf = reinterpret_cast<uint32_t*>(h->val_buf + h->lay.total);
        if (e == cudaSuccess && h->with_index && wide) h->idx_buf64 = reinterpret_cast<uint64_t*>(h->val_buf + h->lay.total);
        if (e == cudaSuccess && counter_bytes > 0) {
            h->counters = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(h->val_buf) + level_bytes);
            e = cudaMemsetAsync(h->counters, 0, counter_bytes, s);
        }
    }
    if (e == cudaSuccess) e = cudaMalloc(&h->err, sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        rmq_destroy(h);
        return cuda_status(e);
    }

    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    if (e == cudaSuccess)
        e = wide ? rmq::launch_build64(h->lay, d_values, h->val_buf, h->idx_buf64, s, h->counters)
                 : rmq::launch_build(h->lay, d_values, h->val_buf, h->idx_buf, s, h->counters);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&h->build_ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rmq_destroy(h);
        return cuda_status(e);
    }

    if (h->l2_persist && h->lay.num_levels > 1) {
        int max_persist = 0, max_window = 0;
        cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, h->device);
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, h->device);
        size_t bytes = h->lay.total * (sizeof(float) + (h->idx_buf ? sizeof(uint32_t) : 0) +
                                       (h->idx_buf64 ? sizeof(uint64_t) : 0));
        if (bytes > size_t(max_window)) bytes = size_t(max_window);
        if (bytes > 0 && max_persist > 0) {
            // Set-aside for persisting lines: the window, up to the device maximum
            // (a context-wide limit, kept if a larger one is already set).
            const size_t want = bytes < size_t(max_persist) ? bytes : size_t(max_persist);
            size_t cur = 0;
            cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize);
            if (cur < want) cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want);
            h->persist_bytes = bytes;
            h->persist_hit_ratio = float(want) / float(bytes);
        }
        cudaGetLastError();
    }
    *out = h;
    return RMQ_OK;
}

// Launch arguments of one query call on device buffers (err left null).
static rmq::QueryArgs query_args(const rmq_handle* h, const void* d_lr, uint64_t q, float* d_min,
                                 void* d_argmin) {
    rmq::QueryArgs a;
    std::memset(&a, 0, sizeof(a));
    for (uint32_t k = 0; k < h->lay.num_levels; ++k) {
        const float* val = k == 0 ? h->d_values : h->val_buf + h->lay.offset[k];
        if (h->wide) {
            a.lv64.val[k] = val;
            a.lv64.idx[k] = (k == 0 || h->idx_buf64 == nullptr) ? nullptr : h->idx_buf64 + h->lay.offset[k];
            a.lv64.size[k] = h->lay.size[k];
        } else {
            a.lv.val[k] = val;
            a.lv.idx[k] = (k == 0 || h->idx_buf == nullptr) ? nullptr : h->idx_buf + h->lay.offset[k];
            a.lv.size[k] = uint32_t(h->lay.size[k]);
        }
    }
    a.lv.num_levels = h->lay.num_levels;
    a.lv64.num_levels = h->lay.num_levels;
    a.wide = h->wide;
    a.q = q;
    a.out_min = d_min;
    if (h->wide) {
        a.qs64 = static_cast<const uint64_t*>(d_lr);
        a.out_idx64 = static_cast<uint64_t*>(d_argmin);
    } else {
        a.qs = static_cast<const uint2*>(d_lr);
        a.out_idx = static_cast<uint32_t*>(d_argmin);
    }
    a.variant = h->variant;
    a.lanes = h->lanes;
    a.rf_log = h->lay.rf_log;
    a.persist_base = h->persist_bytes ? h->val_buf : nullptr;
    a.persist_bytes = h->persist_bytes;
    a.persist_hit_ratio = h->persist_hit_ratio;
    return a;
}

static int query_common(const rmq_handle* hc, const void* d_lr, uint64_t q, float* d_min, void* d_argmin,
                        bool wide_call, rmq_stream_t stream) {
    rmq::NvtxRange nvtx_range("rmq_query");
    if (hc == nullptr) return RMQ_ERR_ARG;
    if (hc->wide != wide_call) return RMQ_ERR_UNSUPPORTED;
    if (q == 0) return RMQ_OK;
    if (!wide_call && q > 0xFFFFFFFFull) return RMQ_ERR_UNSUPPORTED;
    const uintptr_t qalign = wide_call ? 15u : 7u;
    if (d_lr == nullptr || (reinterpret_cast<uintptr_t>(d_lr) & qalign) != 0) return RMQ_ERR_ARG;
    if (d_min == nullptr && d_argmin == nullptr) return RMQ_ERR_ARG;
    // results are stored element by element: each pointer must be aligned to its element
    if ((reinterpret_cast<uintptr_t>(d_min) & 3u) != 0 ||
        (reinterpret_cast<uintptr_t>(d_argmin) & (wide_call ? 7u : 3u)) != 0)
        return RMQ_ERR_ARG;
    if (d_argmin != nullptr && !hc->with_index && hc->lay.num_levels > 1) return RMQ_ERR_NO_INDEX;
    rmq_handle* h = const_cast<rmq_handle*>(hc);
    DeviceGuard guard(h->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    rmq::QueryArgs a = query_args(h, d_lr, q, d_min, d_argmin);

    if (!h->validate) {
        a.err = nullptr;
        return cuda_status(rmq::launch_query(a, s));
    }
    std::lock_guard<std::mutex> lock(h->validate_mu);
    a.err = h->err;
    cudaError_t e = cudaMemsetAsync(h->err, 0, sizeof(uint32_t), s);
    if (e == cudaSuccess) e = rmq::launch_query(a, s);
    uint32_t bad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, h->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e);
    return bad ? RMQ_ERR_QUERY_RANGE : RMQ_OK;
}


// Queries per staging buffer of the host-buffer calls: large enough that the
// per-chunk launch and copy overheads are small against a chunk's kernel
// time, small enough that the first upload and the last download (which
// nothing overlaps) stay short.
#ifndef RMQ_HOST_CHUNK_LOG
#define RMQ_HOST_CHUNK_LOG 22  // tuning knob
#endif
constexpr uint64_t kHostChunk = uint64_t(1) << RMQ_HOST_CHUNK_LOG;

static void free_pipe(rmq_handle::HostPipe& p) {
    for (int b = 0; b < rmq_handle::HostPipe::kBufs; ++b) {
        if (p.d_q[b]) cudaFree(p.d_q[b]);
        if (p.d_min[b]) cudaFree(p.d_min[b]);
        if (p.d_idx[b]) cudaFree(p.d_idx[b]);
        if (p.ev_up[b]) cudaEventDestroy(p.ev_up[b]);
        if (p.ev_run[b]) cudaEventDestroy(p.ev_run[b]);
        if (p.ev_down[b]) cudaEventDestroy(p.ev_down[b]);
        p.d_q[b] = nullptr;
        p.d_min[b] = nullptr;
        p.d_idx[b] = nullptr;
        p.ev_up[b] = p.ev_run[b] = p.ev_down[b] = nullptr;
    }
    if (p.up) cudaStreamDestroy(p.up);
    if (p.run) cudaStreamDestroy(p.run);
    if (p.down) cudaStreamDestroy(p.down);
    p.up = p.run = p.down = nullptr;
    p.chunk = 0;
    cudaGetLastError();
}

// Staging for chunks of `chunk` queries (caller holds p.mu).
// (chunk = 0: streams and events only.)
static cudaError_t ensure_pipe(rmq_handle* h, uint64_t chunk) {
    rmq_handle::HostPipe& p = h->pipe;
    if (p.run != nullptr && p.chunk >= chunk) return cudaSuccess;
    free_pipe(p);
    const size_t qbytes = chunk * (h->wide ? 2 * sizeof(uint64_t) : 2 * sizeof(uint32_t));
    const size_t ibytes = chunk * (h->wide ? sizeof(uint64_t) : sizeof(uint32_t));
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < rmq_handle::HostPipe::kBufs && e == cudaSuccess; ++b) {
        if (chunk > 0) {
            e = cudaMalloc(&p.d_q[b], qbytes);
            if (e == cudaSuccess) e = cudaMalloc(&p.d_min[b], chunk * sizeof(float));
            if (e == cudaSuccess) e = cudaMalloc(&p.d_idx[b], ibytes);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.ev_up[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.ev_run[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.ev_down[b], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p.up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p.run, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p.down, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_pipe(p);
        return e;
    }
    p.chunk = chunk;
    return cudaSuccess;
}

// Device address of host memory [p, p + bytes) that the device can read and
// write directly (page-locked: cudaHostAlloc / cudaHostRegister), aligned to
// `align` bytes; nullptr when any of it is not (the first and the last byte
// must map into one contiguous device range), so such buffers are staged.
static void* mapped_host(const void* p, size_t bytes, uintptr_t align) {
    if (p == nullptr || bytes == 0 || (reinterpret_cast<uintptr_t>(p) & (align - 1)) != 0) return nullptr;
    cudaPointerAttributes a0, a1;
    const char* last = static_cast<const char*>(p) + (bytes - 1);
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || a0.devicePointer == nullptr ||
        a1.devicePointer != static_cast<char*>(a0.devicePointer) + (bytes - 1))
        return nullptr;
    return a0.devicePointer;
}

// Host-buffer queries.  When every host buffer is page-locked, one kernel
// launch reads the queries and writes the results in host memory directly
// (no staging, no copy-engine passes).  Otherwise chunks of the host query
// array are uploaded into one of three device staging buffers, answered and
// downloaded, the upload of chunk c + 1 and the download of chunk c - 1
// overlapping the kernel of chunk c (three streams; a buffer is reused once
// its download is done).
static int query_host_common(const rmq_handle* hc, const void* h_lr, uint64_t q, float* h_min, void* h_argmin,
                             bool wide_call) {
    rmq::NvtxRange nvtx_range("rmq_query_host");
    if (hc == nullptr) return RMQ_ERR_ARG;
    if (hc->wide != wide_call) return RMQ_ERR_UNSUPPORTED;
    if (q == 0) return RMQ_OK;
    if (!wide_call && q > 0xFFFFFFFFull) return RMQ_ERR_UNSUPPORTED;
    if (h_lr == nullptr || (h_min == nullptr && h_argmin == nullptr)) return RMQ_ERR_ARG;
    if (h_argmin != nullptr && !hc->with_index && hc->lay.num_levels > 1) return RMQ_ERR_NO_INDEX;
    rmq_handle* h = const_cast<rmq_handle*>(hc);
    DeviceGuard guard(h->device);
    rmq_handle::HostPipe& p = h->pipe;
    std::lock_guard<std::mutex> lock(p.mu);
    const size_t qsize = wide_call ? 2 * sizeof(uint64_t) : 2 * sizeof(uint32_t);
    const size_t isize = wide_call ? sizeof(uint64_t) : sizeof(uint32_t);

    void* m_lr = mapped_host(h_lr, q * qsize, qsize);
    void* m_min = h_min != nullptr ? mapped_host(h_min, q * sizeof(float), sizeof(float)) : nullptr;
    void* m_idx = h_argmin != nullptr ? mapped_host(h_argmin, q * isize, isize) : nullptr;
    if (m_lr != nullptr && (h_min == nullptr || m_min != nullptr) && (h_argmin == nullptr || m_idx != nullptr)) {
        cudaError_t e = ensure_pipe(h, 0);
        if (e != cudaSuccess) return cuda_status(e);
        std::unique_lock<std::mutex> vlock;
        rmq::QueryArgs a = query_args(h, m_lr, q, static_cast<float*>(m_min), m_idx);
        uint32_t bad = 0;
        if (h->validate) {
            vlock = std::unique_lock<std::mutex>(h->validate_mu);
            a.err = h->err;
            e = cudaMemsetAsync(h->err, 0, sizeof(uint32_t), p.run);
        }
        if (e == cudaSuccess) e = rmq::launch_query(a, p.run);
        if (e == cudaSuccess && h->validate)
            e = cudaMemcpyAsync(&bad, h->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, p.run);
        const cudaError_t es = cudaStreamSynchronize(p.run);
        if (e == cudaSuccess) e = es;
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cuda_status(e);
        }
        return bad ? RMQ_ERR_QUERY_RANGE : RMQ_OK;
    }

    cudaError_t e = ensure_pipe(h, q < kHostChunk ? q : kHostChunk);
    if (e != cudaSuccess) return cuda_status(e);
    const uint64_t chunk = q < p.chunk ? q : p.chunk;
    const char* src = static_cast<const char*>(h_lr);
    char* dst_idx = static_cast<char*>(h_argmin);

    // The error counter is shared with the device-buffer calls in validate mode.
    std::unique_lock<std::mutex> vlock;
    if (h->validate) {
        vlock = std::unique_lock<std::mutex>(h->validate_mu);
        e = cudaMemsetAsync(h->err, 0, sizeof(uint32_t), p.run);
    }
    const uint64_t nchunks = (q + chunk - 1) / chunk;
    for (uint64_t c = 0; c < nchunks && e == cudaSuccess; ++c) {
        const int b = int(c % rmq_handle::HostPipe::kBufs);
        const uint64_t lo = c * chunk;
        const uint64_t m = q - lo < chunk ? q - lo : chunk;
        if (c >= uint64_t(rmq_handle::HostPipe::kBufs)) e = cudaStreamWaitEvent(p.up, p.ev_down[b], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(p.d_q[b], src + lo * qsize, m * qsize, cudaMemcpyHostToDevice, p.up);
        if (e == cudaSuccess) e = cudaEventRecord(p.ev_up[b], p.up);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(p.run, p.ev_up[b], 0);
        if (e == cudaSuccess) {
            rmq::QueryArgs a = query_args(h, p.d_q[b], m, h_min ? p.d_min[b] : nullptr,
                                          h_argmin ? p.d_idx[b] : nullptr);
            a.err = h->validate ? h->err : nullptr;
            e = rmq::launch_query(a, p.run);
        }
        if (e == cudaSuccess) e = cudaEventRecord(p.ev_run[b], p.run);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(p.down, p.ev_run[b], 0);
        if (e == cudaSuccess && h_argmin)
            e = cudaMemcpyAsync(dst_idx + lo * isize, p.d_idx[b], m * isize, cudaMemcpyDeviceToHost, p.down);
        if (e == cudaSuccess && h_min)
            e = cudaMemcpyAsync(h_min + lo, p.d_min[b], m * sizeof(float), cudaMemcpyDeviceToHost, p.down);
        if (e == cudaSuccess) e = cudaEventRecord(p.ev_down[b], p.down);
    }
    uint32_t bad = 0;
    if (e == cudaSuccess && h->validate) {
        e = cudaStreamWaitEvent(p.down, p.ev_run[int((nchunks - 1) % rmq_handle::HostPipe::kBufs)], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, h->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, p.down);
    }
    // Drain all three streams even after a failure: staging buffers must be idle.
    const cudaError_t e1 = cudaStreamSynchronize(p.up);
    const cudaError_t e2 = cudaStreamSynchronize(p.run);
    const cudaError_t e3 = cudaStreamSynchronize(p.down);
    if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_status(e);
    }
    return bad ? RMQ_ERR_QUERY_RANGE : RMQ_OK;
}

int rmq_query_host(const rmq_handle* h, const uint32_t* h_lr, uint64_t q, float* h_min) {
    if (h_min == nullptr) return RMQ_ERR_ARG;
    return query_host_common(h, h_lr, q, h_min, nullptr, false);
}

int rmq_query_idx_host(const rmq_handle* h, const uint32_t* h_lr, uint64_t q, uint32_t* h_argmin,
                       float* h_min_or_null) {
    if (h_argmin == nullptr) return RMQ_ERR_ARG;
    return query_host_common(h, h_lr, q, h_min_or_null, h_argmin, false);
}

int rmq_query64_host(const rmq_handle* h, const uint64_t* h_lr, uint64_t q, float* h_min) {
    if (h_min == nullptr) return RMQ_ERR_ARG;
    return query_host_common(h, h_lr, q, h_min, nullptr, true);
}

int rmq_query_idx64_host(const rmq_handle* h, const uint64_t* h_lr, uint64_t q, uint64_t* h_argmin,
                         float* h_min_or_null) {
    if (h_argmin == nullptr) return RMQ_ERR_ARG;
    return query_host_common(h, h_lr, q, h_min_or_null, h_argmin, true);
}

int rmq_query(const rmq_handle* h, const uint32_t* d_lr, uint64_t q, float* d_min,
              rmq_stream_t stream) {
    if (d_min == nullptr) return RMQ_ERR_ARG;
    return query_common(h, d_lr, q, d_min, nullptr, false, stream);
}

int rmq_query_idx(const rmq_handle* h, const uint32_t* d_lr, uint64_t q, uint32_t* d_argmin,
                  float* d_min_or_null, rmq_stream_t stream) {
    if (d_argmin == nullptr) return RMQ_ERR_ARG;
    return query_common(h, d_lr, q, d_min_or_null, d_argmin, false, stream);
}

int rmq_query64(const rmq_handle* h, const uint64_t* d_lr, uint64_t q, float* d_min,
                rmq_stream_t stream) {
    if (d_min == nullptr) return RMQ_ERR_ARG;
    return query_common(h, d_lr, q, d_min, nullptr, true, stream);
}

int rmq_query_idx64(const rmq_handle* h, const uint64_t* d_lr, uint64_t q, uint64_t* d_argmin,
                    float* d_min_or_null, rmq_stream_t stream) {
    if (d_argmin == nullptr) return RMQ_ERR_ARG;
    return query_common(h, d_lr, q, d_min_or_null, d_argmin, true, stream);
}

int rmq_scan_bruteforce(const float* d_values, uint64_t n, const uint32_t* d_lr, uint64_t q,
                        float* d_min_or_null, uint32_t* d_argmin_or_null, rmq_stream_t stream) {
    if (q == 0) return RMQ_OK;
    if (d_values == nullptr || n == 0 || d_lr == nullptr) return RMQ_ERR_ARG;
    if (d_min_or_null == nullptr && d_argmin_or_null == nullptr) return RMQ_ERR_ARG;
    if (n > kMaxN || q > 0xFFFFFFFFull) return RMQ_ERR_UNSUPPORTED;
    if ((reinterpret_cast<uintptr_t>(d_lr) & 7u) != 0 || (reinterpret_cast<uintptr_t>(d_values) & 3u) != 0 ||
        (reinterpret_cast<uintptr_t>(d_min_or_null) & 3u) != 0 ||
        (reinterpret_cast<uintptr_t>(d_argmin_or_null) & 3u) != 0)
        return RMQ_ERR_ARG;
    return cuda_status(rmq::launch_bruteforce(d_values, uint32_t(n), reinterpret_cast<const uint2*>(d_lr),
                                              uint32_t(q), d_min_or_null, d_argmin_or_null,
                                              reinterpret_cast<cudaStream_t>(stream)));
}

int rmq_get_info(const rmq_handle* h, rmq_info* info) {
    if (h == nullptr || info == nullptr) return RMQ_ERR_ARG;
    fill_info(h->lay, h->variant, h->lanes, info);
    info->index_bits = h->wide ? 64 : 32;
    info->level_bytes = h->lay.num_levels > 1
                            ? h->lay.total * (sizeof(float) + (h->idx_buf ? sizeof(uint32_t) : 0) +
                                              (h->idx_buf64 ? sizeof(uint64_t) : 0))
                            : 0;
    info->build_ms = h->build_ms;
    return RMQ_OK;
}

void rmq_destroy(rmq_handle* h) {
    if (h == nullptr) return;
    {
        DeviceGuard guard(h->device);
        free_pipe(h->pipe);
        if (h->val_buf) cudaFree(h->val_buf);
        if (h->err) cudaFree(h->err);
        cudaGetLastError();
    }
    delete h;
}

}  // extern "C"
