// rmq_batch.cu — batched build and queries over many independent arrays
// (include/rmq_gb300_batch.h).
//
// Packed layout: every array keeps its values where the caller put them
// (d_values + value_offsets[a]); all coarse levels of all arrays live in one
// value buffer and one argmin buffer, array a's levels starting at lvl_base[a]
// with the single-array layout (src/xxx.h:225-243 rule, rf = 8).  A device
// descriptor table gives each CTA its array.
//
// Work lists: the build's fused kernel runs one CTA per 8192-entry tile of any
// array (tile -> array by binary search over tile offsets), a tail kernel one
// CTA per array; the query kernel one warp per 32 queries of one array.  Build + queries can be captured as one CUDA graph.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/rmq_gb300_batch.h"
#include "rmq_buildk.cuh"
#include "rmq_internal.h"
#include "rmq_vl.cuh"

namespace rmq {

// Largest a in [0, num) with offs[a] <= x, for non-decreasing offs with
// offs[0] = 0 <= x < offs[num]; arrays owning no work are skipped.
__device__ __forceinline__ uint32_t find_owner(const uint64_t* __restrict__ offs, uint32_t num, uint64_t x) {
    uint32_t lo = 0, hi = num;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (offs[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void fill_levelout(const ArrayDesc& d, float* lvl_val, uint32_t* lvl_idx, LevelOut& lo) {
    for (uint32_t k = 0; k < uint32_t(kMaxLevels); ++k) {
        const bool has = k > 0 && k < d.num_levels;
        lo.val[k] = has ? lvl_val + d.lvl_base + d.off[k] : nullptr;
        lo.idx[k] = (has && lvl_idx != nullptr) ? lvl_idx + d.idx_base + d.off[k] : nullptr;
        lo.size[k] = k < d.num_levels ? d.size[k] : 0u;
    }
}

template <int R>
__global__ void __launch_bounds__(kFusedThreads)
batch_fused_kernel(const float* __restrict__ values, const ArrayDesc* __restrict__ descs,
                   const uint64_t* __restrict__ tile_off, uint32_t num_arrays, float* lvl_val,
                   uint32_t* lvl_idx) {
    __shared__ float sv[kTileSectors];
    __shared__ uint32_t sp[kTileSectors];
    __shared__ LevelOut lo;
    __shared__ const float* s_a;
    __shared__ uint32_t s_n, s_depth, s_tile;
    if (threadIdx.x == 0) {
        const uint32_t a = find_owner(tile_off, num_arrays, blockIdx.x);
        const ArrayDesc& d = descs[a];
        fill_levelout(d, lvl_val, lvl_idx, lo);
        s_a = values + d.val_off;
        s_n = d.size[0];
        s_tile = uint32_t(blockIdx.x - tile_off[a]);
        const uint32_t top = d.num_levels - 1u;
        s_depth = top < fused_depth<R>() ? top : fused_depth<R>();
    }
    __syncthreads();
    if (s_depth > 0) fused_tile<R>(s_a, s_n, lo, s_depth, s_tile, sv, sp);
}

template <int R>
__global__ void __launch_bounds__(256)
batch_tail_kernel(const ArrayDesc* __restrict__ descs, float* lvl_val, uint32_t* lvl_idx) {
    __shared__ LevelOut lo;
    __shared__ uint32_t s_from, s_last;
    if (threadIdx.x == 0) {
        const ArrayDesc& d = descs[blockIdx.x];
        fill_levelout(d, lvl_val, lvl_idx, lo);
        s_last = d.num_levels - 1u;
        s_from = s_last < fused_depth<R>() ? s_last : fused_depth<R>();
    }
    __syncthreads();
    if (s_from < s_last) tail_levels<R>(lo, s_from, s_last);
}

// Work unit of the query kernel: 32 consecutive queries of one array, owned
// by one warp (a loop over several units per warp made the compiler keep the
// unit's level pointers in registers: 62-75 instead of 40).  unit_owner[u]
// (filled on the device by fill_owner_kernel) names the array, so a warp's
// prologue is two dependent loads; the descriptor is unpacked by 20 lanes at
// once into the warp's own shared Levels, and no CTA-wide barrier is needed.
constexpr uint32_t kUnitQueries = 32;
constexpr uint32_t kMaxQueryThreads = 512;

__global__ void fill_owner_kernel(const uint64_t* __restrict__ unit_off, uint32_t* __restrict__ owner) {
    const uint32_t a = blockIdx.x;
    const uint64_t u0 = unit_off[a], u1 = unit_off[a + 1];
    for (uint64_t u = u0 + threadIdx.x; u < u1; u += blockDim.x) owner[u] = a;
}

template <int R, bool ARGMIN>
__global__ void __launch_bounds__(kMaxQueryThreads)
batch_query_kernel(const float* __restrict__ values, const ArrayDesc* __restrict__ descs,
                   const uint32_t* __restrict__ unit_owner, const uint64_t* __restrict__ unit_off,
                   const uint64_t* __restrict__ q_off, uint64_t total_units,
                   const float* __restrict__ lvl_val, const uint32_t* __restrict__ lvl_idx,
                   const uint2* __restrict__ qs, float* __restrict__ out_min, uint32_t* __restrict__ out_idx) {
    __shared__ Levels wlv[kMaxQueryThreads / 32];
    __shared__ uint64_t wq[kMaxQueryThreads / 32][2];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t unit = uint64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
    if (unit >= total_units) return;  // the whole warp leaves
    const uint32_t a = __ldg(unit_owner + unit);
    const ArrayDesc& d = descs[a];
    Levels& lv = wlv[warp];
    const uint32_t nl = d.num_levels;
    if (lane < uint32_t(kMaxLevels)) {
        const uint32_t k = lane;
        const bool has = k > 0 && k < nl;
        lv.val[k] = k == 0 ? values + d.val_off : (has ? lvl_val + d.lvl_base + d.off[k] : nullptr);
        lv.idx[k] = (has && lvl_idx != nullptr) ? lvl_idx + d.idx_base + d.off[k] : nullptr;
        lv.size[k] = k < nl ? d.size[k] : 0u;
    } else if (lane == 31) {
        lv.num_levels = nl;
        const uint64_t q0 = q_off[a] + (unit - unit_off[a]) * kUnitQueries;
        const uint64_t qe = q0 + kUnitQueries;
        const uint64_t q1 = q_off[a + 1];
        wq[warp][0] = q0;
        wq[warp][1] = qe < q1 ? qe : q1;
    }
    __syncwarp();
    const uint32_t cnt = uint32_t(wq[warp][1] - wq[warp][0]);
    const bool in_range = lane < cnt;
    uint2 Q = make_uint2(1u, 0u);
    if (in_range) Q = ld_query(qs + wq[warp][0] + lane);
    float v;
    uint32_t idx;
    const bool valid = vl_compute<R, ARGMIN>(lv, Q, in_range, v, idx);
    const uint64_t at = wq[warp][0] + lane;  // base re-read after the descent
    vl_store<ARGMIN>(in_range, valid, v, idx, out_min != nullptr ? out_min + at : nullptr,
                     ARGMIN ? out_idx + at : nullptr, nullptr);
}

// The served batch's kernel: as batch_query_kernel, but every entry (a
// request) reads its queries and writes its results through its own ServeIO
// (staging buffers or the request's page-locked host buffers), and counts
// its invalid queries so the host needs no pass over the results.
template <int R>
__global__ void __launch_bounds__(kMaxQueryThreads)
serve_query_kernel(const float* __restrict__ values, const ArrayDesc* __restrict__ descs,
                   const uint32_t* __restrict__ unit_owner, const uint64_t* __restrict__ unit_off,
                   const uint64_t* __restrict__ q_off, uint64_t total_units,
                   const float* __restrict__ lvl_val, const uint32_t* __restrict__ lvl_idx,
                   const ServeIO* __restrict__ io, uint32_t* __restrict__ bad) {
    __shared__ Levels wlv[kMaxQueryThreads / 32];
    __shared__ uint64_t wq[kMaxQueryThreads / 32][2];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t unit = uint64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
    if (unit >= total_units) return;  // the whole warp leaves
    const uint32_t a = __ldg(unit_owner + unit);
    const ArrayDesc& d = descs[a];
    Levels& lv = wlv[warp];
    const uint32_t nl = d.num_levels;
    if (lane < uint32_t(kMaxLevels)) {
        const uint32_t k = lane;
        const bool has = k > 0 && k < nl;
        lv.val[k] = k == 0 ? values + d.val_off : (has ? lvl_val + d.lvl_base + d.off[k] : nullptr);
        lv.idx[k] = (has && lvl_idx != nullptr) ? lvl_idx + d.idx_base + d.off[k] : nullptr;
        lv.size[k] = k < nl ? d.size[k] : 0u;
    } else if (lane == 31) {
        lv.num_levels = nl;
        const uint64_t q0 = (unit - unit_off[a]) * kUnitQueries;  // local to the request
        const uint64_t qe = q0 + kUnitQueries;
        const uint64_t q1 = q_off[a + 1] - q_off[a];
        wq[warp][0] = q0;
        wq[warp][1] = qe < q1 ? qe : q1;
    }
    __syncwarp();
    const ServeIO r = io[a];
    const uint64_t q0 = wq[warp][0];
    const uint32_t cnt = uint32_t(wq[warp][1] - q0);
    const bool in_range = lane < cnt;
    uint2 Q = make_uint2(1u, 0u);
    if (in_range) Q = ld_query(r.qs + q0 + lane);
    float v;
    uint32_t idx;
    const bool valid = vl_compute<R, true>(lv, Q, in_range, v, idx);
    if (in_range) {
        if (r.out_min != nullptr) st_stream(r.out_min + q0 + lane, v);
        if (r.out_idx != nullptr) st_stream(r.out_idx + q0 + lane, idx);
    }
    const uint32_t nbad = __popc(__ballot_sync(0xffffffffu, in_range && !valid));
    if (lane == 0 && nbad != 0) atomicAdd(bad + a, nbad);
}

cudaError_t launch_serve_query(const ServeQueryArgs& a, cudaStream_t s) {
    if (a.total_units == 0) return cudaSuccess;
    const uint32_t warps = a.threads / 32u;
    const uint32_t grid = uint32_t((a.total_units + warps - 1) / warps);
    serve_query_kernel<3><<<grid, a.threads, 0, s>>>(a.values, a.descs, a.owner, a.unit_off, a.q_off,
                                                     a.total_units, a.lvl_val, a.lvl_idx, a.io, a.bad);
    return cudaGetLastError();
}

cudaError_t launch_fill_owner(const uint64_t* unit_off, uint32_t num, uint32_t* owner, cudaStream_t s) {
    if (num == 0) return cudaSuccess;
    fill_owner_kernel<<<num, 256, 0, s>>>(unit_off, owner);
    return cudaGetLastError();
}

#if RMQ_DEBUG_BOUNDS
RMQ_BOUNDS_COUNTER_READER(bounds_bad_batch)
#endif

cudaError_t launch_batch_query(const BatchQueryArgs& a, cudaStream_t s) {
    if (a.total_units == 0) return cudaSuccess;
    const uint32_t warps = a.threads / 32u;
    const uint32_t grid = uint32_t((a.total_units + warps - 1) / warps);
    if (a.out_idx != nullptr) {
        batch_query_kernel<3, true><<<grid, a.threads, 0, s>>>(a.values, a.descs, a.owner, a.unit_off, a.q_off,
                                                               a.total_units, a.lvl_val, a.lvl_idx, a.qs,
                                                               a.out_min, a.out_idx);
    } else {
        batch_query_kernel<3, false><<<grid, a.threads, 0, s>>>(a.values, a.descs, a.owner, a.unit_off, a.q_off,
                                                                a.total_units, a.lvl_val, a.lvl_idx, a.qs,
                                                                a.out_min, nullptr);
    }
    return cudaGetLastError();
}

}  // namespace rmq

using rmq::ArrayDesc;

struct rmq_batch {
    const float* d_values = nullptr;
    uint32_t num_arrays = 0;
    std::vector<uint64_t> val_off, sizes;
    uint64_t t = 64;        // scan threshold of the largest size class (the batch-wide t when uniform)
    uint64_t tc[3] = {64, 64, 64};  // scan threshold per size class (rmq_batch_info.class_upper)
    uint32_t qblock = 128;  // threads per CTA of the query kernel (untuned default)
    int with_index = 1;
    int device = 0;
    // levels
    float* lvl_val = nullptr;
    uint32_t* lvl_idx = nullptr;
    uint64_t lvl_capacity = 0;  // entries
    uint64_t lvl_used = 0;
    uint32_t max_levels = 1;
    ArrayDesc* d_descs = nullptr;
    uint64_t* d_tile_off = nullptr;
    uint64_t total_tiles = 0;
    // queries
    std::vector<uint64_t> q_off;
    uint64_t* d_q_off = nullptr;
    uint64_t* d_blk_off = nullptr;  // work-unit offsets per array
    uint32_t* d_owner = nullptr;    // array of every work unit
    uint64_t owner_capacity = 0;
    uint64_t total_blocks = 0;      // work units
    const uint32_t* d_lr = nullptr;
    uint32_t* d_argmin = nullptr;
    float* d_min = nullptr;
    bool queries_set = false;
    std::vector<ArrayDesc> h_descs;  // host copy of the descriptors (per-array loop)
    // graph + timing
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool build_timed = false;
    float build_ms = 0.f, query_ms = 0.f;
};

namespace {

constexpr uint64_t kBatchDefaultT = 64;
constexpr uint64_t kTuneT[] = {16, 32, 64, 256, 1024};
// Size classes of the per-class thresholds: arrays below 2^14 entries, below
// 2^18, and the rest.
constexpr int kClasses = 3;
constexpr uint64_t kClassUpper[kClasses] = {uint64_t(1) << 14, uint64_t(1) << 18, ~uint64_t(0)};

int size_class(uint64_t n) {
    int c = 0;
    while (c + 1 < kClasses && n >= kClassUpper[c]) ++c;
    return c;
}
constexpr uint32_t kTuneBlock[] = {64, 128, 256, 512};  // threads per CTA of the query kernel

int status_of(cudaError_t e) {
    if (e == cudaSuccess) return RMQ_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? RMQ_ERR_OOM : RMQ_ERR_CUDA;
}

uint64_t layout_entries(uint64_t n, uint64_t t) {
    const rmq::Layout lay = rmq::plan_layout(n, t, 3);
    return lay.num_levels > 1 ? lay.total : 0;
}

void drop_graph(rmq_batch* b) {
    if (b->graph != nullptr) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
}

// Lays out every array with its size class's threshold tc[class], uploads
// descriptors and tile offsets.
int plan(rmq_batch* b, const uint64_t (&tc)[kClasses], cudaStream_t s) {
    std::vector<ArrayDesc> descs(b->num_arrays);
    std::vector<uint64_t> tile_off(b->num_arrays + 1, 0);
    uint64_t base = 0;
    uint32_t max_levels = 1;
    for (uint32_t a = 0; a < b->num_arrays; ++a) {
        const rmq::Layout lay = rmq::plan_layout(b->sizes[a], tc[size_class(b->sizes[a])], 3);
        ArrayDesc& d = descs[a];
        std::memset(&d, 0, sizeof(d));
        d.val_off = b->val_off[a];
        d.lvl_base = base;
        d.idx_base = base;
        d.num_levels = lay.num_levels;
        for (uint32_t k = 0; k < lay.num_levels; ++k) {
            d.size[k] = uint32_t(lay.size[k]);
            d.off[k] = k == 0 ? 0u : uint32_t(lay.offset[k]);
        }
        if (lay.num_levels > 1) base += lay.total;
        max_levels = std::max(max_levels, lay.num_levels);
        const uint64_t tiles = lay.num_levels > 1 ? (b->sizes[a] + rmq::kTile - 1) / rmq::kTile : 0;
        tile_off[a + 1] = tile_off[a] + tiles;
    }
    if (base > b->lvl_capacity) return RMQ_ERR_UNSUPPORTED;
    cudaError_t e = cudaMemcpyAsync(b->d_descs, descs.data(), sizeof(ArrayDesc) * b->num_arrays,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_tile_off, tile_off.data(), sizeof(uint64_t) * (b->num_arrays + 1),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // tile_off dies here; descs are kept
    if (e != cudaSuccess) return status_of(e);
    b->h_descs.swap(descs);
    for (int c = 0; c < kClasses; ++c) b->tc[c] = tc[c];
    b->t = tc[kClasses - 1];
    b->lvl_used = base;
    b->max_levels = max_levels;
    b->total_tiles = tile_off[b->num_arrays];
    drop_graph(b);
    return RMQ_OK;
}

int plan(rmq_batch* b, uint64_t t, cudaStream_t s) {
    const uint64_t tc[kClasses] = {t, t, t};
    return plan(b, tc, s);
}

int upload_blocks(rmq_batch* b, cudaStream_t s) {
    std::vector<uint64_t> blk(b->num_arrays + 1, 0);
    for (uint32_t a = 0; a < b->num_arrays; ++a) {
        const uint64_t qa = b->q_off[a + 1] - b->q_off[a];
        blk[a + 1] = blk[a] + (qa + rmq::kUnitQueries - 1) / rmq::kUnitQueries;
    }
    const uint64_t units = blk[b->num_arrays];
    cudaError_t e = cudaSuccess;
    if (units > b->owner_capacity) {
        if (b->d_owner != nullptr) cudaFree(b->d_owner);
        b->d_owner = nullptr;
        b->owner_capacity = 0;
        e = cudaMalloc(&b->d_owner, sizeof(uint32_t) * units);
        if (e != cudaSuccess) return status_of(e);
        b->owner_capacity = units;
    }
    e = cudaMemcpyAsync(b->d_blk_off, blk.data(), sizeof(uint64_t) * (b->num_arrays + 1),
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && units > 0) e = rmq::launch_fill_owner(b->d_blk_off, b->num_arrays, b->d_owner, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return status_of(e);
    b->total_blocks = units;
    drop_graph(b);
    return RMQ_OK;
}

cudaError_t enqueue_build(rmq_batch* b, cudaStream_t s) {
    if (b->total_tiles == 0) return cudaSuccess;
    rmq::batch_fused_kernel<3><<<uint32_t(b->total_tiles), rmq::kFusedThreads, 0, s>>>(
        b->d_values, b->d_descs, b->d_tile_off, b->num_arrays, b->lvl_val, b->lvl_idx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (b->max_levels - 1 > rmq::fused_depth<3>()) {
        rmq::batch_tail_kernel<3><<<b->num_arrays, 256, 0, s>>>(b->d_descs, b->lvl_val, b->lvl_idx);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t enqueue_query(rmq_batch* b, cudaStream_t s) {
    rmq::BatchQueryArgs a;
    a.values = b->d_values;
    a.descs = b->d_descs;
    a.owner = b->d_owner;
    a.unit_off = b->d_blk_off;
    a.q_off = b->d_q_off;
    a.total_units = b->total_blocks;
    a.lvl_val = b->lvl_val;
    a.lvl_idx = b->lvl_idx;
    a.qs = reinterpret_cast<const uint2*>(b->d_lr);
    a.out_min = b->d_min;
    a.out_idx = b->d_argmin;
    a.threads = b->qblock;
    return rmq::launch_batch_query(a, s);
}

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

}  // namespace

extern "C" {

int rmq_batch_create(const float* d_values, const uint64_t* value_offsets, const uint64_t* sizes,
                     uint32_t num_arrays, const rmq_config* cfg, rmq_stream_t stream, rmq_batch** out) {
    if (out == nullptr) return RMQ_ERR_ARG;
    *out = nullptr;
    if (d_values == nullptr || value_offsets == nullptr || sizes == nullptr || num_arrays == 0) return RMQ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d_values) & 31u) != 0) return RMQ_ERR_ARG;
    for (uint32_t a = 0; a < num_arrays; ++a) {
        if (sizes[a] == 0 || (value_offsets[a] & 7u) != 0) return RMQ_ERR_ARG;
        if (sizes[a] > 0xFFFFFF00ull) return RMQ_ERR_UNSUPPORTED;
    }
    const uint64_t t = (cfg != nullptr && cfg->scan_threshold != 0) ? cfg->scan_threshold : kBatchDefaultT;
    if (t < 8) return RMQ_ERR_ARG;  // VL precondition t >= rf (src/xxx.h:938)
    if (cfg != nullptr && cfg->rf_log != 0 && cfg->rf_log != 3) return RMQ_ERR_UNSUPPORTED;

    rmq_batch* b = new (std::nothrow) rmq_batch();
    if (b == nullptr) return RMQ_ERR_OOM;
    if (cudaGetDevice(&b->device) != cudaSuccess) {
        delete b;
        return RMQ_ERR_CUDA;
    }
    b->d_values = d_values;
    b->num_arrays = num_arrays;
    b->val_off.assign(value_offsets, value_offsets + num_arrays);
    b->sizes.assign(sizes, sizes + num_arrays);
    b->with_index = cfg != nullptr ? (cfg->with_index != 0) : 1;
    // capacity: the deepest layout among the user's t and the tuner's candidates
    uint64_t cap = 0;
    for (uint32_t a = 0; a < num_arrays; ++a) {
        uint64_t m = layout_entries(sizes[a], t);
        for (uint64_t ct : kTuneT) m = std::max(m, layout_entries(sizes[a], ct));
        cap += m;
    }
    b->lvl_capacity = cap;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (cap > 0) {
        e = cudaMalloc(&b->lvl_val, cap * sizeof(float));
        if (e == cudaSuccess && b->with_index) e = cudaMalloc(&b->lvl_idx, cap * sizeof(uint32_t));
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_descs, sizeof(ArrayDesc) * num_arrays);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tile_off, sizeof(uint64_t) * (num_arrays + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_q_off, sizeof(uint64_t) * (num_arrays + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_blk_off, sizeof(uint64_t) * (num_arrays + 1));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    int st = status_of(e);
    if (st == RMQ_OK) st = plan(b, t, s);
    if (st != RMQ_OK) {
        rmq_batch_destroy(b);
        return st;
    }
    *out = b;
    return RMQ_OK;
}

int rmq_batch_set_queries(rmq_batch* b, const uint32_t* d_lr, const uint64_t* query_offsets,
                          uint32_t* d_argmin, float* d_min, rmq_stream_t stream) {
    if (b == nullptr || query_offsets == nullptr) return RMQ_ERR_ARG;
    if (d_argmin == nullptr && d_min == nullptr) return RMQ_ERR_ARG;
    if (d_argmin != nullptr && !b->with_index) return RMQ_ERR_NO_INDEX;
    if (query_offsets[0] != 0) return RMQ_ERR_ARG;
    for (uint32_t a = 0; a < b->num_arrays; ++a)
        if (query_offsets[a + 1] < query_offsets[a]) return RMQ_ERR_ARG;
    const uint64_t total = query_offsets[b->num_arrays];
    if (total > 0 && (d_lr == nullptr || (reinterpret_cast<uintptr_t>(d_lr) & 7u) != 0)) return RMQ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d_argmin) & 3u) != 0 || (reinterpret_cast<uintptr_t>(d_min) & 3u) != 0)
        return RMQ_ERR_ARG;  // results are stored element by element
    DeviceGuard guard(b->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    b->q_off.assign(query_offsets, query_offsets + b->num_arrays + 1);
    cudaError_t e = cudaMemcpyAsync(b->d_q_off, b->q_off.data(), sizeof(uint64_t) * (b->num_arrays + 1),
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return status_of(e);
    b->d_lr = d_lr;
    b->d_argmin = d_argmin;
    b->d_min = d_min;
    const int st = upload_blocks(b, s);
    b->queries_set = st == RMQ_OK;
    return st;
}

int rmq_batch_build(rmq_batch* b, rmq_stream_t stream) {
    rmq::NvtxRange nvtx_range("rmq_batch_build");
    if (b == nullptr) return RMQ_ERR_ARG;
    DeviceGuard guard(b->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaEventRecord(b->ev0, s);
    if (e == cudaSuccess) e = enqueue_build(b, s);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev1, s);
    b->build_timed = e == cudaSuccess;
    return status_of(e);
}

int rmq_batch_query(rmq_batch* b, rmq_stream_t stream) {
    rmq::NvtxRange nvtx_range("rmq_batch_query");
    if (b == nullptr || !b->queries_set) return RMQ_ERR_ARG;
    DeviceGuard guard(b->device);
    return status_of(enqueue_query(b, reinterpret_cast<cudaStream_t>(stream)));
}

int rmq_batch_run(rmq_batch* b, rmq_stream_t stream) {
    rmq::NvtxRange nvtx_range("rmq_batch_run");
    if (b == nullptr || !b->queries_set) return RMQ_ERR_ARG;
    DeviceGuard guard(b->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (b->graph == nullptr) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return status_of(e);
        cudaError_t e1 = enqueue_build(b, b->cap_stream);
        cudaError_t e2 = e1 == cudaSuccess ? enqueue_query(b, b->cap_stream) : e1;
        e = cudaStreamEndCapture(b->cap_stream, &g);
        if (e2 != cudaSuccess || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return status_of(e2 != cudaSuccess ? e2 : e);
        }
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return status_of(e);
        }
    }
    return status_of(cudaGraphLaunch(b->graph, s));
}

int rmq_batch_run_per_array(rmq_batch* b, rmq_stream_t stream) {
    rmq::NvtxRange nvtx_range("rmq_batch_run_per_array");
    if (b == nullptr || !b->queries_set) return RMQ_ERR_ARG;
    DeviceGuard guard(b->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    for (uint32_t a = 0; a < b->num_arrays; ++a) {
        const ArrayDesc& d = b->h_descs[a];
        const rmq::Layout lay = rmq::plan_layout(b->sizes[a], b->tc[size_class(b->sizes[a])], 3);
        const float* vals = b->d_values + d.val_off;
        float* lvl = b->lvl_val + d.lvl_base;
        uint32_t* idx = b->lvl_idx != nullptr ? b->lvl_idx + d.idx_base : nullptr;
        cudaError_t e = rmq::launch_build(lay, vals, lvl, idx, s);
        if (e != cudaSuccess) return status_of(e);
        const uint64_t q0 = b->q_off[a], q = b->q_off[a + 1] - q0;
        if (q == 0) continue;
        rmq::QueryArgs qa;
        std::memset(&qa, 0, sizeof(qa));
        for (uint32_t k = 0; k < lay.num_levels; ++k) {
            qa.lv.val[k] = k == 0 ? vals : lvl + lay.offset[k];
            qa.lv.idx[k] = (k == 0 || idx == nullptr) ? nullptr : idx + lay.offset[k];
            qa.lv.size[k] = uint32_t(lay.size[k]);
        }
        qa.lv.num_levels = lay.num_levels;
        qa.qs = reinterpret_cast<const uint2*>(b->d_lr) + q0;
        qa.q = q;
        qa.out_min = b->d_min != nullptr ? b->d_min + q0 : nullptr;
        qa.out_idx = b->d_argmin != nullptr ? b->d_argmin + q0 : nullptr;
        qa.variant = RMQ_VARIANT_VL;
        qa.lanes = 8;
        qa.rf_log = 3;
        e = rmq::launch_query(qa, s);
        if (e != cudaSuccess) return status_of(e);
    }
    return RMQ_OK;
}

// Device time of one query pass with the current plan and CTA size (one
// warm-up launch, then the mean of `reps` timed launches).
int time_query(rmq_batch* b, cudaStream_t s, int reps, float* ms_out) {
    cudaError_t e = enqueue_query(b, s);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(b->ev0, s);
    for (int rep = 0; rep < reps && e == cudaSuccess; ++rep) e = enqueue_query(b, s);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->ev1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (e != cudaSuccess) return status_of(e);
    *ms_out = ms / float(reps);
    return RMQ_OK;
}

int rmq_batch_autotune(rmq_batch* b, rmq_stream_t stream, rmq_batch_info* info) {
    rmq::NvtxRange nvtx_range("rmq_batch_autotune");
    if (b == nullptr || !b->queries_set) return RMQ_ERR_ARG;
    DeviceGuard guard(b->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // 1. one threshold for every array x CTA size
    float best = -1.f;
    uint64_t best_t = b->t;
    uint32_t best_block = b->qblock;
    for (uint64_t t : kTuneT) {
        int st = plan(b, t, s);
        if (st != RMQ_OK) return st;
        cudaError_t e = enqueue_build(b, s);
        if (e != cudaSuccess) return status_of(e);
        for (uint32_t qb : kTuneBlock) {
            b->qblock = qb;
            st = upload_blocks(b, s);
            if (st != RMQ_OK) return st;
            float ms = 0.f;
            st = time_query(b, s, 2, &ms);
            if (st != RMQ_OK) return st;
            if (best < 0.f || ms < best) {
                best = ms;
                best_t = t;
                best_block = qb;
            }
        }
    }
    // 2. each size class's threshold in turn (largest arrays first, they
    // carry most of the queries), the others held; a change is kept only
    // when it is faster by more than 0.5 %, above the timing noise.
    b->qblock = best_block;
    int st = upload_blocks(b, s);
    if (st != RMQ_OK) return st;
    uint64_t best_tc[kClasses] = {best_t, best_t, best_t};
    for (int c = kClasses - 1; c >= 0; --c) {
        for (uint64_t t : kTuneT) {
            if (t == best_tc[c]) continue;
            uint64_t tc[kClasses] = {best_tc[0], best_tc[1], best_tc[2]};
            tc[c] = t;
            st = plan(b, tc, s);
            if (st != RMQ_OK) return st;
            cudaError_t e = enqueue_build(b, s);
            if (e != cudaSuccess) return status_of(e);
            float ms = 0.f;
            st = time_query(b, s, 2, &ms);
            if (st != RMQ_OK) return st;
            if (ms < best * 0.995f) {
                best = ms;
                best_tc[c] = t;
            }
        }
    }
    st = plan(b, best_tc, s);
    if (st != RMQ_OK) return st;
    cudaError_t e = enqueue_build(b, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return status_of(e);
    b->build_timed = false;
    b->query_ms = best;
    return info != nullptr ? rmq_batch_get_info(b, info) : RMQ_OK;
}

int rmq_batch_set_tuning(rmq_batch* b, uint64_t scan_threshold, uint32_t query_block, rmq_stream_t stream) {
    if (b == nullptr || scan_threshold < 8 || query_block < 32 || query_block > rmq::kMaxQueryThreads ||
        query_block % 32 != 0)
        return RMQ_ERR_ARG;
    DeviceGuard guard(b->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int st = plan(b, scan_threshold, s);  // RMQ_ERR_UNSUPPORTED when the levels would not fit
    if (st != RMQ_OK) return st;
    b->qblock = query_block;
    if (b->queries_set) {
        st = upload_blocks(b, s);
        if (st != RMQ_OK) return st;
    }
    drop_graph(b);
    b->build_timed = false;
    return RMQ_OK;
}

int rmq_batch_set_class_tuning(rmq_batch* b, const uint64_t* class_thresholds, uint32_t query_block,
                               rmq_stream_t stream) {
    if (b == nullptr || class_thresholds == nullptr || query_block < 32 || query_block > rmq::kMaxQueryThreads ||
        query_block % 32 != 0)
        return RMQ_ERR_ARG;
    uint64_t tc[kClasses];
    for (int c = 0; c < kClasses; ++c) {
        if (class_thresholds[c] < 8) return RMQ_ERR_ARG;
        tc[c] = class_thresholds[c];
    }
    DeviceGuard guard(b->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int st = plan(b, tc, s);  // RMQ_ERR_UNSUPPORTED when the levels would not fit
    if (st != RMQ_OK) return st;
    b->qblock = query_block;
    if (b->queries_set) {
        st = upload_blocks(b, s);
        if (st != RMQ_OK) return st;
    }
    drop_graph(b);
    b->build_timed = false;
    return RMQ_OK;
}

int rmq_batch_get_info(const rmq_batch* bc, rmq_batch_info* info) {
    if (bc == nullptr || info == nullptr) return RMQ_ERR_ARG;
    rmq_batch* b = const_cast<rmq_batch*>(bc);
    std::memset(info, 0, sizeof(*info));
    info->num_arrays = b->num_arrays;
    for (uint64_t n : b->sizes) info->total_values += n;
    info->level_bytes = b->lvl_used * (sizeof(float) + (b->lvl_idx ? sizeof(uint32_t) : 0));
    info->scan_threshold = b->t;
    info->query_block = b->qblock;
    info->max_levels = b->max_levels;
    info->total_queries = b->queries_set ? b->q_off[b->num_arrays] : 0;
    if (b->build_timed) {
        DeviceGuard guard(b->device);
        if (cudaEventSynchronize(b->ev1) == cudaSuccess) cudaEventElapsedTime(&b->build_ms, b->ev0, b->ev1);
        cudaGetLastError();
    }
    info->build_ms = b->build_ms;
    info->query_ms = b->query_ms;
    for (int c = 0; c < kClasses; ++c) {
        info->class_threshold[c] = b->tc[c];
        info->class_upper[c] = kClassUpper[c];
    }
    return RMQ_OK;
}

void rmq_batch_destroy(rmq_batch* b) {
    if (b == nullptr) return;
    {
        DeviceGuard guard(b->device);
        drop_graph(b);
        if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
        if (b->ev0) cudaEventDestroy(b->ev0);
        if (b->ev1) cudaEventDestroy(b->ev1);
        cudaFree(b->lvl_val);
        cudaFree(b->lvl_idx);
        cudaFree(b->d_descs);
        cudaFree(b->d_tile_off);
        cudaFree(b->d_q_off);
        cudaFree(b->d_blk_off);
        cudaFree(b->d_owner);
        cudaGetLastError();
    }
    delete b;
}

}  // extern "C"
