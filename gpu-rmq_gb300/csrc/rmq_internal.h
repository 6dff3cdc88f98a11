// rmq_internal.h — launchers shared between the kernel translation units and
// the C ABI implementation.  Host-only declarations (no device code).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "rmq_common.cuh"

namespace rmq {

// Names this library's calls on a profiler's timeline (an NVTX range for
// the scope; without an attached tool it costs one pointer check).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Host level-layout rule (reference src/xxx.h:225-243, generalised to rf = 2^rf_log).
Layout plan_layout(uint64_t n, uint64_t t, uint32_t rf_log);

// Build level k+1 from level k for every k in [0, num_levels-1).
// `val_buf`/`idx_buf` are the level buffers (layout.total entries each);
// `idx_buf` may be null (no argmin support).  With `counters` (at least
// tail_counters(lay) zeroed entries, left zeroed by every build, never used
// by two builds at once) the levels above the fused tiles are built inside
// the fused kernel (one launch in all); without, by extra launches.
cudaError_t launch_build(const Layout& lay, const float* d_values, float* val_buf,
                         uint32_t* idx_buf, cudaStream_t s, unsigned* counters = nullptr);
// Same with 64-bit positions (arrays beyond 2^32 entries).
cudaError_t launch_build64(const Layout& lay, const float* d_values, float* val_buf,
                           uint64_t* idx_buf, cudaStream_t s, unsigned* counters = nullptr);
// Arrival counters the single-launch build needs for `lay` (0: none).
uint64_t tail_counters(const Layout& lay);

struct QueryArgs {
    Levels lv;
    const uint2* qs;
    uint64_t q;
    float* out_min;      // may be null for argmin queries
    uint32_t* out_idx;   // null for min queries
    bool wide;           // 64-bit positions: lv64 / qs64 / out_idx64 are used instead
    Levels64 lv64;
    const uint64_t* qs64;
    uint64_t* out_idx64;
    uint32_t* err;       // invalid-query counter or null
    int variant;         // rmq_variant: 1 = CL, 2 = VL, 3 / 4 / 5 = CL without shuffles / a tile per query / atomic combine
    int lanes;           // CL tile width
    uint32_t rf_log;
    const void* persist_base;   // L2 access-policy window (null = none)
    size_t persist_bytes;
    float persist_hit_ratio;
};

cudaError_t launch_query(const QueryArgs& a, cudaStream_t s);

cudaError_t launch_bruteforce(const float* vals, uint32_t n, const uint2* qs, uint32_t q,
                              float* out_min, uint32_t* out_idx, cudaStream_t s);

// Query launch over packed work: entry e (an array, or a request's array in
// serving mode) owns queries [q_off[e], q_off[e+1]) of qs, in units of 32
// queries per warp; owner[u] gives the entry of unit u (launch_fill_owner).
struct BatchQueryArgs {
    const float* values;
    const ArrayDesc* descs;
    const uint32_t* owner;
    const uint64_t* unit_off;
    const uint64_t* q_off;
    uint64_t total_units;
    const float* lvl_val;
    const uint32_t* lvl_idx;
    const uint2* qs;
    float* out_min;
    uint32_t* out_idx;  // null: minima only
    uint32_t threads;   // CTA size, multiple of 32, <= 512
};

cudaError_t launch_batch_query(const BatchQueryArgs& a, cudaStream_t s);

// Where one served request's queries come from and its results go: device
// staging buffers, or the request's own page-locked host buffers, which the
// kernel reads and writes directly over the CPU-GPU link.  Either result
// pointer may be null.
struct ServeIO {
    const uint2* qs;
    uint32_t* out_idx;
    float* out_min;
};

// The served batch: entry e (a request) answers its q_off[e+1] - q_off[e]
// queries through io[e] and counts its invalid queries in bad[e] (zeroed by
// the caller); units of 32 queries as for launch_batch_query.
struct ServeQueryArgs {
    const float* values;
    const ArrayDesc* descs;
    const uint32_t* owner;
    const uint64_t* unit_off;
    const uint64_t* q_off;
    uint64_t total_units;
    const float* lvl_val;
    const uint32_t* lvl_idx;
    const ServeIO* io;
    uint32_t* bad;
    uint32_t threads;  // CTA size, multiple of 32, <= 512
};

cudaError_t launch_serve_query(const ServeQueryArgs& a, cudaStream_t s);
cudaError_t launch_fill_owner(const uint64_t* unit_off, uint32_t num, uint32_t* owner, cudaStream_t s);

#if RMQ_DEBUG_BOUNDS
// Violations counted by the checked kernels of the query / batched units
// since the last read (each read clears them).
unsigned int bounds_bad_query();
unsigned int bounds_bad_batch();
#endif

// Number of kernel launches the last launch_build issued (for accounting).
int build_launch_count(const Layout& lay);

}  // namespace rmq
