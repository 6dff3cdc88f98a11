// rmq_noalloc.cu — the allocation-free entry point rmq_query_idx_static.
//
// Some callers cannot allocate device memory at the moment they need a range
// minimum: hosts that reserve the whole device up front for their own memory
// pool (a further cudaMalloc fails or fragments that pool), and latency-bound
// callers for whom cudaMalloc / cudaFree are off limits because those calls
// can block and synchronise the device.  For them this file keeps the
// hierarchy's coarse levels in one file-scope device array of fixed size.
// The caller still provides the values, the queries and the output buffers.
//
// When the array exists on a device: CUDA loads device code lazily by default
// (CUDA_MODULE_LOADING=LAZY), so the array, and the build and query kernels
// this entry point launches, are placed on a device by the first call made
// on it, not when the library is loaded.  That first call can therefore need
// device memory for the array and the kernels' code; a caller that is about
// to reserve the whole device should make one call (q = 0 is enough for the
// array and the build kernel; q > 0 also loads the query kernel) before
// reserving it, and before any stream capture.  From then on the device holds
// the array until its context is destroyed (process exit or cudaDeviceReset).
#include <cstring>
#include <mutex>

#include <cuda.h>  // CUcontext / CUresult types only; the driver calls are looked up at run time

#include "../../include/rmq_gb300.h"
#include "rmq_internal.h"

namespace {

// 8 MiB: coarse levels (fp32 value + uint32 index per entry) of arrays of up
// to 2^22 entries at rf = 8 take about 4.8 MiB.
constexpr size_t kScratchBytes = size_t(8) << 20;
constexpr uint64_t kStaticMaxN = uint64_t(1) << 22;
constexpr uint32_t kStaticRfLog = 3;
constexpr uint64_t kStaticDefaultT = 32;
constexpr int kMaxDevices = 64;

// Shared by every call on a device; it keeps the last call's contents.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host code cannot use g_scratch's name as a device address (on the host it
// names a stand-in object); its device address is looked up at set-up, once
// per device context, with that context current.  A context is told apart by
// its id (cuCtxGetId), so a device reset, which destroys the context and
// reloads the array elsewhere in a new one, is followed by a fresh lookup
// rather than a stale address.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct ScratchAddr {
    unsigned long long ctx_id = 0;
    bool set = false;
    void* ptr = nullptr;
};

std::mutex g_setup_mu;
ScratchAddr g_scratch_addr[kMaxDevices];
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

bool current_context_id(unsigned long long* id) {
    if (g_ctx_get_current == nullptr || g_ctx_get_id == nullptr) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || f1 == nullptr ||
            f2 == nullptr) {
            cudaGetLastError();
            return false;
        }
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

int scratch_for_current_device(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return RMQ_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return RMQ_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    ScratchAddr& slot = g_scratch_addr[dev];
    unsigned long long id = 0;
    // Before the runtime has made a context current on this thread there is
    // no id to compare: the lookup below makes it current.
    const bool have_id = current_context_id(&id);
    if (!slot.set || !have_id || slot.ctx_id != id) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return RMQ_ERR_CUDA;
        }
        if (!current_context_id(&id)) return RMQ_ERR_CUDA;
        slot.ctx_id = id;
        slot.ptr = p;
        slot.set = true;
    }
    *out = slot.ptr;
    return RMQ_OK;
}

}  // namespace

extern "C" int rmq_query_idx_static(const float* d_values, uint64_t n, uint64_t scan_threshold,
                                    const uint32_t* d_lr, uint64_t q, uint32_t* d_argmin,
                                    float* d_min_or_null, rmq_stream_t stream) {
    if (d_values == nullptr || n == 0 || d_argmin == nullptr) return RMQ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d_values) & 31u) != 0) return RMQ_ERR_ARG;
    if (q > 0 && (d_lr == nullptr || (reinterpret_cast<uintptr_t>(d_lr) & 7u) != 0)) return RMQ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d_argmin) & 3u) != 0 || (reinterpret_cast<uintptr_t>(d_min_or_null) & 3u) != 0)
        return RMQ_ERR_ARG;
    if (n > kStaticMaxN || q > 0xFFFFFFFFull) return RMQ_ERR_UNSUPPORTED;  // above the fixed scratch
    const uint64_t t = scan_threshold != 0 ? scan_threshold : kStaticDefaultT;
    if (t < (uint64_t(1) << kStaticRfLog)) return RMQ_ERR_ARG;  // VL precondition, src/xxx.h:938
    const rmq::Layout lay = rmq::plan_layout(n, t, kStaticRfLog);
    if (lay.total * (sizeof(float) + sizeof(uint32_t)) > kScratchBytes) return RMQ_ERR_UNSUPPORTED;

    void* scratch = nullptr;
    const int st = scratch_for_current_device(&scratch);
    if (st != RMQ_OK) return st;
    float* val_buf = static_cast<float*>(scratch);
    uint32_t* idx_buf = reinterpret_cast<uint32_t*>(val_buf + lay.total);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

    // Every level entry a query reads is rewritten by the build of this call, so nothing
    // in the scratch needs clearing between calls.
    cudaError_t e = rmq::launch_build(lay, d_values, val_buf, idx_buf, s);
    if (e == cudaSuccess && q > 0) {
        rmq::QueryArgs a;
        std::memset(&a, 0, sizeof(a));
        for (uint32_t k = 0; k < lay.num_levels; ++k) {
            a.lv.val[k] = k == 0 ? d_values : val_buf + lay.offset[k];
            a.lv.idx[k] = k == 0 ? nullptr : idx_buf + lay.offset[k];
            a.lv.size[k] = uint32_t(lay.size[k]);
        }
        a.lv.num_levels = lay.num_levels;
        a.qs = reinterpret_cast<const uint2*>(d_lr);
        a.q = q;
        a.out_min = d_min_or_null;
        a.out_idx = d_argmin;
        a.variant = RMQ_VARIANT_VL;
        a.lanes = 8;
        a.rf_log = lay.rf_log;
        e = rmq::launch_query(a, s);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return RMQ_ERR_CUDA;
    }
    return RMQ_OK;
}
