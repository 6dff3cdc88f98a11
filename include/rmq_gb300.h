/*
 * rmq_gb300.h — C ABI of the GB300-native hierarchical range-minimum library.
 *
 * A handle holds a multi-level block-minimum structure over a caller-owned
 * fp32 array that stays resident in device memory.  Queries are inclusive
 * index pairs {l, r} (uint2 layout: 8 bytes per query, l first) and are
 * answered on the device, stream-ordered, into caller-provided device buffers.
 *
 * Semantics (identical to the reference's brute-force scan):
 *   min(l, r)    = A[argmin(l, r)]  (the bits of that element are returned)
 *   argmin(l, r) = lowest i in [l, r] such that no j in [l, r] has A[j] < A[i]
 *                  (IEEE-754 "<", so ties, including -0.0 vs +0.0, go to the
 *                  lowest index).
 * Inputs holding NaN are outside the contract.  A query with l > r or r >= n
 * is invalid: its min is written as NaN and its argmin as all ones
 * (0xFFFFFFFF, or 2^64 - 1 for 64-bit queries), and with cfg.validate set the
 * call reports RMQ_ERR_QUERY_RANGE.
 *
 * No entry point exits the process or traps the GPU; all return a status.
 * rmq_query / rmq_query_idx do not allocate, do not synchronise (unless
 * cfg.validate is set) and may be issued concurrently on different streams:
 * a handle is immutable after rmq_build returns.
 */
#ifndef RMQ_GB300_H
#define RMQ_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CUDA stream handle without pulling in the CUDA headers (same type as cudaStream_t). */
typedef struct CUstream_st* rmq_stream_t;

typedef struct rmq_handle rmq_handle;

typedef enum {
    RMQ_OK = 0,
    RMQ_ERR_ARG = 1,          /* bad argument (null pointer, bad alignment, bad config) */
    RMQ_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    RMQ_ERR_OOM = 3,          /* device allocation failed */
    RMQ_ERR_QUERY_RANGE = 4,  /* at least one query had l > r or r >= n (validate mode) */
    RMQ_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    RMQ_ERR_NO_INDEX = 6,     /* argmin asked of a handle built with with_index = 0 */
    RMQ_ERR_UNSUPPORTED = 7   /* size or configuration outside what this library supports */
} rmq_status;

typedef enum {
    RMQ_VARIANT_AUTO = 0,  /* the measured best: VL with rf = 8                                          */
    RMQ_VARIANT_CL = 1,    /* tile of lanes answering its queries one after another (reference alg 16 family) */
    RMQ_VARIANT_VL = 2,    /* one thread per query, 256-bit loads (reference alg 20 family)              */
    /* The reference's ablations of its CL kernel: the same hierarchy and
     * results, other work distributions (src/xxx.h:302-790). */
    RMQ_VARIANT_CL_NO_SHUFFLE = 3,     /* each lane loads the turn's query itself (alg 23)              */
    RMQ_VARIANT_CL_QUERY_PER_TILE = 4, /* one query per tile of lanes, no turns (alg 24)               */
    RMQ_VARIANT_CL_ATOMIC = 5,         /* lanes combine with atomic minima, no shuffle reduction (alg 19);
                                          scan threshold below 2^27                                      */
    /* VL for workloads of short queries (rf 8, 32-bit positions; otherwise
     * VL): a query of at most 512 entries takes its level-0 winner while it
     * folds level 0 instead of reading that sector again to locate it, which
     * its evict-first L2 line seldom survives.  Same results. */
    RMQ_VARIANT_VL_SHORT = 6
} rmq_variant;

typedef struct {
    int32_t  variant;         /* rmq_variant                                                    */
    uint64_t scan_threshold;  /* t: build levels while a level holds more than t entries (0 = variant default) */
    int32_t  rf_log;          /* log2 of the per-level reduction factor, 3..5 (0 = variant default)       */
    int32_t  lanes;           /* CL: lanes cooperating on one query, 2/4/8/16/32 (0 = default)          */
    int32_t  with_index;      /* build the per-block argmin arrays (needed by rmq_query_idx)             */
    int32_t  l2_persist;      /* put the coarse levels in an L2 persisting access-policy window          */
    int32_t  validate;        /* count invalid queries on the device; query calls then synchronise       */
    int32_t  index_bits;      /* 32 or 64 (0 = 32, or 64 when n > 0xFFFFFF00); 64 = rmq_query*64 only, VL   */
} rmq_config;

typedef struct {
    uint32_t num_levels;        /* including level 0 (the caller's array)               */
    uint32_t rf_log;            /* reduction factor of every level step                 */
    int32_t  variant;           /* resolved variant (never AUTO)                         */
    int32_t  lanes;             /* resolved lanes per query (CL)                         */
    uint64_t n;                 /* number of values                                      */
    uint64_t scan_threshold;    /* resolved t                                            */
    uint64_t level_size[20];    /* entries per level                                     */
    uint64_t level_offset[20];  /* element offset of level k >= 1 in the level buffer    */
    uint64_t level_bytes;       /* device bytes of level values (+ argmin arrays)        */
    float    build_ms;          /* device time of the last build (CUDA events)           */
    int32_t  index_bits;        /* 32 or 64                                              */
} rmq_info;

/* Fills *cfg with the defaults: AUTO variant, default t and rf, with_index = 1,
 * l2_persist = 0, validate = 0. */
void rmq_config_init(rmq_config* cfg);

/* Builds the hierarchy over d_values[0..n) on `stream`.  d_values must be
 * 32-byte aligned and must outlive the handle (level 0 is the caller's array).
 * Replaces the build half of xxx_rmq (src/xxx.h:225-268) and of
 * hierarchical_vector_load (src/xxx.h:958-1010).  Returns after the build is
 * enqueued and its device time recorded (the call waits for the build). */
int rmq_build(const float* d_values, uint64_t n, const rmq_config* cfg,
              rmq_stream_t stream, rmq_handle** out);

/* Range minima of q inclusive queries d_lr[2i] = l, d_lr[2i+1] = r into d_min[q].
 * Replaces the query half of xxx_rmq (src/xxx.h:273-294, kernel src/xxx.h:124-200)
 * and of hierarchical_vector_load (src/xxx.h:1012-1036, kernel src/xxx.h:883-930);
 * the results are those of gpu_rmq_basic (src/cuda_methods.cuh:72). */
int rmq_query(const rmq_handle* h, const uint32_t* d_lr, uint64_t q, float* d_min,
              rmq_stream_t stream);

/* Range argmin (lowest index on ties) into d_argmin[q]; also the minima into
 * d_min_or_null when it is not NULL.  The reference has no hierarchical argmin;
 * the results are those of gpu_rmq_basic_idx (src/cuda_methods.cuh:106) and
 * cpu_rmq_idx (src/cpu_methods.h:56). */
int rmq_query_idx(const rmq_handle* h, const uint32_t* d_lr, uint64_t q,
                  uint32_t* d_argmin, float* d_min_or_null, rmq_stream_t stream);
/* For every query call: d_lr is aligned to its pair (8 bytes; 16 for the
 * 64-bit forms) and each result pointer to its element (4 bytes; 8 for
 * 64-bit argmin); anything else returns RMQ_ERR_ARG before any launch. */

/* 64-bit counterparts for handles built with index_bits = 64 (the
 * reference's IS_LONG build: uint64_t indices and ulong2 queries,
 * src/main.cu:21-27, for arrays beyond 2^32 entries): d_lr holds q inclusive
 * pairs of uint64 {l, r}; argmin results are uint64.  Same semantics; the VL
 * work distribution.  A 32-bit handle returns RMQ_ERR_UNSUPPORTED here, and a
 * 64-bit handle does so from rmq_query / rmq_query_idx. */
int rmq_query64(const rmq_handle* h, const uint64_t* d_lr, uint64_t q, float* d_min,
                rmq_stream_t stream);
int rmq_query_idx64(const rmq_handle* h, const uint64_t* d_lr, uint64_t q, uint64_t* d_argmin,
                    float* d_min_or_null, rmq_stream_t stream);

/* The same queries with HOST buffers, the form of the reference's host
 * drivers (xxx_rmq / hierarchical_vector_load return a host array,
 * src/xxx.h:203-298, :932-1040).  h_lr holds the q inclusive pairs in host
 * memory; results are written to host memory.  Blocking: returns when every
 * result is in place; calls on one handle are serialised (on streams the
 * handle owns, created on the first call and kept until rmq_destroy).
 * When every buffer is page-locked (cudaHostAlloc / cudaHostRegister) over
 * its whole length and naturally aligned, one kernel launch reads the
 * queries from and writes the results to host memory directly.  Otherwise chunks of 2^22 queries go
 * through device staging buffers (three chunks, allocated on first use and
 * kept), the upload of one chunk and the download of the previous one
 * overlapping the kernel of the current one. */
int rmq_query_host(const rmq_handle* h, const uint32_t* h_lr, uint64_t q, float* h_min);
int rmq_query_idx_host(const rmq_handle* h, const uint32_t* h_lr, uint64_t q, uint32_t* h_argmin,
                       float* h_min_or_null);
int rmq_query64_host(const rmq_handle* h, const uint64_t* h_lr, uint64_t q, float* h_min);
int rmq_query_idx64_host(const rmq_handle* h, const uint64_t* h_lr, uint64_t q, uint64_t* h_argmin,
                         float* h_min_or_null);

/* Brute-force scan, one thread per query (the reference's GPU checker,
 * kernel_rmq_basic / kernel_rmq_basic_idx, src/cuda_methods.cuh:4-44).
 * Either output may be NULL.  Used by the driver's --check and as alg 2/102. */
int rmq_scan_bruteforce(const float* d_values, uint64_t n, const uint32_t* d_lr,
                        uint64_t q, float* d_min_or_null, uint32_t* d_argmin_or_null,
                        rmq_stream_t stream);

/* Layout and build statistics of a handle. */
int rmq_get_info(const rmq_handle* h, rmq_info* info);

/* Frees the level buffers.  Safe on NULL.  Waits for work using the handle
 * on the build stream. */
void rmq_destroy(rmq_handle* h);

/* Static, human-readable name of a status code. */
const char* rmq_strerror(int status);

/* Range argmin (and, when d_min_or_null is not NULL, minima) of q inclusive
 * queries over d_values[0..n), without any device allocation.  For callers
 * that cannot allocate device memory when they query: hosts that reserve the
 * whole device for their own memory pool, and latency-bound callers for whom
 * cudaMalloc / cudaFree are off limits because those calls can block and
 * synchronise the device.  It has no counterpart in the reference.
 *
 * The hierarchy (VL, rf = 8, scan threshold t; 0 = 32) is built into one
 * fixed 8 MiB device array owned by the library, which every GPU that loads
 * the library holds until the process exits; then the queries are answered,
 * both on `stream`.  Limit: n <= 2^22 (4,194,304 entries); a larger n, or a t
 * whose levels do not fit, returns RMQ_ERR_UNSUPPORTED before any device
 * work.  The first call on each device (each device context: after a
 * cudaDeviceReset the next call counts as a first call again) looks up the
 * array's device address (cudaGetSymbolAddress).  CUDA loads device code
 * lazily by default, so that first call is also what places the array and
 * the kernels of this entry point on the device and may need device memory
 * for them: make it before reserving the whole device for a pool, and
 * before any stream capture (a call with q = 0 places the array and the
 * build kernel; one with q > 0 also the query kernel).
 * All calls on a device share the array, which keeps the last call's
 * contents (each call rewrites every entry it reads, so nothing needs
 * clearing): calls whose device work overlaps, on different streams or from
 * different host threads, race on it.  Inputs and results are as for
 * rmq_query_idx; d_values must be 32-byte aligned. */
int rmq_query_idx_static(const float* d_values, uint64_t n, uint64_t scan_threshold,
                         const uint32_t* d_lr, uint64_t q, uint32_t* d_argmin,
                         float* d_min_or_null, rmq_stream_t stream);

/* Bounds-checked builds only (librmq_gb300_checked.so, compiled with
 * RMQ_DEBUG_BOUNDS=1): *count = level loads of the query kernels that fell
 * outside their level since the last call on this device (each such load is
 * skipped, not made), then the count is cleared.  The regular library
 * returns RMQ_ERR_UNSUPPORTED. */
int rmq_debug_bounds_violations(uint64_t* count);

/* Measurement aid, no counterpart in the reference: the rate at which this
 * GPU's SMs read L2-resident 32-byte sectors with the query kernels' load
 * form, the bound of the coarse levels' reads.  Reads d_buf[0 .. bytes)
 * (bytes / 32 a power of two, at least 1024; the buffer should fit in L2 and
 * hold values >= -1) once to bring it into L2, then `passes` more times,
 * in address order (random = 0) or at hashed sector positions (random = 1),
 * on `stream`; *ms_out = device time of those passes (CUDA events).  Blocks
 * until done. */
int rmq_measure_l2_read(const float* d_buf, uint64_t bytes, uint32_t passes, int32_t random,
                        rmq_stream_t stream, float* ms_out);

/* Level layout only (host computation, no device work): the reference's rule
 * (src/xxx.h:225-243) generalised to rf = 2^rf_log.  Returns RMQ_ERR_ARG when
 * t is below the variant's minimum.  Usable without a GPU. */
int rmq_plan_layout(uint64_t n, uint64_t scan_threshold, int32_t rf_log,
                    int32_t variant, rmq_info* info);

#ifdef __cplusplus
}
#endif

#endif /* RMQ_GB300_H */
