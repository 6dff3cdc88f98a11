/*
 * rmq_gb300_batch.h — batched range-minimum queries over many independent
 * arrays, and seeded device-side input generators.
 *
 * The reference answers one array per run of its driver (src/main.cu:71-287),
 * so a workload of thousands of arrays is a loop of builds and query launches
 * (src/xxx.h:258-281 per array).  A batch packs the arrays' coarse levels in
 * one allocation, builds all of them with two kernels, answers all their
 * query sets with one kernel, and can replay build + queries as one CUDA
 * graph launch.  Semantics per query are exactly those of rmq_query_idx
 * (include/rmq_gb300.h).  The work distribution is VL with rf = 8.
 */
#ifndef RMQ_GB300_BATCH_H
#define RMQ_GB300_BATCH_H

#include <stdint.h>

#include "rmq_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rmq_batch rmq_batch;

typedef struct {
    uint32_t num_arrays;
    uint64_t total_values;      /* sum of the array sizes                                   */
    uint64_t level_bytes;       /* device bytes of all coarse levels (values + argmin)      */
    uint64_t scan_threshold;    /* t used for every array (after autotuning, if run)         */
    uint32_t query_block;       /* threads per CTA of the query kernel (one warp = 32 queries) */
    uint32_t max_levels;        /* deepest hierarchy in the batch                            */
    uint64_t total_queries;     /* of the last rmq_batch_set_queries                         */
    float    build_ms;          /* device time of the last rmq_batch_build (CUDA events)    */
    float    query_ms;          /* device time of the last timed query pass (autotune)      */
    uint64_t class_threshold[3];  /* t of each array-size class (scan_threshold = the last)  */
    uint64_t class_upper[3];      /* class c holds the arrays with class_upper[c-1] <= n < class_upper[c] */
} rmq_batch_info;

/* Creates a batch over num_arrays arrays packed in d_values: array a is
 * d_values[value_offsets[a] .. value_offsets[a] + sizes[a]) (host arrays of
 * num_arrays entries; offsets multiples of 8 so every array is 32-byte
 * aligned; 1 <= sizes[a] <= 0xFFFFFF00).  cfg: scan_threshold (0 = 64) and
 * with_index are used; rf is 8.  Allocates the packed level buffers and the
 * device descriptors; nothing is built yet.  d_values must outlive the batch. */
int rmq_batch_create(const float* d_values, const uint64_t* value_offsets, const uint64_t* sizes,
                     uint32_t num_arrays, const rmq_config* cfg, rmq_stream_t stream,
                     rmq_batch** out);

/* Registers the query sets: array a's queries are the inclusive pairs
 * d_lr[2i], d_lr[2i+1] for query_offsets[a] <= i < query_offsets[a+1]
 * (host array of num_arrays + 1 non-decreasing offsets; indices local to
 * array a).  Results go to the same positions of d_argmin (may be NULL for
 * minima only) and d_min (may be NULL when d_argmin is given).  Uploads the
 * work list (synchronises `stream`); invalidates a captured graph. */
int rmq_batch_set_queries(rmq_batch* b, const uint32_t* d_lr, const uint64_t* query_offsets,
                          uint32_t* d_argmin, float* d_min, rmq_stream_t stream);

/* Enqueues the build of every array's coarse levels (two kernel launches). */
int rmq_batch_build(rmq_batch* b, rmq_stream_t stream);

/* Enqueues one query launch over every registered query of every array. */
int rmq_batch_query(rmq_batch* b, rmq_stream_t stream);

/* Build + queries as one CUDA graph launch (captured on the first call after
 * rmq_batch_set_queries / rmq_batch_autotune, replayed afterwards). */
int rmq_batch_run(rmq_batch* b, rmq_stream_t stream);

/* The comparator of the batched form: the same work as a per-array loop of
 * the plain single-array kernels, the way a caller without this header would
 * run it with buffers allocated up front.  For each array in turn, the
 * single-array build (the kernels of rmq_build) into the batch's own level
 * buffers, then the single-array query kernel of rmq_query_idx over its
 * queries; all on `stream`, nothing synchronised between arrays.  Results
 * are identical to rmq_batch_run's. */
int rmq_batch_run_per_array(rmq_batch* b, rmq_stream_t stream);

/* Autotuner: times the query kernel on the registered queries for each
 * candidate scan threshold t in {16, 32, 64, 256, 1024} (the same for every
 * array) and CTA size in {64, 128, 256, 512} threads; then, keeping the best
 * CTA size, tries each t for each array-size class in turn (arrays below 2^14
 * entries, below 2^18, and the rest; the largest class first) and keeps a
 * class's new t when it is faster by more than 0.5 %.  Rebuilds with the
 * choice.  Blocking.  The choice is reported in *info (may be NULL). */
int rmq_batch_autotune(rmq_batch* b, rmq_stream_t stream, rmq_batch_info* info);

/* Applies a known choice (for example one rmq_batch_autotune made earlier for
 * the same workload): scan threshold t (>= 8) and CTA size (a multiple of 32,
 * <= 512) of the query kernel.  The levels must be rebuilt (rmq_batch_build or
 * rmq_batch_run) before querying.  RMQ_ERR_UNSUPPORTED when t would need more
 * level storage than the batch holds (any t >= 16, or the creation t, fits). */
int rmq_batch_set_tuning(rmq_batch* b, uint64_t scan_threshold, uint32_t query_block, rmq_stream_t stream);

/* The same with one t per array-size class (class_thresholds[3], each >= 8,
 * in the order of rmq_batch_info.class_upper), as rmq_batch_autotune
 * reports it. */
int rmq_batch_set_class_tuning(rmq_batch* b, const uint64_t* class_thresholds, uint32_t query_block,
                               rmq_stream_t stream);

int rmq_batch_get_info(const rmq_batch* b, rmq_batch_info* info);

/* Frees the batch's device memory and graph.  Safe on NULL. */
void rmq_batch_destroy(rmq_batch* b);

/* ---- seeded device-side generators (inputs of the batched and serving
 * workloads; no counterpart in the reference, whose generators run on the
 * host, src/rand.cuh:49-217) ------------------------------------------------ */

/* n fp32 values uniform in [0, 1) (24-bit resolution) from a counter-based
 * hash of (seed, i): the same seed gives the same values on any GPU. */
int rmq_gen_values_device(float* d_out, uint64_t n, uint64_t seed, rmq_stream_t stream);

/* q inclusive queries over an array of n entries into d_lr (2q uint32):
 * law 0: length uniform in [1, n]; law 1: length = round(exp(N(ln median,
 * sigma))) clamped to [1, n]; l uniform in [0, n - len]. */
int rmq_gen_queries_device(uint32_t* d_lr, uint64_t q, uint64_t n, int32_t law, double median,
                           double sigma, uint64_t seed, rmq_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* RMQ_GB300_BATCH_H */
