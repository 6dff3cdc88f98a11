/*
 * rmq_gb300_serve.h — a range-minimum query server: built structures stay
 * resident in device memory, new arrays are admitted against a fixed HBM
 * budget with least-recently-used eviction, and query requests of any size
 * are coalesced into shared launches while earlier batches still run
 * (continuous batching over several in-flight slots).  The reference has no
 * server (its driver answers one array per process run, src/main.cu:71-287);
 * per query the results are exactly those of rmq_query_idx.
 */
#ifndef RMQ_GB300_SERVE_H
#define RMQ_GB300_SERVE_H

#include <stdint.h>

#include "rmq_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rmq_server rmq_server;

typedef struct {
    uint64_t hbm_budget_bytes;    /* device arena for values + levels (default 64 GiB)           */
    uint32_t slots;               /* batches in flight at once, each on its own stream (default 4) */
    uint64_t max_batch_queries;   /* queries per batch launch (default 2^21; >= 2^16)             */
    uint32_t max_batch_requests;  /* requests per batch (default 4096)                            */
    uint64_t scan_threshold;      /* t of every served array (default 64)                         */
    uint32_t query_threads;       /* CTA size of the query kernel (default 256)                   */
} rmq_server_config;

typedef struct {
    uint64_t requests_done;
    uint64_t queries_done;
    uint64_t batches;
    uint64_t registrations;
    uint64_t evictions;
    uint64_t readmissions;
    uint64_t resident_arrays;
    uint64_t resident_bytes;
    uint64_t max_requests_per_batch;
    uint64_t max_batches_in_flight;
    uint64_t direct_requests;  /* requests whose page-locked buffers the kernel read and wrote in place */
} rmq_server_stats;

/* One event of a recorded request stream (rmq_server_replay). */
typedef struct {
    double   t_arrival_s;  /* offset from the start of the replay                          */
    int32_t  kind;         /* 0 = query request, 1 = register a generated array             */
    uint64_t array_id;     /* kind 0: target array                                          */
    uint64_t n;            /* kind 1: size of the new array                                 */
    uint64_t seed;         /* kind 1: its seed (values from rmq_gen_values_device)          */
    uint64_t q_offset;     /* kind 0: queries h_lr[2 q_offset ..], results at q_offset      */
    uint64_t q;            /* kind 0: number of queries                                     */
} rmq_trace_event;

void rmq_server_config_init(rmq_server_config* cfg);

/* Allocates the arena (one cudaMalloc of the budget) and the slots' staging
 * buffers, and starts the dispatcher thread on the current device. */
int rmq_server_create(const rmq_server_config* cfg, rmq_server** out);

/* Registers an array whose values the server generates on the device from
 * `seed` (rmq_gen_values_device); if it is evicted later, a request for it
 * re-admits it by regenerating and rebuilding.  Ids are assigned in
 * registration order from 0.  Returns RMQ_ERR_OOM when the array cannot fit
 * even after evicting every idle array. */
int rmq_server_register_generated(rmq_server* s, uint64_t n, uint64_t seed, uint64_t* array_id);

/* Registers an array from host memory; the server keeps the pointer (the
 * buffer must stay valid while the array is registered) to re-upload it
 * after an eviction. */
int rmq_server_register_host(rmq_server* s, const float* h_values, uint64_t n, uint64_t* array_id);

/* Submits q inclusive queries (h_lr[2i] = l, h_lr[2i+1] = r) on array_id.
 * The server writes the argmin and / or minimum of each query into h_argmin
 * / h_min (either may be NULL, not both); the buffers must stay valid until
 * the request is done.  Non-blocking.  When every buffer given is
 * page-locked and mapped (cudaHostAlloc, cudaHostRegister; h_lr 8-byte and
 * the results 4-byte aligned), the batch's kernel reads the queries and
 * writes the results in place over the CPU-GPU link; otherwise the server
 * copies them through its pinned staging buffers. */
int rmq_server_submit(rmq_server* s, uint64_t array_id, const uint32_t* h_lr, uint64_t q, uint32_t* h_argmin,
                      float* h_min, uint64_t* request_id);

/* Waits for a request: its status (RMQ_OK; RMQ_ERR_QUERY_RANGE when a
 * query was invalid; RMQ_ERR_CUDA when its batch could not be launched, its
 * argmin then all ones and its minima NaN), or RMQ_ERR_TIMEOUT when it is not done within
 * timeout_ms (< 0: no limit).  *latency_us (may be NULL): submit to results
 * in the host buffers.  A call that returns the status collects the request:
 * the server drops its record and the id is then unknown (RMQ_ERR_ARG);
 * records of requests that are never waited for are kept until
 * rmq_server_destroy. */
int rmq_server_wait(rmq_server* s, uint64_t request_id, int64_t timeout_ms, double* latency_us);

/* Waits until every submitted request is done (RMQ_ERR_TIMEOUT otherwise). */
int rmq_server_drain(rmq_server* s, int64_t timeout_ms);

/* Replays a request stream from the calling thread: each event is issued at
 * its arrival time (registrations and submissions), then the call drains.
 * latency_us[i] receives event i's latency (-1 for registrations and
 * rejected requests); *wall_s the time from the first arrival to the last
 * completion. */
int rmq_server_replay(rmq_server* s, const rmq_trace_event* events, uint64_t count, const uint32_t* h_lr,
                      uint32_t* h_argmin, float* h_min, double* latency_us, double* wall_s);

int rmq_server_get_stats(rmq_server* s, rmq_server_stats* stats);

/* The comparator of the server: the query requests (kind 0) of `events`
 * answered one after another, each by rmq_query_idx_host on a prebuilt
 * handle of its array (handles[array_id], num_handles of them) and waited for
 * before the next one starts: a caller's per-request loop of the plain
 * kernel, without batching or overlap.  Arrival times are ignored; results
 * land at the same positions as rmq_server_replay's.  *wall_s (may be NULL):
 * time of the whole loop.  Returns the first failing call's status. */
int rmq_serve_serial_loop(rmq_handle* const* handles, uint64_t num_handles, const rmq_trace_event* events,
                          uint64_t count, const uint32_t* h_lr, uint32_t* h_argmin, float* h_min, double* wall_s);

/* Fault injection for tests of the failure path: the next `count` batches
 * the dispatcher packs fail as if their upload had returned a CUDA error
 * (nothing of theirs is issued to the device); their requests complete with
 * RMQ_ERR_CUDA.  count = 0 cancels what is left.  Made on the host: no
 * device work fails. */
int rmq_server_fail_next_batches(rmq_server* s, uint32_t count);

/* Stops the dispatcher (after finishing queued work) and frees everything. */
void rmq_server_destroy(rmq_server* s);

#ifdef __cplusplus
}
#endif

#endif /* RMQ_GB300_SERVE_H */
