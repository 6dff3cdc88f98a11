/*
 * rmq_oracle.c — CPU oracle for the hierarchical range-minimum path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library or driver links,
 * loads or calls this file; only the tests, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py use it, always as the checker or
 * as the timed CPU baseline, never as the thing measured on the GPU.
 *
 * Parity pin: the brute-force functions below are checked, in the CPU test
 * suite, against the reference's own cpu_rmq / cpu_rmq_idx compiled from the
 * reference sources (oracle/build_ref.sh) and against committed fixtures
 * produced by that build (tests/golden/).
 *
 * Contents
 *   oracle_cpu_rmq / _idx        cpu_rmq / cpu_rmq_idx as the reference runs
 *                                them (default OpenMP schedule): the timed
 *                                CPU baseline
 *   oracle_min / oracle_argmin   restatement of cpu_min / cpu_min_idx
 *                                (src/cpu_methods.h:7-16, :42-53) run over a
 *                                query batch as cpu_rmq / cpu_rmq_idx do
 *                                (src/cpu_methods.h:18-39, :55-77): the scan
 *                                starts with A[l] and only a strictly smaller
 *                                value replaces it, so ties go to the lowest
 *                                index.
 *   oracle_sparse_*              an independent fast oracle for full-size
 *                                checks: block minima (64 entries) plus a
 *                                sparse table over blocks, combined by
 *                                (value, index); validated against brute force.
 *   oracle_layout                restatement of the level-layout loop
 *                                (src/xxx.h:225-243, src/xxx.h:958-977).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- brute force (src/cpu_methods.h:7-16, :42-53) ---------------------- */

static float scan_min(const float* A, uint32_t l, uint32_t r) {
    float m = A[l];
    for (uint64_t i = l; i <= r; ++i) {
        if (A[i] < m) m = A[i];
    }
    return m;
}

static uint32_t scan_argmin(const float* A, uint32_t l, uint32_t r) {
    float m = A[l];
    uint32_t mi = l;
    for (uint64_t i = l; i <= r; ++i) {
        if (A[i] < m) {
            m = A[i];
            mi = (uint32_t)i;
        }
    }
    return mi;
}

/* Q holds q inclusive pairs {l, r}.  Invalid pairs (l > r or r >= n) produce
 * NaN / 0xFFFFFFFF, the library's convention for invalid queries (the
 * reference does not check and reads out of bounds).  The checker: queries
 * are dealt out dynamically (64 at a time), which keeps the threads busy on
 * mixed lengths. */
void oracle_min(const float* A, uint64_t n, const uint32_t* Q, uint64_t q, float* out, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < (int64_t)q; ++i) {
        const uint32_t l = Q[2 * i], r = Q[2 * i + 1];
        if (l > r || (uint64_t)r >= n) {
            uint32_t nanbits = 0x7fc00000u;
            memcpy(&out[i], &nanbits, 4);
            continue;
        }
        out[i] = scan_min(A, l, r);
    }
    (void)nthreads;
}

void oracle_argmin(const float* A, uint64_t n, const uint32_t* Q, uint64_t q, uint32_t* out,
                   int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < (int64_t)q; ++i) {
        const uint32_t l = Q[2 * i], r = Q[2 * i + 1];
        if (l > r || (uint64_t)r >= n) {
            out[i] = 0xFFFFFFFFu;
            continue;
        }
        out[i] = scan_argmin(A, l, r);
    }
    (void)nthreads;
}

/* cpu_rmq / cpu_rmq_idx as the reference runs them (src/cpu_methods.h:18-39,
 * :55-77): one OpenMP parallel for over the queries with the default
 * schedule, each query a cpu_min / cpu_min_idx scan.  The timed CPU baseline;
 * valid queries only (the reference does not check them). */
void oracle_cpu_rmq(const float* A, const uint32_t* Q, uint64_t q, float* out, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for
#endif
    for (int64_t i = 0; i < (int64_t)q; ++i) out[i] = scan_min(A, Q[2 * i], Q[2 * i + 1]);
    (void)nthreads;
}

void oracle_cpu_rmq_idx(const float* A, const uint32_t* Q, uint64_t q, uint32_t* out, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for
#endif
    for (int64_t i = 0; i < (int64_t)q; ++i) out[i] = scan_argmin(A, Q[2 * i], Q[2 * i + 1]);
    (void)nthreads;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- fast oracle: block minima + sparse table over blocks --------------- */

#define SB_LOG 6
#define SB (1u << SB_LOG)

typedef struct {
    const float* A;
    uint64_t n;
    uint64_t nb;      /* number of blocks */
    int levels;       /* sparse-table levels */
    uint32_t* table;  /* levels x nb argmin indices into A */
} oracle_sparse;

/* (value, index) order: smaller value first, then lower index. */
static uint32_t better(const float* A, uint32_t a, uint32_t b) {
    if (A[b] < A[a]) return b;
    if (A[a] < A[b]) return a;
    return a < b ? a : b;
}

oracle_sparse* oracle_sparse_build(const float* A, uint64_t n) {
    oracle_sparse* s = (oracle_sparse*)calloc(1, sizeof(oracle_sparse));
    if (!s) return NULL;
    s->A = A;
    s->n = n;
    s->nb = (n + SB - 1) / SB;
    int lv = 1;
    while (((uint64_t)1 << lv) <= s->nb) ++lv;
    s->levels = lv;
    s->table = (uint32_t*)malloc(sizeof(uint32_t) * s->nb * (uint64_t)lv);
    if (!s->table) {
        free(s);
        return NULL;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t b = 0; b < (int64_t)s->nb; ++b) {
        uint64_t lo = (uint64_t)b * SB, hi = lo + SB;
        if (hi > n) hi = n;
        s->table[b] = scan_argmin(A, (uint32_t)lo, (uint32_t)(hi - 1));
    }
    for (int k = 1; k < lv; ++k) {
        uint32_t* prev = s->table + (uint64_t)(k - 1) * s->nb;
        uint32_t* cur = s->table + (uint64_t)k * s->nb;
        const uint64_t half = (uint64_t)1 << (k - 1);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t b = 0; b < (int64_t)s->nb; ++b) {
            if ((uint64_t)b + half < s->nb) cur[b] = better(A, prev[b], prev[b + half]);
            else cur[b] = prev[b];
        }
    }
    return s;
}

void oracle_sparse_free(oracle_sparse* s) {
    if (!s) return;
    free(s->table);
    free(s);
}

static uint32_t sparse_argmin(const oracle_sparse* s, uint32_t l, uint32_t r) {
    const float* A = s->A;
    const uint64_t bl = l >> SB_LOG, br = r >> SB_LOG;
    if (br - bl <= 1) return scan_argmin(A, l, r);
    /* left partial block, full blocks (bl, br), right partial block */
    uint32_t best = scan_argmin(A, l, (uint32_t)((bl + 1) * SB - 1));
    const uint64_t fb = bl + 1, lb = br - 1, cnt = lb - fb + 1;
    int k = 0;
    while (((uint64_t)1 << (k + 1)) <= cnt) ++k;
    const uint32_t* row = s->table + (uint64_t)k * s->nb;
    best = better(A, best, row[fb]);
    best = better(A, best, row[lb + 1 - ((uint64_t)1 << k)]);
    best = better(A, best, scan_argmin(A, (uint32_t)(br * SB), r));
    return best;
}

void oracle_sparse_query(const oracle_sparse* s, const uint32_t* Q, uint64_t q, float* out_min,
                         uint32_t* out_idx, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static, 1024)
#endif
    for (int64_t i = 0; i < (int64_t)q; ++i) {
        const uint32_t l = Q[2 * i], r = Q[2 * i + 1];
        if (l > r || (uint64_t)r >= s->n) {
            uint32_t nanbits = 0x7fc00000u;
            if (out_min) memcpy(&out_min[i], &nanbits, 4);
            if (out_idx) out_idx[i] = 0xFFFFFFFFu;
            continue;
        }
        const uint32_t a = sparse_argmin(s, l, r);
        if (out_min) out_min[i] = s->A[a];
        if (out_idx) out_idx[i] = a;
    }
    (void)nthreads;
}

/* ---- level layout (src/xxx.h:225-243) ----------------------------------- */

/* Writes num_levels and the per-level sizes and buffer offsets (entries) of
 * the hierarchy built over n entries with reduction factor 2^rf_log and scan
 * threshold t.  Offsets of level k >= 1 are aligned to 32 entries; level 0's
 * offset is the all-ones sentinel.  At most 20 levels. */
void oracle_layout(uint64_t n, uint64_t t, int rf_log, uint32_t* num_levels, uint64_t* sizes,
                   uint64_t* offsets) {
    const uint64_t rf = (uint64_t)1 << rf_log;
    uint32_t levels = 1;
    uint64_t size = n, off = 0;
    sizes[0] = n;
    offsets[0] = ~(uint64_t)0;
    for (;;) {
        if (levels >= 20 || size <= t) break;
        size = (size + rf - 1) >> rf_log;
        off = (off + 31) & ~(uint64_t)31;
        offsets[levels] = off;
        sizes[levels] = size;
        levels++;
        off += size;
    }
    *num_levels = levels;
}
