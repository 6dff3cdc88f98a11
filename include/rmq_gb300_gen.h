/*
 * rmq_gb300_gen.h — seeded host-side input generators of the rtxrmq driver.
 *
 * The reference generates its inputs on the host with libstdc++ engines
 * (src/rand.cuh:49-217); these entry points reproduce that sequence of draws
 * bit for bit when built against the same libstdc++, and add the length laws
 * of the GB300 workloads (lr codes -7 and -8).  Host-only: no CUDA calls.
 */
#ifndef RMQ_GB300_GEN_H
#define RMQ_GB300_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Length-law codes (the reference's lr argument, src/tools.h:38-46):
 *   lr > 0  constant length lr                          (src/rand.cuh:65-84)
 *   -1      length uniform in [1, n]                     (src/rand.cuh:86-105)
 *   -2/-3   lognormal, median n^0.6 / n^0.3, sigma 0.3   (src/rand.cuh:107-127, :199-202)
 *   -4/-5   lognormal, median n/2^8 / n/2^15, sigma 0.3  (src/rand.cuh:203-206)
 *   -6      mixture of -1/-2/-3, seeded by `seed`        (src/rand.cuh:129-170)
 *   -7      lognormal, median 2^13, sigma 1.0, rounded and clamped to [1, n]   (new)
 *   -8      one third each of -1, lognormal(2^13, 1.0), lognormal(2^5, 0.7)   (new)
 * For every query l is uniform in [0, n - len] and r = l + len - 1. */

/* Replaces random_array_par_cpu (src/rand.cuh:49-61): n fp32 values uniform in
 * [0, 1) from mt19937(seed). */
void rmq_gen_array(uint64_t n, int32_t seed, float* out);

/* Replaces random_queries_par_cpu (src/rand.cuh:181-217): q inclusive pairs
 * written as out[2i] = l, out[2i+1] = r.  With `trivial` set and q > 2^10 only
 * 2^10 distinct queries are drawn and repeated (src/rand.cuh:172-179, :187-215).
 * As in the reference, codes lr > 0 and -1..-5 draw from mt19937(0) whatever
 * the seed (src/rand.cuh:70, :184).  Returns 0, or -1 for an unknown code or
 * a constant length above n. */
int32_t rmq_gen_queries(uint64_t q, int32_t lr, uint64_t n, int32_t seed, int32_t trivial,
                        uint32_t* out);

/* Tie stress for the large mixed workload: sets round(frac * n) distinct
 * positions, chosen with mt19937_64(seed), to the global minimum of a[0..n). */
void rmq_gen_plant_min_ties(float* a, uint64_t n, double frac, int32_t seed);

/* Replaces randomly_sample_indices (src/rand.cuh:219-240): sample_size indices
 * in [0, original_size) from mt19937(seed) (identity when the sample is not
 * smaller than the population). Returns the number written. */
uint64_t rmq_gen_sample_indices(uint64_t original_size, uint64_t sample_size, int32_t seed,
                                uint32_t* out);

#ifdef __cplusplus
}
#endif

#endif /* RMQ_GB300_GEN_H */
