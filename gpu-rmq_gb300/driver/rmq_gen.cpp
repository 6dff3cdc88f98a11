// rmq_gen.cpp — seeded host input generators (see include/rmq_gb300_gen.h).
//
// The reference's inputs come from libstdc++ engines and distributions
// (src/rand.cuh:49-217).  To give the same arrays and queries for the same
// command line, the draws below are taken from the same engine and
// distribution types in the same order: that order is the generator's
// specification, so it is kept exactly.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/rmq_gb300_gen.h"

namespace {

using u32 = uint32_t;

inline void put(uint32_t* out, uint64_t i, u32 l, u32 len) {
    out[2 * i] = l;
    out[2 * i + 1] = l + (len - 1);
}

// l uniform in [0, n - len] drawn from a fresh distribution object, as the
// reference constructs one per query.
template <typename Engine>
inline u32 draw_left(Engine& gen, u32 n, u32 len) {
    std::uniform_int_distribution<u32> lrand(0, n - 1 - (len - 1));
    return lrand(gen);
}

// Lognormal length with the reference's rejection of 0 and > n
// (src/rand.cuh:118-120): truncation toward zero, then redraw.
template <typename Engine>
inline u32 draw_lognormal_reject(Engine& gen, std::lognormal_distribution<double>& d, u32 n) {
    u32 len;
    do {
        len = static_cast<u32>(d(gen));
    } while (len == 0 || len > n);
    return len;
}

// Lognormal length rounded to nearest and clamped to [1, n] (GB300 workloads).
template <typename Engine>
inline u32 draw_lognormal_clamp(Engine& gen, std::lognormal_distribution<double>& d, u32 n) {
    const double x = std::nearbyint(d(gen));
    if (!(x >= 1.0)) return 1;
    if (x >= double(n)) return n;
    return static_cast<u32>(x);
}

void gen_constant(uint32_t* out, uint64_t q, u32 n, u32 len) {
    std::mt19937 gen(0);  // the reference seeds with seed * thread_id = 0
    for (uint64_t i = 0; i < q; ++i) put(out, i, draw_left(gen, n, len), len);
}

void gen_uniform(uint32_t* out, uint64_t q, u32 n) {
    std::mt19937 gen(0);
    std::uniform_int_distribution<u32> dist(1, n);
    for (uint64_t i = 0; i < q; ++i) {
        const u32 len = dist(gen);
        put(out, i, draw_left(gen, n, len), len);
    }
}

void gen_lognormal(uint32_t* out, uint64_t q, u32 n, int scale) {
    std::mt19937 gen(0);
    std::lognormal_distribution<double> dist(std::log(scale), 0.3);
    for (uint64_t i = 0; i < q; ++i) {
        const u32 len = draw_lognormal_reject(gen, dist, n);
        put(out, i, draw_left(gen, n, len), len);
    }
}

void gen_mixed_reference(uint32_t* out, uint64_t q, u32 n, int seed) {
    std::mt19937 gen(seed);
    std::uniform_int_distribution<int> pick(0, 2);
    std::uniform_int_distribution<u32> d_uniform(1, n);
    std::lognormal_distribution<double> d_medium(std::log(static_cast<u32>(std::pow(double(n), 0.6))), 0.3);
    std::lognormal_distribution<double> d_small(std::log(static_cast<u32>(std::pow(double(n), 0.3))), 0.3);
    for (uint64_t i = 0; i < q; ++i) {
        const int c = pick(gen);
        u32 len;
        if (c == 0) len = d_uniform(gen);
        else if (c == 1) len = draw_lognormal_reject(gen, d_medium, n);
        else len = draw_lognormal_reject(gen, d_small, n);
        put(out, i, draw_left(gen, n, len), len);
    }
}

// -7: lognormal(median 2^13, sigma 1.0), rounded, clamped.
void gen_medium_lognormal(uint32_t* out, uint64_t q, u32 n, int seed) {
    std::mt19937_64 gen(uint64_t(uint32_t(seed)) * 0x9E3779B97F4A7C15ull + 7);
    std::lognormal_distribution<double> d(std::log(8192.0), 1.0);
    for (uint64_t i = 0; i < q; ++i) {
        const u32 len = draw_lognormal_clamp(gen, d, n);
        put(out, i, draw_left(gen, n, len), len);
    }
}

// -8: thirds of uniform [1, n], lognormal(2^13, 1.0), lognormal(2^5, 0.7).
void gen_large_mixture(uint32_t* out, uint64_t q, u32 n, int seed) {
    std::mt19937_64 gen(uint64_t(uint32_t(seed)) * 0x9E3779B97F4A7C15ull + 8);
    std::uniform_int_distribution<int> pick(0, 2);
    std::uniform_int_distribution<u32> d_uniform(1, n);
    std::lognormal_distribution<double> d_medium(std::log(8192.0), 1.0);
    std::lognormal_distribution<double> d_short(std::log(32.0), 0.7);
    for (uint64_t i = 0; i < q; ++i) {
        const int c = pick(gen);
        u32 len;
        if (c == 0) len = d_uniform(gen);
        else if (c == 1) len = draw_lognormal_clamp(gen, d_medium, n);
        else len = draw_lognormal_clamp(gen, d_short, n);
        put(out, i, draw_left(gen, n, len), len);
    }
}

int fill_queries(uint32_t* out, uint64_t q, int lr, u32 n, int seed) {
    if (lr > 0) {
        if (uint64_t(lr) > n) return -1;
        gen_constant(out, q, n, u32(lr));
    } else if (lr == -1) {
        gen_uniform(out, q, n);
    } else if (lr == -2) {
        gen_lognormal(out, q, n, int(static_cast<u32>(std::pow(double(n), 0.6))));
    } else if (lr == -3) {
        gen_lognormal(out, q, n, int(static_cast<u32>(std::pow(double(n), 0.3))));
    } else if (lr == -4) {
        gen_lognormal(out, q, n, int(std::max<u32>(1u, n / (1u << 8))));
    } else if (lr == -5) {
        gen_lognormal(out, q, n, int(std::max<u32>(1u, n / (1u << 15))));
    } else if (lr == -6) {
        gen_mixed_reference(out, q, n, seed);
    } else if (lr == -7) {
        gen_medium_lognormal(out, q, n, seed);
    } else if (lr == -8) {
        gen_large_mixture(out, q, n, seed);
    } else {
        return -1;
    }
    return 0;
}

}  // namespace

extern "C" {

void rmq_gen_array(uint64_t n, int32_t seed, float* out) {
    std::mt19937 gen(seed);
    std::uniform_real_distribution<float> dist(0, 1);
    for (uint64_t i = 0; i < n; ++i) out[i] = dist(gen);
}

int32_t rmq_gen_queries(uint64_t q, int32_t lr, uint64_t n, int32_t seed, int32_t trivial,
                        uint32_t* out) {
    if (n == 0 || n > 0xFFFFFFFFull || out == nullptr) return -1;
    const u32 nn = u32(n);
    constexpr uint64_t kTrivial = uint64_t(1) << 10;  // TRIVCHECK_LOG_NUM_DIFFQ, src/main.cu:30
    if (trivial && q > kTrivial) {
        if (fill_queries(out, kTrivial, lr, nn, seed) != 0) return -1;
        for (uint64_t i = kTrivial; i < q; ++i) {
            out[2 * i] = out[2 * (i & (kTrivial - 1))];
            out[2 * i + 1] = out[2 * (i & (kTrivial - 1)) + 1];
        }
        return 0;
    }
    return fill_queries(out, q, lr, nn, seed);
}

void rmq_gen_plant_min_ties(float* a, uint64_t n, double frac, int32_t seed) {
    if (n == 0 || !(frac > 0.0)) return;
    float m = a[0];
    for (uint64_t i = 1; i < n; ++i)
        if (a[i] < m) m = a[i];
    uint64_t want = uint64_t(std::llround(frac * double(n)));
    if (want > n) want = n;
    std::vector<uint64_t> taken((n + 63) / 64, 0);
    std::mt19937_64 gen(uint64_t(uint32_t(seed)) * 0xD1B54A32D192ED03ull + 1);
    std::uniform_int_distribution<uint64_t> pos(0, n - 1);
    uint64_t done = 0;
    while (done < want) {
        const uint64_t p = pos(gen);
        uint64_t& w = taken[p >> 6];
        const uint64_t bit = uint64_t(1) << (p & 63);
        if (w & bit) continue;
        w |= bit;
        a[p] = m;
        ++done;
    }
}

uint64_t rmq_gen_sample_indices(uint64_t original_size, uint64_t sample_size, int32_t seed,
                                uint32_t* out) {
    if (original_size <= sample_size) {
        for (uint64_t i = 0; i < original_size; ++i) out[i] = u32(i);
        return original_size;
    }
    std::mt19937 gen(seed);
    for (uint64_t i = 0; i < sample_size; ++i) {
        std::uniform_int_distribution<u32> dis(0, u32(original_size - 1));
        out[i] = dis(gen);
    }
    return sample_size;
}

}  // extern "C"
