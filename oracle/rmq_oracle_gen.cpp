// rmq_oracle_gen.cpp — seeded input generators of the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY.  The reference arm of the benchmark needs the
// same arrays and queries as the GPU arm without mapping any of the
// product's libraries, so the oracle carries its own restatement of the
// reference's generators (src/rand.cuh:49-240) and of the two added length
// laws.  The sequence of engine draws is the specification of these
// generators (the same libstdc++ engine and distribution types, called in the
// same order), so the results equal the reference's and the product's
// generators bit for bit; the CPU tests check both equalities (against the
// reference build when present, the committed fixtures, and the product
// generators).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

namespace {

// One query: a length from `len` (a callable drawing from `eng`), then l from
// a distribution object constructed for that length, as the reference does
// per query (src/rand.cuh:74-79).
template <typename Eng, typename Len>
void draw_queries(Eng& eng, Len&& len, uint32_t* out, uint64_t q, uint32_t n) {
    for (uint64_t i = 0; i < q; ++i) {
        const uint32_t s = len(eng);
        std::uniform_int_distribution<uint32_t> left(0, n - s);
        const uint32_t l = left(eng);
        out[2 * i] = l;
        out[2 * i + 1] = l + s - 1;
    }
}

// Reference lognormal lengths: truncated toward zero, redrawn while 0 or
// above n (src/rand.cuh:118-120).
struct RejectingLognormal {
    std::lognormal_distribution<double> d;
    uint32_t n;
    template <typename Eng>
    uint32_t operator()(Eng& eng) {
        for (;;) {
            const uint32_t s = static_cast<uint32_t>(d(eng));
            if (s != 0 && s <= n) return s;
        }
    }
};

// Added laws: rounded to nearest, clamped to [1, n].
struct ClampedLognormal {
    std::lognormal_distribution<double> d;
    uint32_t n;
    template <typename Eng>
    uint32_t operator()(Eng& eng) {
        const double x = std::nearbyint(d(eng));
        if (!(x >= 1.0)) return 1u;
        return x >= double(n) ? n : static_cast<uint32_t>(x);
    }
};

// Seed mixing of the added laws (their engines are 64-bit).
uint64_t mixed_seed(int32_t seed, uint64_t law) {
    return uint64_t(uint32_t(seed)) * 0x9E3779B97F4A7C15ull + law;
}

int fill(uint32_t* out, uint64_t q, int32_t lr, uint32_t n, int32_t seed) {
    // The reference's laws -1..-5 and constant lengths use mt19937(seed * tid)
    // with tid = 0 (src/rand.cuh:70, :91, :112, :184): seed 0 whatever --seed.
    std::mt19937 zero(0);
    if (lr > 0) {
        if (uint64_t(lr) > n) return -1;
        const uint32_t c = uint32_t(lr);
        draw_queries(zero, [c](std::mt19937&) { return c; }, out, q, n);
        return 0;
    }
    switch (lr) {
        case -1: {
            std::uniform_int_distribution<uint32_t> d(1, n);
            draw_queries(zero, [&d](std::mt19937& e) { return d(e); }, out, q, n);
            return 0;
        }
        case -2:
        case -3:
        case -4:
        case -5: {
            uint32_t median;
            if (lr == -2) median = static_cast<uint32_t>(std::pow(double(n), 0.6));
            else if (lr == -3) median = static_cast<uint32_t>(std::pow(double(n), 0.3));
            else median = std::max<uint32_t>(1u, n / (lr == -4 ? (1u << 8) : (1u << 15)));
            // fill_queries_lognormal takes the median as an int (src/rand.cuh:108)
            RejectingLognormal len{std::lognormal_distribution<double>(std::log(int(median)), 0.3), n};
            draw_queries(zero, len, out, q, n);
            return 0;
        }
        case -6: {
            // fill_queries_mixed (src/rand.cuh:129-170): one engine seeded by
            // `seed`; per query a class pick, then that class's length, then l.
            std::mt19937 eng(seed);
            std::uniform_int_distribution<int> pick(0, 2);
            std::uniform_int_distribution<uint32_t> wide(1, n);
            RejectingLognormal mid{std::lognormal_distribution<double>(
                                       std::log(static_cast<uint32_t>(std::pow(double(n), 0.6))), 0.3), n};
            RejectingLognormal low{std::lognormal_distribution<double>(
                                       std::log(static_cast<uint32_t>(std::pow(double(n), 0.3))), 0.3), n};
            draw_queries(eng, [&](std::mt19937& e) {
                const int c = pick(e);
                return c == 0 ? wide(e) : c == 1 ? mid(e) : low(e);
            }, out, q, n);
            return 0;
        }
        case -7: {
            std::mt19937_64 eng(mixed_seed(seed, 7));
            ClampedLognormal len{std::lognormal_distribution<double>(std::log(8192.0), 1.0), n};
            draw_queries(eng, len, out, q, n);
            return 0;
        }
        case -8: {
            std::mt19937_64 eng(mixed_seed(seed, 8));
            std::uniform_int_distribution<int> pick(0, 2);
            std::uniform_int_distribution<uint32_t> wide(1, n);
            ClampedLognormal mid{std::lognormal_distribution<double>(std::log(8192.0), 1.0), n};
            ClampedLognormal low{std::lognormal_distribution<double>(std::log(32.0), 0.7), n};
            draw_queries(eng, [&](std::mt19937_64& e) {
                const int c = pick(e);
                return c == 0 ? wide(e) : c == 1 ? mid(e) : low(e);
            }, out, q, n);
            return 0;
        }
        default:
            return -1;
    }
}

}  // namespace

extern "C" {

// random_array_par_cpu (src/rand.cuh:49-61).
void oracle_gen_array(uint64_t n, int32_t seed, float* out) {
    std::mt19937 eng(seed);
    std::uniform_real_distribution<float> u(0, 1);
    for (uint64_t i = 0; i < n; ++i) out[i] = u(eng);
}

// random_queries_par_cpu (src/rand.cuh:181-217) without the trivial-check
// repetition, plus the added laws -7 and -8.  Returns 0, or -1 for an
// unknown law or a constant length above n.
int32_t oracle_gen_queries(uint64_t q, int32_t lr, uint64_t n, int32_t seed, uint32_t* out) {
    if (n == 0 || n > 0xFFFFFFFFull || out == nullptr) return -1;
    return fill(out, q, lr, uint32_t(n), seed);
}

// The tie stress of the large mixed workload: round(frac * n) distinct
// positions, drawn with mt19937_64 from the seed, set to the global minimum.
void oracle_plant_min_ties(float* a, uint64_t n, double frac, int32_t seed) {
    if (n == 0 || !(frac > 0.0)) return;
    float lowest = a[0];
    for (uint64_t i = 1; i < n; ++i) lowest = a[i] < lowest ? a[i] : lowest;
    const uint64_t want = std::min<uint64_t>(n, uint64_t(std::llround(frac * double(n))));
    std::vector<bool> hit(n, false);
    std::mt19937_64 eng(uint64_t(uint32_t(seed)) * 0xD1B54A32D192ED03ull + 1);
    std::uniform_int_distribution<uint64_t> pos(0, n - 1);
    for (uint64_t placed = 0; placed < want;) {
        const uint64_t p = pos(eng);
        if (hit[p]) continue;
        hit[p] = true;
        a[p] = lowest;
        ++placed;
    }
}

}  // extern "C"
