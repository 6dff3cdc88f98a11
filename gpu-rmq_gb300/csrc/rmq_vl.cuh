// rmq_vl.cuh — the VL query (one thread per query) as device functions,
// shared by the single-array kernel (rmq_query.cu) and the batched kernel
// (rmq_batch.cu).
#pragma once

#include "rmq_common.cuh"

namespace rmq {

// ---------------------------------------------------------------------------
// VL: thread per query
//
// Phase 1 takes the minimum over all pieces with a masked 8-wide min per
// 32-byte sector (one 256-bit load each).  For argmin it also remembers, at
// sector granularity, where that minimum was first seen: left pieces and the
// final piece are visited in ascending position order (strict "<" keeps the
// first), right pieces in descending order ("<=" lets the more-left sector
// win), and a left/final winner beats a right winner on equal values.
// Phase 2 re-reads only the winning sector, takes its first entry equal to the
// minimum and, for a coarse level, loads that entry's stored level-0 index.
// ---------------------------------------------------------------------------

// L2 eviction priorities (tuning knobs; 0 selects the default shown).
#ifndef RMQ_L0_HINT
#define RMQ_L0_HINT 0  // level-0 sectors: 0 = evict_first, 1 = evict_normal
#endif
#ifndef RMQ_UP_HINT
#define RMQ_UP_HINT 0  // coarse-level sectors: 0 = evict_last, 1 = evict_normal
#endif
#ifndef RMQ_IDX_HINT
#define RMQ_IDX_HINT 0  // argmin index lookups: 0 = evict_last, 1 = evict_normal
#endif

struct L2Policies {
    uint64_t fine;    // level 0: read once per query
    uint64_t coarse;  // levels >= 1: shared by all queries
};

__device__ __forceinline__ uint64_t policy_evict_normal() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ L2Policies make_policies() {
    return L2Policies{RMQ_L0_HINT == 0 ? policy_evict_first() : policy_evict_normal(),
                      RMQ_UP_HINT == 0 ? policy_evict_last() : policy_evict_normal()};
}

__device__ __forceinline__ uint32_t ld_index(const uint32_t* p) {
#if RMQ_IDX_HINT == 0
    uint32_t v;
    asm("{\n\t.reg .b64 pol;\n\t"
        "createpolicy.fractional.L2::evict_last.b64 pol, 1.0;\n\t"
        "ld.global.nc.L2::cache_hint.u32 %0, [%1], pol;\n\t}"
        : "=r"(v) : "l"(p));
    return v;
#else
    return __ldg(p);
#endif
}

// Loads the sector starting at s of level k.  Level 0 is the caller's array,
// which is not padded: a sector that crosses its end is read element-wise.
__device__ __forceinline__ void load_level_sector(const Levels& lv, uint32_t k, uint32_t s,
                                                  const L2Policies& pol, float (&v)[8]) {
    const float* base = lv.val[k];
    if (k > 0) {
        ld_sector_policy(base + s, v, pol.coarse);
    } else if (s + 8u <= lv.size[0]) {
        ld_sector_policy(base + s, v, pol.fine);
    } else {
        const uint32_t size = lv.size[0];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (s + j < size) ? base[s + j] : f_inf();
    }
}

// Minimum of v[j] for jlo <= j < jhi (+inf if empty).
__device__ __forceinline__ float sector_min(const float (&v)[8], uint32_t jlo, uint32_t jhi) {
    float w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) w[j] = (uint32_t(j) >= jlo && uint32_t(j) < jhi) ? v[j] : f_inf();
    const float a = fmin3(w[0], w[1], w[2]);
    const float b = fmin3(w[3], w[4], w[5]);
    return fmin3(a, b, fminf(w[6], w[7]));
}

// Sector-granular position of the first minimum.  meta packs the level
// (bits 0-7), jlo (bits 8-15) and jhi (bits 16-23); kNoPos = none yet.
struct Tracker {
    float v;
    uint32_t s;
    uint32_t meta;
};

__device__ __forceinline__ void tracker_init(Tracker& t) {
    t.v = f_inf();
    t.s = 0;
    t.meta = kNoPos;
}

template <bool ARGMIN, bool RIGHT>
__device__ __forceinline__ void scan_sector(const Levels& lv, uint32_t k, uint32_t s, uint32_t jlo,
                                            uint32_t jhi, const L2Policies& pol, float& m, Tracker& t) {
    float v[8];
    load_level_sector(lv, k, s, pol, v);
    const float sm = sector_min(v, jlo, jhi);
    m = fminf(m, sm);
    if (ARGMIN) {
        const bool take = RIGHT ? (sm <= t.v) : (sm < t.v);
        if (take) {
            t.v = sm;
            t.s = s;
            t.meta = k | (jlo << 8) | (jhi << 16);
        }
    }
}

// Ascending scan of [lo, hi) (lo < hi) at level k, sector by sector.
template <bool ARGMIN>
__device__ __forceinline__ void scan_fwd(const Levels& lv, uint32_t k, uint32_t lo, uint32_t hi,
                                         const L2Policies& pol, float& m, Tracker& t) {
    for (uint32_t s = lo & ~7u; s < hi; s += 8u) {
        const uint32_t jlo = s < lo ? lo - s : 0u;
        const uint32_t jhi = hi - s < 8u ? hi - s : 8u;
        scan_sector<ARGMIN, false>(lv, k, s, jlo, jhi, pol, m, t);
    }
}

// Descending scan of [lo, hi) (lo < hi) at level k (right pieces).
template <bool ARGMIN>
__device__ __forceinline__ void scan_bwd(const Levels& lv, uint32_t k, uint32_t lo, uint32_t hi,
                                         const L2Policies& pol, float& m, Tracker& t) {
    const uint32_t first = lo & ~7u;
    for (uint32_t s = (hi - 1u) & ~7u;; s -= 8u) {
        const uint32_t jlo = s < lo ? lo - s : 0u;
        const uint32_t jhi = hi - s < 8u ? hi - s : 8u;
        scan_sector<ARGMIN, true>(lv, k, s, jlo, jhi, pol, m, t);
        if (s == first) break;
    }
}

// Final pieces longer than this many entries (only possible at the top level,
// whose size is bounded by t) are scanned by the whole warp instead of one lane.
constexpr uint32_t kLongScan = 64;

// Phase 1 up to (not including) the final piece; returns the running minimum
// and leaves the final piece [l, r) at level k in the arguments.
template <int R, bool ARGMIN>
__device__ __forceinline__ float vl_descend(const Levels& lv, uint32_t& l, uint32_t& r, uint32_t& k,
                                            const L2Policies& pol, Tracker& tl, Tracker& tr) {
    constexpr uint32_t RF = 1u << R;
    float m = f_inf();
    k = 0;
    while (k + 1 < lv.num_levels && r - l > 2u * RF) {
        const uint32_t nl = (l + RF - 1) & ~(RF - 1);
        const uint32_t pr = r & ~(RF - 1);
        if (R == 3) {
            // rf = 8: each boundary piece is exactly one sector; issue both loads first.
            float a[8], b[8];
            const bool has_l = nl > l, has_r = r > pr;
            if (has_l) load_level_sector(lv, k, l & ~7u, pol, a);
            if (has_r) load_level_sector(lv, k, pr, pol, b);
            if (has_l) {
                const float sm = sector_min(a, l & 7u, 8u);
                m = fminf(m, sm);
                if (ARGMIN && sm < tl.v) {
                    tl.v = sm;
                    tl.s = l & ~7u;
                    tl.meta = k | ((l & 7u) << 8) | (8u << 16);
                }
            }
            if (has_r) {
                const float sm = sector_min(b, 0u, r - pr);
                m = fminf(m, sm);
                if (ARGMIN && sm <= tr.v) {
                    tr.v = sm;
                    tr.s = pr;
                    tr.meta = k | ((r - pr) << 16);
                }
            }
        } else {
            if (nl > l) scan_fwd<ARGMIN>(lv, k, l, nl, pol, m, tl);
            if (r > pr) scan_bwd<ARGMIN>(lv, k, pr, r, pol, m, tr);
        }
        l = nl >> R;
        r = pr >> R;
        ++k;
    }
    return m;
}

// Whole-warp scan of the final piece [lo, hi) of level k owned by lane
// `owner`: lane j reads sectors j, j + 32, ... of the piece (1 KiB contiguous
// per warp load), keeps its first sector holding its minimum, and the warp
// combines by (value, sector start) so the first sector holding the piece
// minimum wins; the owner merges it into its running minimum and tracker.
template <bool ARGMIN>
__device__ __forceinline__ void warp_scan_final(const Levels& lv, uint32_t k, uint32_t lo, uint32_t hi,
                                                uint32_t owner, const L2Policies& pol, float& m, Tracker& tl) {
    const uint32_t lane = threadIdx.x & 31u;
    float best = f_inf();
    uint32_t bs = kNoPos;
    for (uint32_t s = (lo & ~7u) + 8u * lane; s < hi; s += 256u) {
        const uint32_t jlo = s < lo ? lo - s : 0u;
        const uint32_t jhi = hi - s < 8u ? hi - s : 8u;
        float v[8];
        load_level_sector(lv, k, s, pol, v);
        const float sm = sector_min(v, jlo, jhi);
        if (bs == kNoPos || sm < best) {
            best = sm;
            bs = s;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const uint32_t os = __shfl_xor_sync(0xffffffffu, bs, o);
        if (os != kNoPos && (bs == kNoPos || ov < best || (ov == best && os < bs))) {
            best = ov;
            bs = os;
        }
    }
    if (lane == owner) {
        m = fminf(m, best);
        if (ARGMIN && best < tl.v) {
            tl.v = best;
            tl.s = bs;
            const uint32_t jlo = bs < lo ? lo - bs : 0u;
            const uint32_t jhi = hi - bs < 8u ? hi - bs : 8u;
            tl.meta = k | (jlo << 8) | (jhi << 16);
        }
    }
}

// Phase 1 for every lane of the warp (all 32 lanes must call it): private
// descent and short final scans, then the warp's long final scans one by one.
template <int R, bool ARGMIN>
__device__ __forceinline__ float vl_phase1(const Levels& lv, bool active, uint32_t l, uint32_t r,
                                           const L2Policies& pol, Tracker& tl, Tracker& tr) {
    float m = f_inf();
    uint32_t k = 0;
    bool is_long = false;
    if (active) {
        m = vl_descend<R, ARGMIN>(lv, l, r, k, pol, tl, tr);
        if (r - l <= kLongScan) scan_fwd<ARGMIN>(lv, k, l, r, pol, m, tl);
        else is_long = true;
    }
    uint32_t pending = __ballot_sync(0xffffffffu, is_long);
    while (pending != 0u) {
        const uint32_t owner = uint32_t(__ffs(pending) - 1);
        const uint32_t ok = __shfl_sync(0xffffffffu, k, owner);
        const uint32_t olo = __shfl_sync(0xffffffffu, l, owner);
        const uint32_t ohi = __shfl_sync(0xffffffffu, r, owner);
        warp_scan_final<ARGMIN>(lv, ok, olo, ohi, owner, pol, m, tl);
        pending &= pending - 1u;
    }
    return m;
}

// Phase 2: first entry equal to the minimum inside the winning sector.
template <int R>
__device__ __forceinline__ void vl_locate(const Levels& lv, uint32_t l, const Tracker& tl, const Tracker& tr,
                                          const L2Policies& pol, float& out_v, uint32_t& out_i) {
    const bool right = tr.v < tl.v;
    const Tracker& w = right ? tr : tl;
    if (w.meta == kNoPos) {
        // No candidate compared below +inf: every entry is +inf (or NaN,
        // outside the contract); the scan's answer is the first entry.
        out_i = l;
        out_v = __ldg(lv.val[0] + l);
        return;
    }
    const uint32_t k = w.meta & 0xffu;
    const uint32_t jlo = (w.meta >> 8) & 0xffu;
    const uint32_t jhi = (w.meta >> 16) & 0xffu;
    float v[8];
    load_level_sector(lv, k, w.s, pol, v);
    uint32_t j = jlo;
#pragma unroll
    for (int jj = 7; jj >= 0; --jj) {
        if (uint32_t(jj) >= jlo && uint32_t(jj) < jhi && v[jj] == w.v) j = uint32_t(jj);
    }
    float val = v[0];
#pragma unroll
    for (int jj = 1; jj < 8; ++jj) val = (uint32_t(jj) == j) ? v[jj] : val;
    const uint32_t e = w.s + j;
    out_v = val;
    out_i = k == 0 ? e : ld_index(lv.idx[k] + e);
}

// One query per thread, no memory writes: every lane of the warp must call
// it (long final scans are shared by the warp).  For a valid query
// (0 <= l <= r < n) returns true with the minimum in v and, for ARGMIN, the
// argmin in idx; an invalid or absent (active = false) query returns false.
template <int R, bool ARGMIN>
__device__ __forceinline__ bool vl_compute(const Levels& lv, uint2 Q, bool active, float& v, uint32_t& idx) {
    const bool valid = active && Q.x <= Q.y && Q.y < lv.size[0];
    const L2Policies pol = make_policies();
    const uint32_t l = Q.x, r = Q.y + 1;
    Tracker tl, tr;
    tracker_init(tl);
    tracker_init(tr);
    idx = kNoPos;
    if (ARGMIN) {
        vl_phase1<R, true>(lv, valid, l, r, pol, tl, tr);
        v = f_nan();
        if (valid) vl_locate<R>(lv, l, tl, tr, pol, v, idx);
    } else {
        float m = vl_phase1<R, false>(lv, valid, l, r, pol, tl, tr);
        // A zero minimum may be -0.0 or +0.0; the reference returns the bits of
        // the first occurrence, so locate it (warp-uniform participation).
        const bool zero = valid && m == 0.0f;
        if (__any_sync(0xffffffffu, zero)) {
            vl_phase1<R, true>(lv, zero, l, r, pol, tl, tr);
            if (zero) vl_locate<R>(lv, l, tl, tr, pol, m, idx);
        }
        v = valid ? m : f_nan();
    }
    return valid;
}

// Stores of one answered query: NaN / kNoPos for an invalid query, which is
// also counted in *err when err is given.
template <bool ARGMIN>
__device__ __forceinline__ void vl_store(bool in_range, bool valid, float v, uint32_t idx, float* out_min,
                                         uint32_t* out_idx, uint32_t* err) {
    if (!in_range) return;
    if (out_min != nullptr) st_stream(out_min, v);
    if (ARGMIN) st_stream(out_idx, idx);
    if (!valid && err != nullptr) atomicAdd(err, 1u);
}

// Query i of qs (when in_range) into out_min[i] / out_idx[i]; every lane of
// the warp must call it.
template <int R, bool ARGMIN>
__device__ __forceinline__ void vl_answer(const Levels& lv, const uint2* __restrict__ qs, uint32_t i,
                                          bool in_range, float* __restrict__ out_min,
                                          uint32_t* __restrict__ out_idx, uint32_t* __restrict__ err) {
    uint2 Q = make_uint2(1u, 0u);
    if (in_range) Q = ld_query(qs + i);
    float v;
    uint32_t idx;
    const bool valid = vl_compute<R, ARGMIN>(lv, Q, in_range, v, idx);
    vl_store<ARGMIN>(in_range, valid, v, idx, out_min != nullptr ? out_min + i : nullptr,
                     ARGMIN ? out_idx + i : nullptr, err);
}

}  // namespace rmq
