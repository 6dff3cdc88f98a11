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
// minimum and, for a coarse level, that entry's stored level-0 index (for
// 32-bit handles the sector's eight indices come with the values).
//
// The thread's dependent chain of loads (one round trip per level) bounds the
// kernel, so every round trip counts: the two boundary sectors of a level are
// loaded together, forward scans take two sectors per round trip, and the
// small top levels are read through L1 (kL1LevelEntries).  Final pieces
// longer than kLongScan (top level only) are scanned by the whole warp one
// after another or, when that takes more round trips, by their own lanes.
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

__device__ __forceinline__ uint64_t ld_index(const uint64_t* p) {
#if RMQ_IDX_HINT == 0
    uint64_t v;
    asm("{\n\t.reg .b64 pol;\n\t"
        "createpolicy.fractional.L2::evict_last.b64 pol, 1.0;\n\t"
        "ld.global.nc.L2::cache_hint.u64 %0, [%1], pol;\n\t}"
        : "=l"(v) : "l"(p));
    return v;
#else
    return __ldg(reinterpret_cast<const unsigned long long*>(p));
#endif
}

// Coarse levels of at most this many entries (64 KiB of values; with the
// smaller levels above them at most ~73 KiB) are read through L1: every SM
// re-reads these top levels for many queries, and a query that descends to
// them otherwise pays an L2 round trip per level.  Larger levels, and level 0,
// bypass L1.  Measured at n = q = 2^26: uniform-length queries 9.2 -> 23.7 G
// queries/s, the three-way mixture 12.2 -> 20.8, the lognormal(2^13, 1)
// workload +1.4 %; including the 2^17-entry level (512 KiB) cost 5 % on the
// uniform law.  The stored indices of those levels (phase 2) likewise.  The
// CL kernel keeps every level out of L1 (TOP_L1 = false): its tiles re-read
// the same sectors from L2 lane by lane, and the extra branch cost it 2 %.
constexpr uint32_t kL1LevelEntries = 1u << 14;

// Loads the sector starting at s of level k.  Level 0 is the caller's array,
// which is not padded: a sector that crosses its end is read element-wise.
template <typename I, bool TOP_L1 = true>
__device__ __forceinline__ void load_level_sector(const LevelsT<I>& lv, uint32_t k, I s,
                                                  const L2Policies& pol, float (&v)[8]) {
#if RMQ_DEBUG_BOUNDS
    // Level 0 is read up to its last entry; a coarse level up to its 32-entry padding.
    if (!bounds_ok(k < lv.num_levels && (s & I(7)) == 0 &&
                   (k == 0 ? s < lv.size[0] : s + 8u <= ((lv.size[k] + 31u) & ~I(31))))) {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = f_inf();
        return;
    }
#endif
    const float* base = lv.val[k];
    if (k > 0) {
        if (TOP_L1 && lv.size[k] <= kL1LevelEntries) ld_sector_l1_policy(base + s, v, pol.coarse);
        else ld_sector_policy(base + s, v, pol.coarse);
    } else if (s + 8u <= lv.size[0]) {
        ld_sector_policy(base + s, v, pol.fine);
    } else {
        const I size = lv.size[0];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (s + I(j) < size) ? base[s + j] : f_inf();
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

// First entry of v in [jlo, jhi) equal to sm (the minimum over that range).
__device__ __forceinline__ uint32_t sector_first(const float (&v)[8], uint32_t jlo, uint32_t jhi, float sm) {
    uint32_t bits = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) bits |= (v[j] == sm ? 1u : 0u) << j;
    const uint32_t range = ((1u << jhi) - 1u) & ~((1u << jlo) - 1u);
    return uint32_t(__ffs(bits & range) - 1);
}

// The bits of v[j]: the minimum of a range holding both zeros is -0.0 for
// min.f32, but the answer carries the bits of the first one.
__device__ __forceinline__ float sector_bits(const float (&v)[8], uint32_t j, float sm) {
    if (sm != 0.0f) return sm;
    float x = v[0];
#pragma unroll
    for (int jj = 1; jj < 8; ++jj) x = (uint32_t(jj) == j) ? v[jj] : x;
    return x;
}

// Sector-granular position of the first minimum.  meta packs the level
// (bits 0-7), jlo (bits 8-15) and jhi (bits 16-23); kNoPos = none yet.  A
// level-0 candidate also carries its entry: jhi = jlo + 1 with kPosKnown
// set, and v holds that entry's own bits, so phase 2 needs no load for it
// (the sector, read once with evict-first, has usually left L2 by then).
constexpr uint32_t kPosKnown = 1u << 24;
// 32-bit handles only: the 64-bit kernels have no registers to spare.
template <typename I>
constexpr bool kCapture = sizeof(I) == 4;
// Only queries this short take their level-0 entries in phase 1 (the
// short-query variant): a longer query's minimum seldom lies in its level-0
// pieces.
constexpr uint32_t kCaptureLen = 512;

template <typename I>
struct Tracker {
    float v;
    I s;
    uint32_t meta;
};

template <typename I>
__device__ __forceinline__ void tracker_init(Tracker<I>& t) {
    t.v = f_inf();
    t.s = 0;
    t.meta = kNoPos;
}

// Folds the loaded sector v (start s of level k, entries [jlo, jhi)) into
// the running minimum and the side's candidate.
template <bool ARGMIN, bool RIGHT, typename I>
__device__ __forceinline__ void take_sector(const float (&v)[8], uint32_t k, I s, uint32_t jlo, uint32_t jhi,
                                            float& m, Tracker<I>& t) {
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

template <bool ARGMIN, bool RIGHT, typename I>
__device__ __forceinline__ void scan_sector(const LevelsT<I>& lv, uint32_t k, I s, uint32_t jlo,
                                            uint32_t jhi, const L2Policies& pol, float& m, Tracker<I>& t) {
    float v[8];
    load_level_sector(lv, k, s, pol, v);
    take_sector<ARGMIN, RIGHT>(v, k, s, jlo, jhi, m, t);
}

// Ascending scan of [lo, hi) (lo < hi) at level k, two sectors per round
// trip.
template <bool ARGMIN, typename I>
__device__ __forceinline__ void scan_fwd(const LevelsT<I>& lv, uint32_t k, I lo, I hi,
                                         const L2Policies& pol, float& m, Tracker<I>& t) {
    I s = lo & ~I(7);
    for (; s + 8u < hi; s += 16u) {
        // Sector s ends before hi; sector s + 8 starts before hi.
        float a[8], b[8];
        load_level_sector(lv, k, s, pol, a);
        load_level_sector(lv, k, s + 8u, pol, b);
        const I s2 = s + 8u;
        take_sector<ARGMIN, false>(a, k, s, s < lo ? uint32_t(lo - s) : 0u, 8u, m, t);
        take_sector<ARGMIN, false>(b, k, s2, 0u, hi - s2 < 8u ? uint32_t(hi - s2) : 8u, m, t);
    }
    if (s < hi) {
        const uint32_t jlo = s < lo ? uint32_t(lo - s) : 0u;
        const uint32_t jhi = hi - s < 8u ? uint32_t(hi - s) : 8u;
        scan_sector<ARGMIN, false>(lv, k, s, jlo, jhi, pol, m, t);
    }
}

// Descending scan of [lo, hi) (lo < hi) at level k (right pieces).
template <bool ARGMIN, typename I>
__device__ __forceinline__ void scan_bwd(const LevelsT<I>& lv, uint32_t k, I lo, I hi,
                                         const L2Policies& pol, float& m, Tracker<I>& t) {
    const I first = lo & ~I(7);
    for (I s = (hi - 1u) & ~I(7);; s -= 8u) {
        const uint32_t jlo = s < lo ? uint32_t(lo - s) : 0u;
        const uint32_t jhi = hi - s < 8u ? uint32_t(hi - s) : 8u;
        scan_sector<ARGMIN, true>(lv, k, s, jlo, jhi, pol, m, t);
        if (s == first) break;
    }
}

// Final pieces longer than this many entries (only possible at the top level,
// whose size is bounded by t) are scanned by the whole warp instead of one lane.
constexpr uint32_t kLongScan = 64;

// Level 0 of a short query's descent (rf = 8; the caller checked that the
// query spans more than two blocks): both boundary sectors in one round trip,
// and each side's first minimum taken with its entry and bits (kPosKnown),
// so that a level-0 winner needs no load in phase 2.
template <bool ARGMIN, typename I>
__device__ __forceinline__ float vl_level0_capture(const LevelsT<I>& lv, I& l, I& r, const L2Policies& pol,
                                                   Tracker<I>& tl, Tracker<I>& tr) {
    const I nl = (l + 7u) & ~I(7);
    const I pr = r & ~I(7);
    float a[8], b[8];
    const bool has_l = nl > l, has_r = r > pr;
    const uint32_t lo_j = uint32_t(l & 7u), hi_j = uint32_t(r - pr);
    if (has_l) load_level_sector(lv, 0u, l & ~I(7), pol, a);
    if (has_r) load_level_sector(lv, 0u, pr, pol, b);
    float m = f_inf();
    if (has_l) {
        const float sm = sector_min(a, lo_j, 8u);
        m = fminf(m, sm);
        if (ARGMIN && sm < tl.v) {
            const uint32_t j = sector_first(a, lo_j, 8u, sm);
            tl.v = sector_bits(a, j, sm);
            tl.s = l & ~I(7);
            tl.meta = (j << 8) | ((j + 1u) << 16) | kPosKnown;
        }
    }
    if (has_r) {
        const float sm = sector_min(b, 0u, hi_j);
        m = fminf(m, sm);
        if (ARGMIN && sm <= tr.v) {
            const uint32_t j = sector_first(b, 0u, hi_j, sm);
            tr.v = sector_bits(b, j, sm);
            tr.s = pr;
            tr.meta = (j << 8) | ((j + 1u) << 16) | kPosKnown;
        }
    }
    l = nl >> 3;
    r = pr >> 3;
    return m;
}

// Phase 1 up to (not including) the final piece; returns the running minimum
// and leaves the final piece [l, r) at level k in the arguments.  With CAP
// (the short-query variant), a short query's level 0 goes through
// vl_level0_capture, a separate step before the loop.
template <int R, bool ARGMIN, typename I, bool CAP = false>
__device__ __forceinline__ float vl_descend(const LevelsT<I>& lv, I& l, I& r, uint32_t& k,
                                            const L2Policies& pol, Tracker<I>& tl, Tracker<I>& tr) {
    constexpr I RF = I(1) << R;
    float m = f_inf();
    k = 0;
    if (R == 3 && CAP && kCapture<I> && ARGMIN && r - l <= I(kCaptureLen) && 1u < lv.num_levels &&
        r - l > 2u * RF) {
        m = vl_level0_capture<ARGMIN>(lv, l, r, pol, tl, tr);
        k = 1;
    }
    while (k + 1 < lv.num_levels && r - l > 2u * RF) {
        const I nl = (l + RF - 1) & ~(RF - 1);
        const I pr = r & ~(RF - 1);
        if (R == 3) {
            // rf = 8: each boundary piece is exactly one sector; issue both loads first.
            float a[8], b[8];
            const bool has_l = nl > l, has_r = r > pr;
            const uint32_t lo_j = uint32_t(l & 7u), hi_j = uint32_t(r - pr);
            if (has_l) load_level_sector(lv, k, l & ~I(7), pol, a);
            if (has_r) load_level_sector(lv, k, pr, pol, b);
            if (has_l) {
                const float sm = sector_min(a, lo_j, 8u);
                m = fminf(m, sm);
                if (ARGMIN && sm < tl.v) {
                    tl.v = sm;
                    tl.s = l & ~I(7);
                    tl.meta = k | (lo_j << 8) | (8u << 16);
                }
            }
            if (has_r) {
                const float sm = sector_min(b, 0u, hi_j);
                m = fminf(m, sm);
                if (ARGMIN && sm <= tr.v) {
                    tr.v = sm;
                    tr.s = pr;
                    tr.meta = k | (hi_j << 16);
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

// Unsigned key ordered like the float's value (NaN outside the contract):
// negative values map below positive ones with their order reversed, and
// -0.0 maps to the key of +0.0, as the two compare equal.
__device__ __forceinline__ uint32_t min_key(float x) {
    const uint32_t u = x == 0.0f ? 0u : __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Whole-warp scan of the final piece [lo, hi) of level k owned by lane
// `owner`: lane j reads sectors j, j + 32, ... of the piece (1 KiB contiguous
// per warp load), keeps its first sector holding its minimum, and the warp
// combines by (value, sector start) so the first sector holding the piece
// minimum wins; the owner merges it into its running minimum and tracker.
template <bool ARGMIN, typename I>
__device__ __forceinline__ void warp_scan_final(const LevelsT<I>& lv, uint32_t k, I lo, I hi,
                                                uint32_t owner, const L2Policies& pol, float& m, Tracker<I>& tl) {
    constexpr I kNone = IdxTraits<I>::none;
    const uint32_t lane = threadIdx.x & 31u;
    float best = f_inf();
    I bs = kNone;
    for (I s = (lo & ~I(7)) + 8u * lane; s < hi; s += 256u) {
        const uint32_t jlo = s < lo ? uint32_t(lo - s) : 0u;
        const uint32_t jhi = hi - s < 8u ? uint32_t(hi - s) : 8u;
        float v[8];
        load_level_sector(lv, k, s, pol, v);
        const float sm = sector_min(v, jlo, jhi);
        if (bs == kNone || sm < best) {
            best = sm;
            bs = s;
        }
    }
    if constexpr (sizeof(I) == 4) {
        // Two warp reductions (redux.sync): the smallest value, as an
        // order-preserving key with both zeros on one key (they compare
        // equal), then the lowest sector among lanes holding it; the winning
        // lane supplies the value's own bits.  A lane that scanned nothing
        // has sector kNone, the largest key.
        const uint32_t vk = min_key(best);
        const uint32_t mk = __reduce_min_sync(0xffffffffu, vk);
        const uint32_t ws = __reduce_min_sync(0xffffffffu, vk == mk ? uint32_t(bs) : uint32_t(kNone));
        const uint32_t wl = uint32_t(__ffs(__ballot_sync(0xffffffffu, vk == mk && uint32_t(bs) == ws)) - 1);
        best = __shfl_sync(0xffffffffu, best, wl);
        bs = I(ws);
    } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, o);
            const I os = __shfl_xor_sync(0xffffffffu, bs, o);
            if (os != kNone && (bs == kNone || ov < best || (ov == best && os < bs))) {
                best = ov;
                bs = os;
            }
        }
    }
    if (lane == owner) {
        m = fminf(m, best);
        if (ARGMIN && best < tl.v) {
            tl.v = best;
            tl.s = bs;
            const uint32_t jlo = bs < lo ? uint32_t(lo - bs) : 0u;
            const uint32_t jhi = hi - bs < 8u ? uint32_t(hi - bs) : 8u;
            tl.meta = k | (jlo << 8) | (jhi << 16);
        }
    }
}

// Phase 1 for every lane of the warp (all 32 lanes must call it): private
// descent and short final scans, then the warp's long final scans one by one.
template <int R, bool ARGMIN, typename I, bool CAP = false>
__device__ __forceinline__ float vl_phase1(const LevelsT<I>& lv, bool active, I l, I r,
                                           const L2Policies& pol, Tracker<I>& tl, Tracker<I>& tr) {
    float m = f_inf();
    uint32_t k = 0;
    bool is_long = false;
    if (active) {
        m = vl_descend<R, ARGMIN, I, CAP>(lv, l, r, k, pol, tl, tr);
        if (r - l <= kLongScan) scan_fwd<ARGMIN>(lv, k, l, r, pol, m, tl);
        else is_long = true;
    }
    uint32_t pending = __ballot_sync(0xffffffffu, is_long);
    if (pending != 0u && lv.size[lv.num_levels - 1] <= kL1LevelEntries) {
        // Long pieces lie in the top level.  When it is read through L1, the
        // scans are latency-bound: whole-warp scans take one round trip per
        // 32 sectors of each long piece, one piece after another; lane-private
        // scans one round trip per two sectors of the longest piece, all
        // pieces at once.  The warp takes whichever needs fewer round trips
        // (many long pieces: private; a few: whole-warp).  A larger top level
        // is read from L2, where the whole-warp scans' contiguous 1 KiB loads
        // use L2 better (lane-private scans of a 2^16-entry top level: -29 %).
        // Both visit a piece's sectors in ascending order with the same fold,
        // so the results are the same.
        uint32_t sec = 0;
        if (is_long) {
            const uint64_t span = uint64_t(((r - 1u) >> 3) - (l >> 3)) + 1u;
            sec = span < (1u << 26) ? uint32_t(span) : (1u << 26);
        }
        const uint32_t warp_trips = __reduce_add_sync(0xffffffffu, (sec + 31u) >> 5);
        const uint32_t lane_trips = __reduce_max_sync(0xffffffffu, (sec + 1u) >> 1);
        if (lane_trips < warp_trips) {
            if (is_long) scan_fwd<ARGMIN>(lv, k, l, r, pol, m, tl);
            pending = 0u;
        }
    }
    while (pending != 0u) {
        const uint32_t owner = uint32_t(__ffs(pending) - 1);
        const uint32_t ok = __shfl_sync(0xffffffffu, k, owner);
        const I olo = __shfl_sync(0xffffffffu, l, owner);
        const I ohi = __shfl_sync(0xffffffffu, r, owner);
        warp_scan_final<ARGMIN>(lv, ok, olo, ohi, owner, pol, m, tl);
        pending &= pending - 1u;
    }
    return m;
}

// Phase 2: first entry equal to the minimum inside the winning sector.  For
// a coarse winner of a 32-bit handle the sector's eight stored level-0
// indices (one 32-byte sector, level offsets are 32-entry aligned) are loaded
// together with its values, so the index needs no further round trip.
template <int R, typename I, bool CAP = false>
__device__ __forceinline__ void vl_locate(const LevelsT<I>& lv, I l, const Tracker<I>& tl, const Tracker<I>& tr,
                                          const L2Policies& pol, float& out_v, I& out_i) {
    const bool right = tr.v < tl.v;
    const Tracker<I>& w = right ? tr : tl;
    if (w.meta == kNoPos) {
        // No candidate compared below +inf: every entry is +inf (or NaN,
        // outside the contract); the scan's answer is the first entry.
        out_i = l;
        out_v = __ldg(lv.val[0] + l);
        return;
    }
    if (CAP && kCapture<I> && (w.meta & kPosKnown)) {
        // a level-0 winner: its entry and bits were taken in phase 1
        out_i = w.s + I((w.meta >> 8) & 0xffu);
        out_v = w.v;
        return;
    }
    const uint32_t k = w.meta & 0xffu;
    const uint32_t jlo = (w.meta >> 8) & 0xffu;
    const uint32_t jhi = (w.meta >> 16) & 0xffu;
    float v[8];
    load_level_sector(lv, k, w.s, pol, v);
    uint32_t ix[8];
    if constexpr (sizeof(I) == 4) {
#if RMQ_DEBUG_BOUNDS
        if (k > 0 && !bounds_ok(lv.idx[k] != nullptr && w.s + 8u <= ((lv.size[k] + 31u) & ~I(31)))) {
#pragma unroll
            for (int j = 0; j < 8; ++j) ix[j] = 0u;
        } else
#endif
        if (k > 0) {
            if (lv.size[k] <= kL1LevelEntries) ld_sector_u32_l1_policy(lv.idx[k] + w.s, ix, pol.coarse);
            else ld_sector_u32_policy(lv.idx[k] + w.s, ix, pol.coarse);
        }
    }
    uint32_t j = jlo;
#pragma unroll
    for (int jj = 7; jj >= 0; --jj) {
        if (uint32_t(jj) >= jlo && uint32_t(jj) < jhi && v[jj] == w.v) j = uint32_t(jj);
    }
    float val = v[0];
#pragma unroll
    for (int jj = 1; jj < 8; ++jj) val = (uint32_t(jj) == j) ? v[jj] : val;
    const I e = w.s + j;
    out_v = val;
    if constexpr (sizeof(I) == 4) {
        uint32_t x = ix[0];
#pragma unroll
        for (int jj = 1; jj < 8; ++jj) x = (uint32_t(jj) == j) ? ix[jj] : x;
        out_i = k == 0 ? e : x;
    } else {
#if RMQ_DEBUG_BOUNDS
        if (k > 0 && !bounds_ok(lv.idx[k] != nullptr && e < lv.size[k])) {
            out_i = 0;
            return;
        }
#endif
        out_i = k == 0 ? e : ld_index(lv.idx[k] + e);
    }
}

// One query per thread, no memory writes: every lane of the warp must call
// it (long final scans are shared by the warp).  For a valid query
// (0 <= l <= r < n) returns true with the minimum in v and, for ARGMIN, the
// argmin in idx; an invalid or absent (active = false) query returns false.
template <int R, bool ARGMIN, typename I, bool CAP = false>
__device__ __forceinline__ bool vl_compute(const LevelsT<I>& lv, typename IdxTraits<I>::Pair Q, bool active,
                                           float& v, I& idx) {
    const bool valid = active && Q.x <= Q.y && Q.y < lv.size[0];
    const L2Policies pol = make_policies();
    const I l = Q.x, r = Q.y + 1;
    Tracker<I> tl, tr;
    tracker_init(tl);
    tracker_init(tr);
    idx = IdxTraits<I>::none;
    if (ARGMIN) {
        vl_phase1<R, true, I, CAP>(lv, valid, l, r, pol, tl, tr);
        v = f_nan();
        if (valid) vl_locate<R, I, CAP>(lv, l, tl, tr, pol, v, idx);
    } else {
        float m = vl_phase1<R, false, I, CAP>(lv, valid, l, r, pol, tl, tr);
        // A zero minimum may be -0.0 or +0.0; the reference returns the bits of
        // the first occurrence.  min.f32 returns -0.0 whenever a -0.0 meets a
        // zero (checked on sm_103a, and by the signed-zero parity cases), so a
        // +0.0 minimum means the range holds no -0.0 and is already the answer;
        // only a -0.0 minimum needs the first zero located (warp-uniform
        // participation).
        const bool zero = valid && __float_as_uint(m) == 0x80000000u;
        if (__any_sync(0xffffffffu, zero)) {
            vl_phase1<R, true, I, CAP>(lv, zero, l, r, pol, tl, tr);
            if (zero) vl_locate<R, I, CAP>(lv, l, tl, tr, pol, m, idx);
        }
        v = valid ? m : f_nan();
    }
    return valid;
}

// Stores of one answered query: NaN / kNoPos for an invalid query, which is
// also counted in *err when err is given.
template <bool ARGMIN, typename I>
__device__ __forceinline__ void vl_store(bool in_range, bool valid, float v, I idx, float* out_min,
                                         I* out_idx, uint32_t* err) {
    if (!in_range) return;
    if (out_min != nullptr) st_stream(out_min, v);
    if (ARGMIN) st_stream(out_idx, idx);
    if (!valid && err != nullptr) atomicAdd(err, 1u);
}

// Query i of qs (when in_range) into out_min[i] / out_idx[i]; every lane of
// the warp must call it.
template <int R, bool ARGMIN, typename I, bool CAP = false>
__device__ __forceinline__ void vl_answer(const LevelsT<I>& lv, const typename IdxTraits<I>::Pair* __restrict__ qs,
                                          typename IdxTraits<I>::Count i, bool in_range, float* __restrict__ out_min,
                                          I* __restrict__ out_idx, uint32_t* __restrict__ err) {
    typename IdxTraits<I>::Pair Q;
    Q.x = 1u;
    Q.y = 0u;
    if (in_range) Q = ld_query(qs + i);
    float v;
    I idx;
    const bool valid = vl_compute<R, ARGMIN, I, CAP>(lv, Q, in_range, v, idx);
    vl_store<ARGMIN>(in_range, valid, v, idx, out_min != nullptr ? out_min + i : nullptr,
                     ARGMIN ? out_idx + i : nullptr, err);
}

}  // namespace rmq
