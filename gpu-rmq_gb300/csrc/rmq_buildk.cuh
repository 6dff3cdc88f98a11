// rmq_buildk.cuh — build device functions shared by the single-array build
// (rmq_build.cu) and the batched build (rmq_batch.cu).
#pragma once

#include "rmq_common.cuh"

namespace rmq {

constexpr uint32_t kTile = 8192;
constexpr uint32_t kTileSectors = kTile / 8;
constexpr uint32_t kFusedThreads = 256;
constexpr uint32_t kTailMaxEntries = 16384;  // largest level the tail CTA reads

// P: position type (uint32_t, or uint64_t for arrays beyond 2^32 entries).
template <typename P>
struct LevelOutT {
    float* val[kMaxLevels];
    P* idx[kMaxLevels];  // null entries when argmin arrays are not built
    P size[kMaxLevels];
};
using LevelOut = LevelOutT<uint32_t>;

// First-occurrence minimum over candidates visited in ascending position;
// p == none marks an absent candidate.
template <typename P>
struct VPT {
    float v;
    P p;
};

template <typename P>
__device__ __forceinline__ void vp_take(VPT<P>& cur, float v, P p) {
    constexpr P kNone = IdxTraits<P>::none;
    if (p != kNone && (cur.p == kNone || v < cur.v)) {
        cur.v = v;
        cur.p = p;
    }
}

template <int R>
__host__ __device__ constexpr uint32_t fused_depth() {
    return 13u / uint32_t(R);  // largest m with rf^m <= kTile = 2^13
}

// One CTA of kFusedThreads threads builds levels 1..depth of `tile` (entries
// [tile * kTile, (tile + 1) * kTile) of level 0); sv / sp are kTileSectors
// entries of shared memory.
template <int R, typename P>
__device__ __forceinline__ void fused_tile(const float* __restrict__ a, P n, const LevelOutT<P>& out,
                                           uint32_t depth, uint64_t tile, float* sv, P* sp) {
    using VP = VPT<P>;
    constexpr P kNone = IdxTraits<P>::none;
    constexpr uint32_t RF = 1u << R;
    constexpr uint32_t SPB = RF / 8u;  // sectors per level-1 block
    const uint32_t tid = threadIdx.x;
    const uint64_t base = uint64_t(tile) * kTile;
    const uint64_t pol = policy_evict_first();

    // Stage 0: per-sector first minimum.  A whole tile inside the array (all
    // but the last) loads its four sectors per thread at once, takes each
    // sector's minimum with three 3-input min.f32 and then the first entry
    // equal to it (its own bits, so a zero keeps the sign of its first
    // occurrence); the last tile goes entry by entry.
    constexpr uint32_t kSecPer = kTileSectors / kFusedThreads;
    if (base + kTile <= uint64_t(n)) {
        float v[kSecPer][8];
#pragma unroll
        for (uint32_t i = 0; i < kSecPer; ++i) ld_sector_policy(a + base + 8u * (tid + kFusedThreads * i), v[i], pol);
#pragma unroll
        for (uint32_t i = 0; i < kSecPer; ++i) {
            const uint32_t sec = tid + kFusedThreads * i;
            const float m = fmin3(fmin3(v[i][0], v[i][1], v[i][2]), fmin3(v[i][3], v[i][4], v[i][5]),
                                  fminf(v[i][6], v[i][7]));
            uint32_t j = 7;
            float mv = v[i][7];
#pragma unroll
            for (int jj = 6; jj >= 0; --jj) {
                if (v[i][jj] == m) {
                    j = uint32_t(jj);
                    mv = v[i][jj];
                }
            }
            sv[sec] = mv;
            sp[sec] = P(base + 8u * sec + j);
        }
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kSecPer; ++i) {
            const uint32_t sec = tid + kFusedThreads * i;
            const uint64_t s = base + 8u * sec;
            VP c{f_inf(), kNone};
            if (s < n) {
                float v[8];
                if (s + 8u <= n) {
                    ld_sector_policy(a + s, v, pol);
                } else {
#pragma unroll
                    for (int j = 0; j < 8; ++j) v[j] = (s + j < n) ? a[s + j] : f_inf();
                }
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (s + j < n) vp_take(c, v[j], P(s + j));
            }
            sv[sec] = c.v;
            sp[sec] = c.p;
        }
    }
    __syncthreads();

    // Levels 1..depth: level k has kTile / rf^k entries in the tile; an entry
    // combines rf children of level k-1 (SPB sectors for k = 1).
    uint32_t children = kTileSectors;  // entries of the previous stage held in smem
    for (uint32_t k = 1; k <= depth; ++k) {
        const uint32_t fan = (k == 1) ? SPB : RF;
        const uint32_t cnt = children / fan;
        constexpr uint32_t kMaxPer = kTileSectors / kFusedThreads;  // <= 4 entries per thread
        VP res[kMaxPer];
#pragma unroll
        for (uint32_t i = 0; i < kMaxPer; ++i) {
            const uint32_t e = tid + kFusedThreads * i;
            res[i] = VP{f_inf(), kNone};
            if (e < cnt) {
                for (uint32_t j = 0; j < fan; ++j) vp_take(res[i], sv[e * fan + j], sp[e * fan + j]);
            }
        }
        __syncthreads();
        const uint64_t gbase = uint64_t(tile) * cnt;
#pragma unroll
        for (uint32_t i = 0; i < kMaxPer; ++i) {
            const uint32_t e = tid + kFusedThreads * i;
            if (e < cnt) {
                sv[e] = res[i].v;
                sp[e] = res[i].p;
                const uint64_t g = gbase + e;
                if (g < out.size[k]) {
                    out.val[k][g] = res[i].v;
                    if (out.idx[k] != nullptr) out.idx[k][g] = res[i].p;
                }
            }
        }
        __syncthreads();
        children = cnt;
    }
}

// Levels above the fused tiles, built inside the fused kernel.  Entry g of
// level k depends on the tiles (k = depth + 1) or entries of level k - 1
// (k > depth + 1) below it; each of those, when done, adds one arrival to
// g's counter, and the last arrival computes g (one warp: a lane per child,
// first-occurrence reduction) and passes on to g's parent.  No CTA waits:
// whoever completes a group does its work.  Every counter is reset by its
// last arrival, so the counters are all zero again after the build.
struct TailPlan {
    uint32_t depth;     // top level built inside the tiles
    uint32_t top;       // top level of the hierarchy (> depth when there is a tail)
    uint32_t per_tile;  // level-`depth` entries per tile
    unsigned* counters;
    uint64_t coff[kMaxLevels];  // first counter of level k, depth < k <= top
};

template <typename P>
__device__ __forceinline__ P ldcg_pos(const P* p);
template <>
__device__ __forceinline__ uint32_t ldcg_pos(const uint32_t* p) { return __ldcg(p); }
template <>
__device__ __forceinline__ uint64_t ldcg_pos(const uint64_t* p) {
    return __ldcg(reinterpret_cast<const unsigned long long*>(p));
}

template <int R, typename P>
__device__ __forceinline__ void tail_upward(const LevelOutT<P>& out, const TailPlan& tp, uint64_t tile) {
    constexpr uint32_t RF = 1u << R;
    constexpr P kNone = IdxTraits<P>::none;
    __shared__ unsigned s_go;
    __threadfence();  // this tile's level entries before its arrival
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint64_t g = (tile * tp.per_tile) >> R;
        const uint64_t lo = g << R;
        const uint64_t hi = lo + RF < uint64_t(out.size[tp.depth]) ? lo + RF : uint64_t(out.size[tp.depth]);
        const unsigned expect = unsigned((hi - 1) / tp.per_tile - lo / tp.per_tile + 1);
        unsigned* c = tp.counters + tp.coff[tp.depth + 1] + g;
        const unsigned last = atomicAdd(c, 1u) + 1u == expect;
        if (last) *c = 0u;
        s_go = last;
    }
    __syncthreads();
    if (s_go == 0u || threadIdx.x >= 32) return;
    const uint32_t lane = threadIdx.x;
    uint64_t g = (tile * tp.per_tile) >> R;
    for (uint32_t k = tp.depth + 1;; ++k) {
        __threadfence();  // the children's writers fenced before arriving
        const uint64_t child = (g << R) + lane;
        float v = f_inf();
        P p = kNone;
        if (lane < RF && child < uint64_t(out.size[k - 1])) {
            v = __ldcg(out.val[k - 1] + child);
            p = out.idx[k - 1] != nullptr ? ldcg_pos(out.idx[k - 1] + child) : P(child);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, v, o);
            const P op = __shfl_xor_sync(0xffffffffu, p, o);
            if (op != kNone && (p == kNone || ov < v || (ov == v && op < p))) {
                v = ov;
                p = op;
            }
        }
        unsigned go = 0u;
        if (lane == 0) {
            out.val[k][g] = v;
            if (out.idx[k] != nullptr) out.idx[k][g] = p;
            if (k < tp.top) {
                __threadfence();
                const uint64_t gg = g >> R;
                const uint64_t left = uint64_t(out.size[k]) - (gg << R);
                const unsigned expect = unsigned(left < RF ? left : RF);
                unsigned* c = tp.counters + tp.coff[k + 1] + gg;
                go = atomicAdd(c, 1u) + 1u == expect;
                if (go) *c = 0u;
            }
        }
        if (k == tp.top || __shfl_sync(0xffffffffu, go, 0) == 0u) return;
        g >>= R;
    }
}

// Single CTA: builds levels from+1 .. last from level `from` (already built),
// level after level, with a block barrier between levels (global writes of
// the block are visible to it after __syncthreads).
template <int R, typename P>
__device__ __forceinline__ void tail_levels(const LevelOutT<P>& out, uint32_t from, uint32_t last) {
    constexpr uint32_t RF = 1u << R;
    for (uint32_t k = from; k < last; ++k) {
        const float* src = out.val[k];
        const P* src_idx = out.idx[k];
        const P src_size = out.size[k];
        for (P e = threadIdx.x; e < out.size[k + 1]; e += blockDim.x) {
            VPT<P> c{f_inf(), IdxTraits<P>::none};
            for (uint32_t j = 0; j < RF; ++j) {
                const P ch = e * RF + j;
                if (ch < src_size) vp_take(c, src[ch], src_idx != nullptr ? src_idx[ch] : ch);
            }
            out.val[k + 1][e] = c.v;
            if (out.idx[k + 1] != nullptr) out.idx[k + 1][e] = c.p;
        }
        __syncthreads();
    }
}

}  // namespace rmq
