// rmq_query.cu — range-minimum / argmin queries over the hierarchy.
//
// Descent rule (reference CL, src/xxx.h:157-187): with r exclusive, while the
// current level is not the top and r - l > 2 rf, the partial chunks
// [l, ceil_rf(l)) and [floor_rf(r), r) of the current level are scanned and
// the query moves up with l = ceil_rf(l) / rf, r = floor_rf(r) / rf; the
// remaining [l, r) is scanned at the level where the loop stopped.  The pieces
// partition [l, r], so the minimum is the minimum over the pieces and the
// argmin is the lowest-position candidate among those equal to it.
//
// Two work distributions share that descent:
//   VL  one thread per query, 256-bit sector loads (reference alg 20,
//       kernel_hierarchical_vector_load, src/xxx.h:883-930, which uses float4);
//   CL  a tile of G lanes answers its G queries one after another, the lanes
//       sharing each query's sectors (reference alg 16, xxx_query,
//       src/xxx.h:124-200).
#include "rmq_internal.h"
#include "rmq_vl.cuh"

namespace rmq {

// CAP: the short-query variant (RMQ_VARIANT_VL_SHORT), which takes a short
// query's level-0 winner in phase 1 instead of reading it again in phase 2.
template <int R, bool ARGMIN, typename I, bool CAP = false>
__global__ void __launch_bounds__(256)
query_vl_kernel(LevelsT<I> lv, const typename IdxTraits<I>::Pair* __restrict__ qs, uint64_t q,
                float* __restrict__ out_min, I* __restrict__ out_idx, uint32_t* __restrict__ err) {
    // No early return: every lane takes part in the warp's long final scans.
    using C = typename IdxTraits<I>::Count;
    const C i = C(blockIdx.x) * blockDim.x + threadIdx.x;
    vl_answer<R, ARGMIN, I, CAP>(lv, qs, i, i < q, out_min, out_idx, err);
}

// ---------------------------------------------------------------------------
// CL: a tile of G lanes per query, queries of the tile one after another
//
// As in the reference's xxx_query (src/xxx.h:124-200), a tile loads its G
// queries (one per lane, coalesced) and answers them one after another; the
// lanes share the work of each query.  Here the unit of sharing is a 32-byte
// sector: at every level the sectors of the left piece, then of the right
// piece, are dealt to the lanes (rf = 32 with G = 8: one 256-bit load per lane
// per level), and the final piece's sectors likewise.  Each lane keeps the
// running minimum of its sectors and, for argmin, its first sector holding it
// under a position key (left pieces by ascending level, the final piece, right
// pieces by descending level; sectors ascending inside a piece).  The tile
// reduces the minimum, then the lowest key among lanes holding it; that lane
// re-reads its sector, takes the first entry equal to the minimum and, for a
// coarse level, loads the stored index.
// ---------------------------------------------------------------------------
struct LaneBest {
    float v;
    uint64_t key;   // (group << 32) | sector index inside the piece
    uint32_t s;     // sector start
    uint32_t meta;  // level | jlo << 8 | jhi << 16
};

constexpr uint64_t kKeyNone = ~uint64_t(0);
constexpr uint32_t kGroupFinal = 64u;  // left pieces use groups 0..19, right 128 + (19 - k)

template <bool ARGMIN>
__device__ __forceinline__ void cl_sector(const Levels& lv, uint32_t k, uint32_t s, uint32_t lo, uint32_t hi,
                                          uint64_t key, const L2Policies& pol, LaneBest& b) {
    const uint32_t jlo = s < lo ? lo - s : 0u;
    const uint32_t jhi = hi - s < 8u ? hi - s : 8u;
    float v[8];
    load_level_sector<uint32_t, false>(lv, k, s, pol, v);
    const float sm = sector_min(v, jlo, jhi);
    if (ARGMIN) {
        if (sm < b.v || (sm == b.v && key < b.key)) {
            b.v = sm;
            b.key = key;
            b.s = s;
            b.meta = k | (jlo << 8) | (jhi << 16);
        }
    } else {
        b.v = fminf(b.v, sm);
    }
}

// The tile's lanes scan the sectors of [alo, ahi) (group ga) followed by the
// sectors of [blo, bhi) (group gb) of level k; lane `lane` takes sectors
// lane, lane + G, ... of that combined list.
template <int G, bool ARGMIN>
__device__ __forceinline__ void cl_pair(const Levels& lv, uint32_t k, uint32_t alo, uint32_t ahi, uint32_t ga,
                                        uint32_t blo, uint32_t bhi, uint32_t gb, uint32_t lane,
                                        const L2Policies& pol, LaneBest& b) {
    const uint32_t a0 = alo & ~7u, b0 = blo & ~7u;
    const uint32_t na = ahi > alo ? ((ahi - a0 + 7u) >> 3) : 0u;
    const uint32_t nb = bhi > blo ? ((bhi - b0 + 7u) >> 3) : 0u;
    for (uint32_t j = lane; j < na + nb; j += G) {
        const bool in_a = j < na;
        const uint32_t idx = in_a ? j : j - na;
        const uint32_t s = (in_a ? a0 : b0) + 8u * idx;
        const uint64_t key = (uint64_t(in_a ? ga : gb) << 32) | idx;
        cl_sector<ARGMIN>(lv, k, s, in_a ? alo : blo, in_a ? ahi : bhi, key, pol, b);
    }
}

template <int R, int G, bool ARGMIN>
__device__ __forceinline__ void cl_query(const Levels& lv, uint32_t l, uint32_t r, uint32_t lane,
                                         const L2Policies& pol, LaneBest& b) {
    constexpr uint32_t RF = 1u << R;
    uint32_t k = 0;
    while (k + 1 < lv.num_levels && r - l > 2u * RF) {
        const uint32_t nl = (l + RF - 1) & ~(RF - 1);
        const uint32_t pr = r & ~(RF - 1);
        cl_pair<G, ARGMIN>(lv, k, l, nl, k, pr, r, 128u + (19u - k), lane, pol, b);
        l = nl >> R;
        r = pr >> R;
        ++k;
    }
    cl_pair<G, ARGMIN>(lv, k, l, r, kGroupFinal, 0u, 0u, 0u, lane, pol, b);
}

// Work distributions of the CL kernel (rmq_variant): the reference's alg 16
// (a tile answers its G queries one after another, each broadcast to the
// tile by shuffles, src/xxx.h:124-200) and its three ablations:
//   kClNoShuffle     alg 23 (src/xxx.h:302-369): every lane loads the query
//                    of the current turn itself, no ballot or broadcast;
//   kClQueryPerTile  alg 24 (src/xxx.h:470-528): one query per tile, q x G
//                    threads, no turns;
//   kClAtomic        alg 19 (src/xxx.h:631-686): as alg 23, but the lanes
//                    combine their candidates with atomic minima (here on a
//                    64-bit (value, position) key in shared memory) instead
//                    of a shuffle reduction.
// All four give the same results (the reference's alg 24 indexes its output
// by tile in a grid-stride loop and alg 23 reads past q; here every query is
// answered exactly once and nothing is read past q).
constexpr int kClShuffle = 0, kClNoShuffle = 1, kClQueryPerTile = 2, kClAtomic = 3;

// First entry equal to b.v inside lane candidate b's sector: its value bits
// and its level-0 position (for a coarse level, the stored index; only when
// WANT_POS).
template <bool WANT_POS>
__device__ __forceinline__ void cl_locate(const Levels& lv, const LaneBest& b, float m, const L2Policies& pol,
                                          float& val, uint32_t& pos, bool& pos_ok) {
    const uint32_t k = b.meta & 0xffu;
    const uint32_t jlo = (b.meta >> 8) & 0xffu;
    const uint32_t jhi = (b.meta >> 16) & 0xffu;
    float v[8];
    load_level_sector<uint32_t, false>(lv, k, b.s, pol, v);
    uint32_t jj = jlo;
#pragma unroll
    for (int t = 7; t >= 0; --t)
        if (uint32_t(t) >= jlo && uint32_t(t) < jhi && v[t] == m) jj = uint32_t(t);
    val = v[0];
#pragma unroll
    for (int t = 1; t < 8; ++t) val = (uint32_t(t) == jj) ? v[t] : val;
    const uint32_t e = b.s + jj;
    pos_ok = true;
    pos = e;
    if (WANT_POS && k > 0) {
#if RMQ_DEBUG_BOUNDS
        pos_ok = bounds_ok(lv.idx[k] != nullptr && e < lv.size[k]);
        if (!pos_ok) return;
#endif
        pos = ld_index(lv.idx[k] + e);
    }
}

template <int R, int G, bool ARGMIN, int MODE>
__global__ void __launch_bounds__(256)
query_cl_kernel(Levels lv, const uint2* __restrict__ qs, uint32_t q, float* __restrict__ out_min,
                uint32_t* __restrict__ out_idx, uint32_t* __restrict__ err) {
    const uint64_t gtid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint32_t tid = uint32_t(gtid);
    const uint32_t lane = threadIdx.x & (G - 1u);
    const uint32_t wl = threadIdx.x & 31u;
    const uint32_t mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl - lane));
    // The tile's queries: base .. base + G - 1 (one per turn), or the single
    // query gtid / G for kClQueryPerTile.
    const uint64_t base = MODE == kClQueryPerTile ? gtid / G : uint64_t(tid - lane);
    constexpr uint32_t kTurns = MODE == kClQueryPerTile ? 1u : uint32_t(G);
    __shared__ unsigned long long slot[MODE == kClAtomic ? 256 / G : 1];
    const L2Policies pol = make_policies();

    uint32_t vmask = 0;
    uint2 Q = make_uint2(1u, 0u);
    if constexpr (MODE == kClShuffle) {
        if (tid < q) Q = ld_query(qs + tid);
        const bool valid = tid < q && Q.x <= Q.y && Q.y < lv.size[0];
        if (tid < q && !valid) {
            if (out_min != nullptr) st_stream(out_min + tid, f_nan());
            if (ARGMIN) st_stream(out_idx + tid, kNoPos);
            if (err != nullptr) atomicAdd(err, 1u);
        }
        vmask = __ballot_sync(mask, valid) >> (wl - lane);  // the tile's valid queries
    }
    for (uint32_t j = 0; j < kTurns; ++j) {
        const uint64_t qi = base + j;                             // query of this turn
        const uint32_t owner = MODE == kClQueryPerTile ? 0u : j;  // the lane that stores its answer
        uint32_t l, r;
        if constexpr (MODE == kClShuffle) {
            if (((vmask >> j) & 1u) == 0u) continue;  // uniform across the tile
            l = __shfl_sync(mask, Q.x, j, G);
            r = __shfl_sync(mask, Q.y, j, G) + 1u;
        } else {
            if (qi >= q) break;  // uniform across the tile
            const uint2 Qj = ld_query(qs + qi);  // the same address on every lane
            if (!(Qj.x <= Qj.y && Qj.y < lv.size[0])) {
                if (lane == owner) {
                    if (out_min != nullptr) st_stream(out_min + qi, f_nan());
                    if (ARGMIN) st_stream(out_idx + qi, kNoPos);
                    if (err != nullptr) atomicAdd(err, 1u);
                }
                continue;
            }
            l = Qj.x;
            r = Qj.y + 1u;
        }
        if constexpr (MODE == kClAtomic) {
            // Every lane's candidate is its first entry equal to its minimum;
            // the tile keeps the least (value, position order) with atomicMin
            // on a 64-bit key and the lane holding it stores the answer.  The
            // value key puts -0.0 and +0.0 together, so ties among zeros go to
            // the first, whose bits are stored.
            LaneBest b{f_inf(), kKeyNone, 0u, 0u};
            cl_query<R, G, true>(lv, l, r, lane, pol, b);
            unsigned long long key = ~0ull;
            if (b.key != kKeyNone) {
                // position order inside the query: group (8 bits), sector of the piece (24 bits)
                const uint32_t order = (uint32_t(b.key >> 32) << 24) | uint32_t(b.key & 0xffffffu);
                key = (uint64_t(min_key(b.v)) << 32) | order;
            }
            if (lane == owner) slot[threadIdx.x / G] = ~0ull;
            __syncwarp(mask);
            if (key != ~0ull) atomicMin(&slot[threadIdx.x / G], key);
            __syncwarp(mask);
            const unsigned long long win = *reinterpret_cast<volatile unsigned long long*>(&slot[threadIdx.x / G]);
            if (win == ~0ull) {
                // no candidate compared at all: NaN inputs only (outside the
                // contract); the scan's answer is the first entry
                if (lane == owner) {
                    if (ARGMIN) st_stream(out_idx + qi, l);
                    if (out_min != nullptr) st_stream(out_min + qi, __ldg(lv.val[0] + l));
                }
            } else if (key == win) {
                float val;
                uint32_t pos;
                bool pos_ok;
                cl_locate<ARGMIN>(lv, b, b.v, pol, val, pos, pos_ok);
                if (ARGMIN && pos_ok) st_stream(out_idx + qi, pos);
                if (out_min != nullptr) st_stream(out_min + qi, val);
            }
            __syncwarp(mask);  // the slot is reused by the next turn
            continue;
        }
        LaneBest b{f_inf(), kKeyNone, 0u, 0u};
        cl_query<R, G, ARGMIN>(lv, l, r, lane, pol, b);
        float m = b.v;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) m = fminf(m, __shfl_xor_sync(mask, m, o, G));
        bool locate = ARGMIN;
        if (!ARGMIN) {
            // A +0.0 minimum means no -0.0 in the range (min.f32 returns -0.0
            // whenever one meets a zero): only -0.0 needs the first zero's bits.
            if (__float_as_uint(m) != 0x80000000u) {
                if (lane == owner) st_stream(out_min + qi, m);
                continue;
            }
            // A -0.0 minimum: locate the first zero for its bits.
            b = LaneBest{f_inf(), kKeyNone, 0u, 0u};
            cl_query<R, G, true>(lv, l, r, lane, pol, b);
            locate = true;
        }
        if (locate) {
            uint64_t key = (b.v == m) ? b.key : kKeyNone;
#pragma unroll
            for (int o = 1; o < G; o <<= 1) {
                const uint64_t other = __shfl_xor_sync(mask, key, o, G);
                key = other < key ? other : key;
            }
            if (key == kKeyNone) {
                // No entry compared equal to the minimum: NaN inputs only
                // (outside the contract); the scan's answer is the first entry.
                if (lane == owner) {
                    if (out_idx != nullptr) st_stream(out_idx + qi, l);
                    if (out_min != nullptr) st_stream(out_min + qi, __ldg(lv.val[0] + l));
                }
            } else if (b.key == key && b.v == m) {
                float val;
                uint32_t pos;
                bool pos_ok;
                cl_locate<ARGMIN>(lv, b, m, pol, val, pos, pos_ok);
                if (out_idx != nullptr && pos_ok) st_stream(out_idx + qi, pos);
                if (out_min != nullptr) st_stream(out_min + qi, val);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Brute-force checker: one warp per query, lanes stride the range, strict "<"
// per lane then a (value, index) combine — the semantics of kernel_rmq_basic /
// kernel_rmq_basic_idx (src/cuda_methods.cuh:4-44) with coalesced loads.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
bruteforce_kernel(const float* __restrict__ a, uint32_t n, const uint2* __restrict__ qs, uint32_t q,
                  float* __restrict__ out_min, uint32_t* __restrict__ out_idx) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = warp; i < q; i += nwarps) {
        const uint2 Q = qs[i];
        if (Q.x > Q.y || Q.y >= n) {
            if (lane == 0) {
                if (out_min) out_min[i] = f_nan();
                if (out_idx) out_idx[i] = kNoPos;
            }
            continue;
        }
        // Each lane scans its strided elements in ascending order; its first
        // element seeds its minimum (as A[l] seeds the reference scan) and
        // only a strictly smaller value replaces it.
        float best = f_inf();
        uint32_t bidx = kNoPos;
        for (uint64_t e = uint64_t(Q.x) + lane; e <= Q.y; e += 32) {
            const float v = a[e];
            if (bidx == kNoPos || v < best) {
                best = v;
                bidx = uint32_t(e);
            }
        }
        // Lane results combine by (value, index): equal values keep the lower index.
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, o);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, bidx, o);
            const bool take = oi != kNoPos &&
                              (bidx == kNoPos || ov < best || (ov == best && oi < bidx));
            if (take) {
                best = ov;
                bidx = oi;
            }
        }
        if (lane == 0) {
            if (out_min) out_min[i] = best;
            if (out_idx) out_idx[i] = bidx;
        }
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

template <typename K, typename... Args>
static cudaError_t launch_with_window(K kernel, uint32_t grid, uint32_t block, const QueryArgs& a,
                                      cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    if (a.persist_base != nullptr && a.persist_bytes > 0) {
        attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[0].val.accessPolicyWindow.base_ptr = const_cast<void*>(a.persist_base);
        attr[0].val.accessPolicyWindow.num_bytes = a.persist_bytes;
        attr[0].val.accessPolicyWindow.hitRatio = a.persist_hit_ratio;
        attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    } else {
        cfg.attrs = nullptr;
        cfg.numAttrs = 0;
    }
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Query kernels run in 128-thread blocks.  A block keeps its register slots
// until its last query ends, so smaller blocks give finished warps' slots
// back sooner; at the same registers per thread the SM holds as many warps
// (VL 32-bit: 12 blocks of 128 = 6 of 256).  n = q = 2^26, lognormal
// lengths, vs 256-thread blocks: VL +0.5 % (three-way mixture +1.7 %,
// uniform lengths -0.5 %), VL with 64-bit positions +6.3 % (55 registers:
// 9 blocks of 128 hold 36 warps, 4 of 256 held 32), CL (rf 8, 2 lanes)
// +2.1 %.  64-thread blocks: within 1 % of these, uniform lengths -1 %.
constexpr uint32_t kQueryBlock = 128;

template <int R, int MODE>
static cudaError_t launch_cl(const QueryArgs& a, cudaStream_t s, uint32_t grid, uint32_t q32, bool argmin) {
#define RMQ_CL(G)                                                                                                \
    return argmin ? launch_with_window(query_cl_kernel<R, G, true, MODE>, grid, kQueryBlock, a, s, a.lv, a.qs,  \
                                         q32, a.out_min, a.out_idx, a.err)                                        \
                  : launch_with_window(query_cl_kernel<R, G, false, MODE>, grid, kQueryBlock, a, s, a.lv, a.qs, \
                                         q32, a.out_min, static_cast<uint32_t*>(nullptr), a.err)
    switch (a.lanes) {
        case 2: RMQ_CL(2);
        case 4: RMQ_CL(4);
        case 8: RMQ_CL(8);
        case 16: RMQ_CL(16);
        case 32: RMQ_CL(32);
        default: return cudaErrorInvalidValue;
    }
#undef RMQ_CL
}

template <int R>
static cudaError_t launch_query_r(const QueryArgs& a, cudaStream_t s) {
    const bool argmin = a.out_idx != nullptr || a.out_idx64 != nullptr;
    const uint32_t grid = uint32_t((a.q + kQueryBlock - 1u) / kQueryBlock);
    if (a.wide) {
        // 64-bit positions: the VL kernel only (the short-query variant is VL here).
        if (a.variant != 2 && a.variant != 6) return cudaErrorNotSupported;
        const ulonglong2* qs = reinterpret_cast<const ulonglong2*>(a.qs64);
        return argmin ? launch_with_window(query_vl_kernel<R, true, uint64_t>, grid, kQueryBlock, a, s, a.lv64,
                                             qs, a.q, a.out_min, a.out_idx64, a.err)
                      : launch_with_window(query_vl_kernel<R, false, uint64_t>, grid, kQueryBlock, a, s, a.lv64,
                                             qs, a.q, a.out_min, static_cast<uint64_t*>(nullptr), a.err);
    }
    if (a.variant == 6 && R == 3) {
        return argmin ? launch_with_window(query_vl_kernel<3, true, uint32_t, true>, grid, kQueryBlock, a, s, a.lv,
                                           a.qs, a.q, a.out_min, a.out_idx, a.err)
                      : launch_with_window(query_vl_kernel<3, false, uint32_t, true>, grid, kQueryBlock, a, s, a.lv,
                                           a.qs, a.q, a.out_min, static_cast<uint32_t*>(nullptr), a.err);
    }
    if (a.variant == 2 || a.variant == 6) {
        return argmin ? launch_with_window(query_vl_kernel<R, true, uint32_t>, grid, kQueryBlock, a, s, a.lv,
                                             a.qs, a.q, a.out_min, a.out_idx, a.err)
                      : launch_with_window(query_vl_kernel<R, false, uint32_t>, grid, kQueryBlock, a, s, a.lv,
                                             a.qs, a.q, a.out_min, static_cast<uint32_t*>(nullptr), a.err);
    }
    const uint32_t q32 = uint32_t(a.q);
    switch (a.variant) {
        case 1: return launch_cl<R, kClShuffle>(a, s, grid, q32, argmin);
        case 3: return launch_cl<R, kClNoShuffle>(a, s, grid, q32, argmin);
        case 4: {
            // one tile of `lanes` threads per query
            const uint64_t threads = a.q * uint64_t(a.lanes);
            const uint64_t g = (threads + kQueryBlock - 1u) / kQueryBlock;
            if (g > 0x7FFFFFFFull) return cudaErrorInvalidConfiguration;
            return launch_cl<R, kClQueryPerTile>(a, s, uint32_t(g), q32, argmin);
        }
        case 5: return launch_cl<R, kClAtomic>(a, s, grid, q32, argmin);
        default: return cudaErrorInvalidValue;
    }
}

#if RMQ_DEBUG_BOUNDS
RMQ_BOUNDS_COUNTER_READER(bounds_bad_query)
#endif

cudaError_t launch_query(const QueryArgs& a, cudaStream_t s) {
    if (a.q == 0) return cudaSuccess;
    switch (a.rf_log) {
        case 3: return launch_query_r<3>(a, s);
        case 4: return launch_query_r<4>(a, s);
        case 5: return launch_query_r<5>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_bruteforce(const float* vals, uint32_t n, const uint2* qs, uint32_t q,
                              float* out_min, uint32_t* out_idx, cudaStream_t s) {
    if (q == 0) return cudaSuccess;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t warps_needed = q;
    uint64_t grid = (warps_needed * 32 + 255) / 256;
    const uint64_t cap = uint64_t(sms) * 8;  // 8 blocks of 8 warps per SM
    if (grid > cap) grid = cap;
    bruteforce_kernel<<<uint32_t(grid), 256, 0, s>>>(vals, n, qs, q, out_min, out_idx);
    return cudaGetLastError();
}

}  // namespace rmq
