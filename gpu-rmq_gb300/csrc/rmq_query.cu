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
//   CL  a tile of G lanes per query (reference alg 16, xxx_query,
//       src/xxx.h:124-200, where a tile answers its queries one after the
//       other); here the lanes split the query's pieces by level so all
//       loads of one query are in flight together.
#include "rmq_internal.h"
#include "rmq_vl.cuh"

namespace rmq {

template <int R, bool ARGMIN>
__global__ void __launch_bounds__(256)
query_vl_kernel(Levels lv, const uint2* __restrict__ qs, uint32_t q, float* __restrict__ out_min,
                uint32_t* __restrict__ out_idx, uint32_t* __restrict__ err) {
    // No early return: every lane takes part in the warp's long final scans.
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    vl_answer<R, ARGMIN>(lv, qs, i, i < q, out_min, out_idx, err);
}

// ---------------------------------------------------------------------------
// CL: a tile of G lanes per query, level-parallel
//
// Lane j of the tile owns the pieces of side (j & 1) (0 = left, 1 = right) at
// levels j/2, j/2 + G/2, ... and the sectors j, j + G, ... of the final piece.
// Every lane derives the descent (pure index arithmetic, no loads), then all
// of its loads are issued together, so a query costs one memory round trip
// for all levels instead of one per level.  The tile combines lane results by
// (value, order key), where the key orders pieces by position: left pieces by
// ascending level, then the final piece's sectors, then right pieces by
// descending level; the lowest key among equal values is the first
// occurrence.  The winning lane re-reads its sector, takes its first entry
// equal to the minimum and, for a coarse level, loads the stored index.
// ---------------------------------------------------------------------------
constexpr uint32_t kKeyNone = 0xFFFFFFFFu;
constexpr uint32_t kKeyFinal = 64u;  // keys of final sectors start here (levels < 20)

struct LaneBest {
    float v;
    uint32_t key;
    uint32_t s;     // sector start
    uint32_t meta;  // level | jlo << 8 | jhi << 16
};

template <bool ARGMIN>
__device__ __forceinline__ void lane_take(LaneBest& b, float sm, uint32_t key, uint32_t s, uint32_t meta) {
    if (ARGMIN) {
        if (sm < b.v || (sm == b.v && key < b.key)) {
            b.v = sm;
            b.key = key;
            b.s = s;
            b.meta = meta;
        }
    } else {
        b.v = fminf(b.v, sm);
    }
}

// One sector of level k restricted to [lo, hi).
template <bool ARGMIN>
__device__ __forceinline__ void cl_sector(const Levels& lv, uint32_t k, uint32_t s, uint32_t lo, uint32_t hi,
                                          uint32_t key, const L2Policies& pol, LaneBest& b) {
    const uint32_t jlo = s < lo ? lo - s : 0u;
    const uint32_t jhi = hi - s < 8u ? hi - s : 8u;
    float v[8];
    load_level_sector(lv, k, s, pol, v);
    lane_take<ARGMIN>(b, sector_min(v, jlo, jhi), key, s, k | (jlo << 8) | (jhi << 16));
}

template <int R, int G, bool ARGMIN>
__device__ __forceinline__ void cl_lane_work(const Levels& lv, uint32_t l, uint32_t r, uint32_t lane,
                                             const L2Policies& pol, LaneBest& b) {
    constexpr uint32_t RF = 1u << R;
    constexpr uint32_t PAIRS = G / 2u;
    const uint32_t my_level = lane >> 1;
    const bool right = (lane & 1u) != 0u;
    // Descent: stop level s and final piece [l, r) at level s; this lane's
    // boundary pieces are recorded as they are passed (at most
    // ceil(19 / PAIRS) of them; pieces are processed after the loop).
    constexpr uint32_t kMaxPieces = (19u + PAIRS - 1u) / PAIRS;
    uint32_t plo[kMaxPieces], phi[kMaxPieces];
    uint32_t np = 0;
    uint32_t k = 0;
    while (k + 1 < lv.num_levels && r - l > 2u * RF) {
        const uint32_t nl = (l + RF - 1) & ~(RF - 1);
        const uint32_t pr = r & ~(RF - 1);
        if (k % PAIRS == my_level) {
#pragma unroll
            for (uint32_t i = 0; i < kMaxPieces; ++i) {  // constant indices keep plo/phi in registers
                if (np == i) {
                    plo[i] = right ? pr : l;
                    phi[i] = right ? r : nl;
                }
            }
            ++np;
        }
        l = nl >> R;
        r = pr >> R;
        ++k;
    }
    // Final piece sectors: all independent of the pieces, issued alongside.
    const uint32_t f0 = l & ~7u;
    for (uint32_t s = f0 + 8u * lane; s < r; s += 8u * G) {
        cl_sector<ARGMIN>(lv, k, s, l, r, kKeyFinal + ((s - f0) >> 3), pol, b);
    }
#pragma unroll
    for (uint32_t i = 0; i < kMaxPieces; ++i) {
        if (i < np && phi[i] > plo[i]) {
            const uint32_t lvl = my_level + i * PAIRS;
            const uint32_t key = right ? (kKeyNone - 1u - lvl) : lvl;
            for (uint32_t s = plo[i] & ~7u; s < phi[i]; s += 8u)
                cl_sector<ARGMIN>(lv, lvl, s, plo[i], phi[i], key, pol, b);
        }
    }
}

template <int R, int G, bool ARGMIN>
__global__ void __launch_bounds__(256)
query_cl_kernel(Levels lv, const uint2* __restrict__ qs, uint32_t q, float* __restrict__ out_min,
                uint32_t* __restrict__ out_idx, uint32_t* __restrict__ err) {
    const uint32_t lane = threadIdx.x & (G - 1u);
    const uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint32_t wl = threadIdx.x & 31u;
    const uint32_t mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl - lane));
    if (qi >= q) return;  // uniform across the tile
    const uint2 Q = ld_query(qs + qi);
    if (Q.x > Q.y || Q.y >= lv.size[0]) {
        if (lane == 0) {
            if (out_min != nullptr) st_stream(out_min + qi, f_nan());
            if (ARGMIN) st_stream(out_idx + qi, kNoPos);
            if (err != nullptr) atomicAdd(err, 1u);
        }
        return;
    }
    const L2Policies pol = make_policies();
    const uint32_t l = Q.x, r = Q.y + 1;
    LaneBest b{f_inf(), kKeyNone, 0u, 0u};
    bool need_locate = ARGMIN;
    cl_lane_work<R, G, ARGMIN>(lv, l, r, lane, pol, b);
    float m = b.v;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) m = fminf(m, __shfl_xor_sync(mask, m, o, G));
    if (!ARGMIN) {
        if (m != 0.0f) {
            if (lane == 0) st_stream(out_min + qi, m);
            return;
        }
        // A zero minimum may be -0.0 or +0.0: locate the first one for its bits.
        b = LaneBest{f_inf(), kKeyNone, 0u, 0u};
        cl_lane_work<R, G, true>(lv, l, r, lane, pol, b);
        need_locate = true;
    }
    if (need_locate) {
        // The winner: lowest key among the lanes holding the minimum.
        uint32_t key = (b.v == m) ? b.key : kKeyNone;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) key = min(key, __shfl_xor_sync(mask, key, o, G));
        if (key == kKeyNone) {
            // No entry compared equal to the minimum: NaN inputs only (outside
            // the contract); the scan's answer is the first entry.
            if (lane == 0) {
                if (out_idx != nullptr) st_stream(out_idx + qi, l);
                if (out_min != nullptr) st_stream(out_min + qi, __ldg(lv.val[0] + l));
            }
            return;
        }
        if (b.key == key && b.v == m) {
            const uint32_t k = b.meta & 0xffu;
            const uint32_t jlo = (b.meta >> 8) & 0xffu;
            const uint32_t jhi = (b.meta >> 16) & 0xffu;
            float v[8];
            load_level_sector(lv, k, b.s, pol, v);
            uint32_t j = jlo;
#pragma unroll
            for (int jj = 7; jj >= 0; --jj)
                if (uint32_t(jj) >= jlo && uint32_t(jj) < jhi && v[jj] == m) j = uint32_t(jj);
            float val = v[0];
#pragma unroll
            for (int jj = 1; jj < 8; ++jj) val = (uint32_t(jj) == j) ? v[jj] : val;
            const uint32_t e = b.s + j;
            if (out_idx != nullptr) st_stream(out_idx + qi, k == 0 ? e : ld_index(lv.idx[k] + e));
            if (out_min != nullptr) st_stream(out_min + qi, val);
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

template <typename K>
static cudaError_t launch_with_window(K kernel, uint32_t grid, const QueryArgs& a, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
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
    return cudaLaunchKernelEx(&cfg, kernel, a.lv, a.qs, a.q, a.out_min, a.out_idx, a.err);
}

template <int R>
static cudaError_t launch_query_r(const QueryArgs& a, cudaStream_t s) {
    const bool argmin = a.out_idx != nullptr;
    if (a.variant == 2) {
        const uint32_t grid = (a.q + 255u) / 256u;
        return argmin ? launch_with_window(query_vl_kernel<R, true>, grid, a, s)
                      : launch_with_window(query_vl_kernel<R, false>, grid, a, s);
    }
    const uint32_t grid = uint32_t((uint64_t(a.q) * uint64_t(a.lanes) + 255u) / 256u);
    switch (a.lanes) {
        case 4:
            return argmin ? launch_with_window(query_cl_kernel<R, 4, true>, grid, a, s)
                          : launch_with_window(query_cl_kernel<R, 4, false>, grid, a, s);
        case 8:
            return argmin ? launch_with_window(query_cl_kernel<R, 8, true>, grid, a, s)
                          : launch_with_window(query_cl_kernel<R, 8, false>, grid, a, s);
        case 16:
            return argmin ? launch_with_window(query_cl_kernel<R, 16, true>, grid, a, s)
                          : launch_with_window(query_cl_kernel<R, 16, false>, grid, a, s);
        case 32:
            return argmin ? launch_with_window(query_cl_kernel<R, 32, true>, grid, a, s)
                          : launch_with_window(query_cl_kernel<R, 32, false>, grid, a, s);
        default:
            return cudaErrorInvalidValue;
    }
}

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
