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
//   CL  a tile of G lanes per query with 128-bit loads; the tile's G queries
//       are loaded coalesced, one per lane, broadcast by shuffle and answered
//       one after the other (reference alg 16, xxx_query, src/xxx.h:124-200).
#include "rmq_internal.h"

namespace rmq {

// ---------------------------------------------------------------------------
// VL: thread per query
// ---------------------------------------------------------------------------

// Loads the sector starting at s of level k.  Level 0 is the caller's array,
// which is not padded: a sector that crosses its end is read element-wise.
__device__ __forceinline__ void load_level_sector(const float* base, uint32_t size, uint32_t k,
                                                  uint32_t s, float (&v)[8]) {
    if (k > 0 || s + 8u <= size) {
        ld_sector(base + s, v);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (s + j < size) ? base[s + j] : f_inf();
    }
}

// Candidate scan of [lo, hi) at level k (thread-private).
__device__ __forceinline__ void vl_scan_cand(const Levels& lv, uint32_t k, uint32_t shift,
                                             uint32_t lo, uint32_t hi, Cand& c) {
    const float* base = lv.val[k];
    const uint32_t size = lv.size[k];
    for (uint32_t s = lo & ~7u; s < hi; s += 8u) {
        float v[8];
        load_level_sector(base, size, k, s, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t e = s + j;
            if (e >= lo && e < hi) cand_update(c, v[j], e << shift, k);
        }
    }
}

// Minimum-only scan of [lo, hi) at level k.
__device__ __forceinline__ float vl_scan_min(const Levels& lv, uint32_t k, uint32_t lo, uint32_t hi,
                                             float m) {
    const float* base = lv.val[k];
    const uint32_t size = lv.size[k];
    for (uint32_t s = lo & ~7u; s < hi; s += 8u) {
        float v[8];
        load_level_sector(base, size, k, s, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t e = s + j;
            m = fminf(m, (e >= lo && e < hi) ? v[j] : f_inf());
        }
    }
    return m;
}

template <int R>
__device__ __forceinline__ Cand vl_descend_cand(const Levels& lv, uint32_t l, uint32_t r) {
    constexpr uint32_t RF = 1u << R;
    Cand c;
    cand_init(c);
    uint32_t k = 0;
    while (k + 1 < lv.num_levels && r - l > 2u * RF) {
        const uint32_t nl = (l + RF - 1) & ~(RF - 1);
        const uint32_t pr = r & ~(RF - 1);
        const uint32_t shift = k * R;
        if (nl > l) vl_scan_cand(lv, k, shift, l, nl, c);
        if (r > pr) vl_scan_cand(lv, k, shift, pr, r, c);
        l = nl >> R;
        r = pr >> R;
        ++k;
    }
    vl_scan_cand(lv, k, k * R, l, r, c);
    return c;
}

template <int R>
__device__ __forceinline__ float vl_descend_min(const Levels& lv, uint32_t l, uint32_t r) {
    constexpr uint32_t RF = 1u << R;
    float m = f_inf();
    uint32_t k = 0;
    while (k + 1 < lv.num_levels && r - l > 2u * RF) {
        const uint32_t nl = (l + RF - 1) & ~(RF - 1);
        const uint32_t pr = r & ~(RF - 1);
        if (nl > l) m = vl_scan_min(lv, k, l, nl, m);
        if (r > pr) m = vl_scan_min(lv, k, pr, r, m);
        l = nl >> R;
        r = pr >> R;
        ++k;
    }
    return vl_scan_min(lv, k, l, r, m);
}

// Level-0 index of a candidate (one dependent load for coarse-level winners).
template <int R>
__device__ __forceinline__ uint32_t cand_index(const Levels& lv, const Cand& c, uint32_t l) {
    if (c.pos == kNoPos) return l;  // only reachable with NaN inputs (out of contract)
    if (c.lvl == 0) return c.pos;
    return __ldg(lv.idx[c.lvl] + (c.pos >> (c.lvl * R)));
}

template <int R, bool ARGMIN>
__global__ void __launch_bounds__(256)
query_vl_kernel(Levels lv, const uint2* __restrict__ qs, uint32_t q, float* __restrict__ out_min,
                uint32_t* __restrict__ out_idx, uint32_t* __restrict__ err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q) return;
    const uint2 Q = ld_query(qs + i);
    if (Q.x > Q.y || Q.y >= lv.size[0]) {
        if (out_min != nullptr) st_stream(out_min + i, f_nan());
        if (ARGMIN) st_stream(out_idx + i, kNoPos);
        if (err != nullptr) atomicAdd(err, 1u);
        return;
    }
    const uint32_t l = Q.x, r = Q.y + 1;
    if (ARGMIN) {
        const Cand c = vl_descend_cand<R>(lv, l, r);
        st_stream(out_idx + i, cand_index<R>(lv, c, l));
        if (out_min != nullptr) st_stream(out_min + i, c.v);
    } else {
        float m = vl_descend_min<R>(lv, l, r);
        // A zero minimum may be -0.0 or +0.0; the reference returns the bits of
        // the first occurrence, so redo the query with positions in that case.
        if (m == 0.0f) m = vl_descend_cand<R>(lv, l, r).v;
        st_stream(out_min + i, m);
    }
}

// ---------------------------------------------------------------------------
// CL: tile of G lanes per query
// ---------------------------------------------------------------------------

__device__ __forceinline__ void load_level_quad(const float* base, uint32_t size, uint32_t k,
                                                uint32_t s, float (&v)[4]) {
    if (k > 0 || s + 4u <= size) {
        ld_quad(base + s, v);
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = (s + j < size) ? base[s + j] : f_inf();
    }
}

// The tile scans two ranges of level k (either may be empty) as one list of
// aligned quads: quads of A first, then quads of B; lane `lane` takes quads
// lane, lane + G, ...
template <int G, bool CAND>
__device__ __forceinline__ void cl_scan_pair(const Levels& lv, uint32_t k, uint32_t shift,
                                             uint32_t alo, uint32_t ahi, uint32_t blo, uint32_t bhi,
                                             uint32_t lane, Cand& c, float& m) {
    const float* base = lv.val[k];
    const uint32_t size = lv.size[k];
    const uint32_t a0 = alo & ~3u;
    const uint32_t na = ahi > alo ? ((ahi - a0 + 3u) >> 2) : 0u;
    const uint32_t b0 = blo & ~3u;
    const uint32_t nb = bhi > blo ? ((bhi - b0 + 3u) >> 2) : 0u;
    const uint32_t total = na + nb;
    for (uint32_t j = lane; j < total; j += G) {
        const bool in_a = j < na;
        const uint32_t s = in_a ? a0 + 4u * j : b0 + 4u * (j - na);
        const uint32_t lo = in_a ? alo : blo;
        const uint32_t hi = in_a ? ahi : bhi;
        float v[4];
        load_level_quad(base, size, k, s, v);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const uint32_t e = s + t;
            const bool inside = e >= lo && e < hi;
            if (CAND) {
                if (inside) cand_update(c, v[t], e << shift, k);
            } else {
                m = fminf(m, inside ? v[t] : f_inf());
            }
        }
    }
}

template <int R, int G, bool CAND>
__device__ __forceinline__ void cl_descend(const Levels& lv, uint32_t l, uint32_t r, uint32_t lane,
                                           Cand& c, float& m) {
    constexpr uint32_t RF = 1u << R;
    uint32_t k = 0;
    while (k + 1 < lv.num_levels && r - l > 2u * RF) {
        const uint32_t nl = (l + RF - 1) & ~(RF - 1);
        const uint32_t pr = r & ~(RF - 1);
        cl_scan_pair<G, CAND>(lv, k, k * R, l, nl, pr, r, lane, c, m);
        l = nl >> R;
        r = pr >> R;
        ++k;
    }
    cl_scan_pair<G, CAND>(lv, k, k * R, l, r, 0u, 0u, lane, c, m);
}

template <int G>
__device__ __forceinline__ void cl_reduce_cand(Cand& c, uint32_t mask) {
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
        const float ov = __shfl_xor_sync(mask, c.v, o, G);
        const uint32_t op = __shfl_xor_sync(mask, c.pos, o, G);
        const uint32_t ol = __shfl_xor_sync(mask, c.lvl, o, G);
        cand_update(c, ov, op, ol);
    }
}

template <int G>
__device__ __forceinline__ float cl_reduce_min(float m, uint32_t mask) {
#pragma unroll
    for (int o = 1; o < G; o <<= 1) m = fminf(m, __shfl_xor_sync(mask, m, o, G));
    return m;
}

template <int R, int G, bool ARGMIN>
__global__ void __launch_bounds__(256)
query_cl_kernel(Levels lv, const uint2* __restrict__ qs, uint32_t q, float* __restrict__ out_min,
                uint32_t* __restrict__ out_idx, uint32_t* __restrict__ err) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & (G - 1);
    const uint32_t wl = threadIdx.x & 31u;
    const uint32_t mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl - lane));
    const uint32_t n = lv.size[0];

    uint2 Q = make_uint2(1u, 0u);
    if (tid < q) Q = ld_query(qs + tid);
    const bool valid = tid < q && Q.x <= Q.y && Q.y < n;
    if (tid < q && !valid && err != nullptr) atomicAdd(err, 1u);

    float my_min = f_nan();
    Cand my_c;
    cand_init(my_c);

    for (int j = 0; j < G; ++j) {
        const uint32_t l = __shfl_sync(mask, Q.x, j, G);
        const uint32_t r = __shfl_sync(mask, Q.y, j, G) + 1u;
        const bool v = __shfl_sync(mask, valid ? 1u : 0u, j, G) != 0u;
        if (!v) continue;  // uniform across the tile
        Cand c;
        cand_init(c);
        float m = f_inf();
        if (ARGMIN) {
            cl_descend<R, G, true>(lv, l, r, lane, c, m);
            cl_reduce_cand<G>(c, mask);
            if (lane == uint32_t(j)) {
                my_c = c;
                my_min = c.v;
            }
        } else {
            cl_descend<R, G, false>(lv, l, r, lane, c, m);
            m = cl_reduce_min<G>(m, mask);
            if (m == 0.0f) {  // signed-zero tie: take the bits of the first occurrence
                cand_init(c);
                cl_descend<R, G, true>(lv, l, r, lane, c, m);
                cl_reduce_cand<G>(c, mask);
                m = c.v;
            }
            if (lane == uint32_t(j)) my_min = m;
        }
    }
    if (tid < q) {
        if (ARGMIN) {
            const uint32_t idx = valid ? cand_index<R>(lv, my_c, Q.x) : kNoPos;
            st_stream(out_idx + tid, idx);
            if (out_min != nullptr) st_stream(out_min + tid, valid ? my_min : f_nan());
        } else {
            st_stream(out_min + tid, my_min);
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
        attr[0].val.accessPolicyWindow.hitRatio = 1.0f;
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
    const uint32_t grid = (a.q + 255u) / 256u;
    const bool argmin = a.out_idx != nullptr;
    if (a.variant == 2) {
        return argmin ? launch_with_window(query_vl_kernel<R, true>, grid, a, s)
                      : launch_with_window(query_vl_kernel<R, false>, grid, a, s);
    }
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
