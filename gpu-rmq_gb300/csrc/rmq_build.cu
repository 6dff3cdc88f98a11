// rmq_build.cu — construction of the block-minimum hierarchy.
//
// Reference: xxx_build_step (src/xxx.h:91-120) reduces each aligned chunk of
// rf source entries to one minimum with a cooperative-groups tile, one launch
// per level (src/xxx.h:258-265).  Here the levels whose blocks fit in an
// 8192-entry tile are built by one fused streaming kernel (level 0 is read
// once), and the small levels above by a single-CTA tail kernel.  Every block
// stores its first-occurring minimum and that entry's level-0 index, which
// argmin queries use.  build_step_kernel (one level step, rf/8 lanes per
// block) covers large intermediate levels of very large arrays.
#include "rmq_internal.h"

namespace rmq {

__device__ __forceinline__ void ld_sector_u32(const uint32_t* p, uint32_t (&v)[8]) {
    asm(
        "ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]),
          "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "l"(p));
}

// One output block per group of LPB = rf/8 lanes.
//   src, src_size : level k (level 0 = caller's array, not padded)
//   src_idx       : level-0 indices of level k's entries (null for k = 0)
//   src_padded    : src has at least round_up(src_size, 8) readable entries
template <int R>
__global__ void __launch_bounds__(256)
build_step_kernel(const float* __restrict__ src, const uint32_t* __restrict__ src_idx,
                  uint32_t src_size, int src_padded, float* __restrict__ dst,
                  uint32_t* __restrict__ dst_idx, uint32_t dst_size) {
    constexpr uint32_t LPB = (1u << R) / 8u;
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t blk = gt / LPB;
    const uint32_t sub = gt % LPB;

    Cand c;
    cand_init(c);
    if (blk < dst_size) {
        const uint32_t s = (blk << R) + 8u * sub;
        if (s < src_size) {
            float v[8];
            if (src_padded || s + 8u <= src_size) {
                ld_sector(src + s, v);
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) v[j] = (s + j < src_size) ? src[s + j] : f_inf();
            }
            uint32_t ix[8];
            if (src_idx != nullptr) {
                ld_sector_u32(src_idx + s, ix);  // level >= 1 buffers are padded
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) ix[j] = s + j;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (s + j < src_size) cand_update(c, v[j], ix[j], 0);
            }
        }
    }
    // Combine the LPB lanes of a block (groups never straddle a warp).
#pragma unroll
    for (uint32_t o = 1; o < LPB; o <<= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, c.v, o);
        const uint32_t op = __shfl_xor_sync(0xffffffffu, c.pos, o);
        cand_update(c, ov, op, 0);
    }
    if (blk < dst_size && sub == 0) {
        dst[blk] = c.v;
        if (dst_idx != nullptr) dst_idx[blk] = c.pos;
    }
}

Layout plan_layout(uint64_t n, uint64_t t, uint32_t rf_log) {
    Layout lay;
    lay.n = n;
    lay.t = t;
    lay.rf_log = rf_log;
    lay.num_levels = 1;
    lay.size[0] = n;
    lay.offset[0] = ~uint64_t(0);
    uint64_t size = n;
    uint64_t off = 0;
    const uint64_t rf = uint64_t(1) << rf_log;
    while (lay.num_levels < uint32_t(kMaxLevels) && size > t) {
        size = (size + rf - 1) >> rf_log;
        off = (off + kLevelAlign - 1) & ~uint64_t(kLevelAlign - 1);
        lay.offset[lay.num_levels] = off;
        lay.size[lay.num_levels] = size;
        lay.num_levels++;
        off += size;
    }
    // Pad the end so that full-sector reads of the last level stay in bounds.
    lay.total = (off + kLevelAlign - 1) & ~uint64_t(kLevelAlign - 1);
    return lay;
}

// ---------------------------------------------------------------------------
// Fused build: one CTA reads a tile of kTile level-0 entries once (256-bit
// loads, a warp covers 1 KiB contiguous) and produces every level whose
// blocks fit inside the tile (rf^m <= kTile: 4 levels at rf = 8, 3 at 16,
// 2 at 32), keeping intermediate (value, first index) pairs in shared memory.
// The levels above are small; a single-CTA tail kernel finishes them (or
// grid-wide build_step launches while they are still large).
// ---------------------------------------------------------------------------
constexpr uint32_t kTile = 8192;
constexpr uint32_t kTileSectors = kTile / 8;
constexpr uint32_t kFusedThreads = 256;
constexpr uint32_t kTailMaxEntries = 16384;  // largest level the tail CTA reads

struct LevelOut {
    float* val[kMaxLevels];
    uint32_t* idx[kMaxLevels];  // null entries when argmin arrays are not built
    uint32_t size[kMaxLevels];
};

// First-occurrence minimum over candidates visited in ascending position;
// p == kNoPos marks an absent candidate.
struct VP {
    float v;
    uint32_t p;
};

__device__ __forceinline__ void vp_take(VP& cur, float v, uint32_t p) {
    if (p != kNoPos && (cur.p == kNoPos || v < cur.v)) {
        cur.v = v;
        cur.p = p;
    }
}

template <int R>
constexpr uint32_t fused_depth() {
    return 13u / uint32_t(R);  // largest m with rf^m <= kTile = 2^13
}

template <int R>
__global__ void __launch_bounds__(kFusedThreads)
build_fused_kernel(const float* __restrict__ a, uint32_t n, LevelOut out, uint32_t depth) {
    constexpr uint32_t RF = 1u << R;
    constexpr uint32_t SPB = RF / 8u;  // sectors per level-1 block
    __shared__ float sv[kTileSectors];
    __shared__ uint32_t sp[kTileSectors];
    const uint32_t tid = threadIdx.x;
    const uint64_t base = uint64_t(blockIdx.x) * kTile;
    const uint64_t pol = policy_evict_first();

    // Stage 0: per-sector first minimum.
#pragma unroll
    for (uint32_t i = 0; i < kTileSectors / kFusedThreads; ++i) {
        const uint32_t sec = tid + kFusedThreads * i;
        const uint64_t s = base + 8u * sec;
        VP c{f_inf(), kNoPos};
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
                if (s + j < n) vp_take(c, v[j], uint32_t(s + j));
        }
        sv[sec] = c.v;
        sp[sec] = c.p;
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
            res[i] = VP{f_inf(), kNoPos};
            if (e < cnt) {
                for (uint32_t j = 0; j < fan; ++j) vp_take(res[i], sv[e * fan + j], sp[e * fan + j]);
            }
        }
        __syncthreads();
        const uint64_t gbase = uint64_t(blockIdx.x) * cnt;
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

// Single CTA: builds levels from+1 .. last from level `from` (already built),
// level after level, with a block barrier between levels (global writes of
// the block are visible to it after __syncthreads).
template <int R>
__global__ void __launch_bounds__(1024) build_tail_kernel(LevelOut out, uint32_t from, uint32_t last) {
    constexpr uint32_t RF = 1u << R;
    for (uint32_t k = from; k < last; ++k) {
        const float* src = out.val[k];
        const uint32_t* src_idx = out.idx[k];
        const uint32_t src_size = out.size[k];
        for (uint32_t e = threadIdx.x; e < out.size[k + 1]; e += blockDim.x) {
            VP c{f_inf(), kNoPos};
            for (uint32_t j = 0; j < RF; ++j) {
                const uint32_t ch = e * RF + j;
                if (ch < src_size) vp_take(c, src[ch], src_idx != nullptr ? src_idx[ch] : ch);
            }
            out.val[k + 1][e] = c.v;
            if (out.idx[k + 1] != nullptr) out.idx[k + 1][e] = c.p;
        }
        __syncthreads();
    }
}

template <int R>
static int plan_launches(const Layout& lay, uint32_t* fused, uint32_t* grid_steps, bool* tail) {
    const uint32_t top = lay.num_levels - 1;
    *fused = top < fused_depth<R>() ? top : fused_depth<R>();
    uint32_t k = *fused;
    *grid_steps = 0;
    while (k < top && lay.size[k] > kTailMaxEntries) {
        ++*grid_steps;
        ++k;
    }
    *tail = k < top;
    return (*fused > 0 ? 1 : 0) + int(*grid_steps) + (*tail ? 1 : 0);
}

int build_launch_count(const Layout& lay) {
    uint32_t f, g;
    bool t;
    switch (lay.rf_log) {
        case 3: return plan_launches<3>(lay, &f, &g, &t);
        case 4: return plan_launches<4>(lay, &f, &g, &t);
        case 5: return plan_launches<5>(lay, &f, &g, &t);
        default: return 0;
    }
}

template <int R>
static cudaError_t build_levels(const Layout& lay, const float* d_values, float* val_buf,
                                uint32_t* idx_buf, cudaStream_t s) {
    constexpr uint32_t LPB = (1u << R) / 8u;
    if (lay.num_levels < 2) return cudaSuccess;
    LevelOut out;
    for (uint32_t k = 0; k < uint32_t(kMaxLevels); ++k) {
        out.val[k] = nullptr;
        out.idx[k] = nullptr;
        out.size[k] = 0;
    }
    for (uint32_t k = 0; k < lay.num_levels; ++k) {
        out.size[k] = uint32_t(lay.size[k]);
        if (k > 0) {
            out.val[k] = val_buf + lay.offset[k];
            out.idx[k] = idx_buf == nullptr ? nullptr : idx_buf + lay.offset[k];
        }
    }
    uint32_t fused, steps;
    bool tail;
    plan_launches<R>(lay, &fused, &steps, &tail);
    const uint32_t n = uint32_t(lay.size[0]);
    const uint32_t tiles = uint32_t((uint64_t(n) + kTile - 1) / kTile);
    build_fused_kernel<R><<<tiles, kFusedThreads, 0, s>>>(d_values, n, out, fused);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint32_t k = fused;
    for (uint32_t i = 0; i < steps; ++i, ++k) {
        const uint32_t dst_size = out.size[k + 1];
        const uint64_t threads = uint64_t(dst_size) * LPB;
        const uint32_t grid = uint32_t((threads + 255) / 256);
        build_step_kernel<R><<<grid, 256, 0, s>>>(out.val[k], out.idx[k], out.size[k], 1, out.val[k + 1],
                                                 out.idx[k + 1], dst_size);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (tail) {
        build_tail_kernel<R><<<1, 1024, 0, s>>>(out, k, lay.num_levels - 1);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t launch_build(const Layout& lay, const float* d_values, float* val_buf,
                         uint32_t* idx_buf, cudaStream_t s) {
    switch (lay.rf_log) {
        case 3: return build_levels<3>(lay, d_values, val_buf, idx_buf, s);
        case 4: return build_levels<4>(lay, d_values, val_buf, idx_buf, s);
        case 5: return build_levels<5>(lay, d_values, val_buf, idx_buf, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace rmq
