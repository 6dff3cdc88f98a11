// rmq_build.cu — construction of the block-minimum hierarchy.
//
// Reference: xxx_build_step (src/xxx.h:91-120) reduces each aligned chunk of
// rf source entries to one minimum with a cooperative-groups tile, one launch
// per level (src/xxx.h:258-265).  Here the levels whose blocks fit in an
// 8192-entry tile are built by one fused streaming kernel (level 0 is read
// once), and the small levels above by a single-CTA tail kernel, or, for up
// to kInKernelTailMaxTiles tiles, inside the fused kernel itself
// (tail_upward: the tile completing a group computes the group's entry).  Every block
// stores its first-occurring minimum and that entry's level-0 index, which
// argmin queries use.  build_step_kernel (one level step, rf/8 lanes per
// block) covers large intermediate levels of very large arrays.  The kernels
// after the fused one are chained by programmatic dependent launch, so each
// is scheduled before its predecessor ends and no launch gap separates them.
#include "rmq_internal.h"
#include "rmq_buildk.cuh"

namespace rmq {

// Programmatic dependent launch: the kernels after the fused one are launched
// with programmatic stream serialization, so they are scheduled while the
// previous kernel's last CTAs still run and wait here (griddepcontrol.wait
// returns once the previous grid has completed and its writes are visible;
// in a kernel launched without the attribute it returns at once).
__device__ __forceinline__ void wait_previous_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Lets the next kernel of the stream be scheduled (its CTAs then wait in
// wait_previous_grid until this grid completes).
__device__ __forceinline__ void allow_next_grid() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// One output block per group of LPB = rf/8 lanes (P: position type).
//   src, src_size : level k (level 0 = caller's array, not padded)
//   src_idx       : level-0 indices of level k's entries (null for k = 0)
//   src_padded    : src has at least round_up(src_size, 8) readable entries
template <int R, typename P>
__global__ void __launch_bounds__(256)
build_step_kernel(const float* __restrict__ src, const P* __restrict__ src_idx, P src_size, int src_padded,
                  float* __restrict__ dst, P* __restrict__ dst_idx, P dst_size) {
    constexpr uint32_t LPB = (1u << R) / 8u;
    constexpr P kNone = IdxTraits<P>::none;
    wait_previous_grid();
    allow_next_grid();
    const uint64_t gt = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const P blk = P(gt / LPB);
    const uint32_t sub = uint32_t(gt % LPB);

    VPT<P> c{f_inf(), kNone};
    if (blk < dst_size) {
        const P s = (blk << R) + 8u * sub;
        if (s < src_size) {
            float v[8];
            if (src_padded || s + 8u <= src_size) {
                ld_sector(src + s, v);
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) v[j] = (s + j < src_size) ? src[s + j] : f_inf();
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (s + j < src_size) vp_take(c, v[j], src_idx != nullptr ? __ldg(src_idx + s + j) : P(s + j));
            }
        }
    }
    // Combine the LPB lanes of a block (groups never straddle a warp; the
    // lanes' positions are disjoint, so equal values keep the lower one).
#pragma unroll
    for (uint32_t o = 1; o < LPB; o <<= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, c.v, o);
        const P op = __shfl_xor_sync(0xffffffffu, c.p, o);
        if (op != kNone && (c.p == kNone || ov < c.v || (ov == c.v && op < c.p))) {
            c.v = ov;
            c.p = op;
        }
    }
    if (blk < dst_size && sub == 0) {
        dst[blk] = c.v;
        if (dst_idx != nullptr) dst_idx[blk] = c.p;
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
template <int R, typename P>
__global__ void __launch_bounds__(kFusedThreads)
build_fused_kernel(const float* __restrict__ a, P n, LevelOutT<P> out, uint32_t depth, TailPlan tp) {
    __shared__ float sv[kTileSectors];
    __shared__ P sp[kTileSectors];
    allow_next_grid();
    fused_tile<R>(a, n, out, depth, blockIdx.x, sv, sp);
    if (tp.top > tp.depth) tail_upward<R>(out, tp, blockIdx.x);
}

template <int R, typename P>
__global__ void __launch_bounds__(1024) build_tail_kernel(LevelOutT<P> out, uint32_t from, uint32_t last) {
    wait_previous_grid();
    tail_levels<R>(out, from, last);
}

// Launch with programmatic stream serialization (see wait_previous_grid).
template <typename... KArgs, typename... Args>
static cudaError_t launch_dependent(void (*kernel)(KArgs...), uint32_t grid, uint32_t block, cudaStream_t s,
                                    Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
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

// The in-kernel tail pays per tile (a fence and an atomic each, and a warp
// of every tile that completes a group staying on for the parent's entry);
// it wins over the two extra launches up to about a thousand tiles (n up to
// 2^23: 18.3 -> 15 us at n = 2^20, t = 64; 24.5 -> 21.7 us at n = 2^23) and
// loses beyond (70 -> 75 us at n = 2^26, 230 -> 261 us at n = 2^28).
constexpr uint32_t kInKernelTailMaxTiles = 1024;

uint64_t tail_counters(const Layout& lay) {
    if (lay.num_levels < 2 || lay.rf_log < 3 || lay.rf_log > 5) return 0;
    const uint32_t top = lay.num_levels - 1;
    const uint32_t fd = 13u / lay.rf_log;  // fused_depth<R>()
    const uint32_t depth = top < fd ? top : fd;
    uint64_t c = 0;
    for (uint32_t k = depth + 1; k <= top; ++k) c += lay.size[k];
    return c;
}

template <int R, typename P>
static cudaError_t build_levels(const Layout& lay, const float* d_values, float* val_buf, P* idx_buf,
                                cudaStream_t s, unsigned* counters) {
    constexpr uint32_t LPB = (1u << R) / 8u;
    if (lay.num_levels < 2) return cudaSuccess;
    LevelOutT<P> out;
    for (uint32_t k = 0; k < uint32_t(kMaxLevels); ++k) {
        out.val[k] = nullptr;
        out.idx[k] = nullptr;
        out.size[k] = 0;
    }
    for (uint32_t k = 0; k < lay.num_levels; ++k) {
        out.size[k] = P(lay.size[k]);
        if (k > 0) {
            out.val[k] = val_buf + lay.offset[k];
            out.idx[k] = idx_buf == nullptr ? nullptr : idx_buf + lay.offset[k];
        }
    }
    uint32_t fused, steps;
    bool tail;
    plan_launches<R>(lay, &fused, &steps, &tail);
    const P n = P(lay.size[0]);
    const uint32_t tiles = uint32_t((uint64_t(n) + kTile - 1) / kTile);
    TailPlan tp = {};
    tp.depth = fused;
    tp.top = fused;  // no tail inside the kernel
    if (counters != nullptr && fused + 1 < lay.num_levels && tiles <= kInKernelTailMaxTiles) {
        tp.top = lay.num_levels - 1;
        tp.per_tile = kTile >> (uint32_t(R) * fused);
        tp.counters = counters;
        uint64_t c = 0;
        for (uint32_t k = fused + 1; k <= tp.top; ++k) {
            tp.coff[k] = c;
            c += lay.size[k];
        }
    }
    build_fused_kernel<R, P><<<tiles, kFusedThreads, 0, s>>>(d_values, n, out, fused, tp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || tp.top > tp.depth) return e;
    uint32_t k = fused;
    for (uint32_t i = 0; i < steps; ++i, ++k) {
        const P dst_size = out.size[k + 1];
        const uint64_t threads = uint64_t(dst_size) * LPB;
        const uint32_t grid = uint32_t((threads + 255) / 256);
        e = launch_dependent(build_step_kernel<R, P>, grid, 256, s, out.val[k], (const P*)out.idx[k], out.size[k],
                             1, out.val[k + 1], out.idx[k + 1], dst_size);
        if (e != cudaSuccess) return e;
    }
    if (tail) {
        e = launch_dependent(build_tail_kernel<R, P>, 1, 1024, s, out, k, lay.num_levels - 1);
    }
    return e;
}

template <typename P>
static cudaError_t launch_build_p(const Layout& lay, const float* d_values, float* val_buf, P* idx_buf,
                                  cudaStream_t s, unsigned* counters) {
    switch (lay.rf_log) {
        case 3: return build_levels<3, P>(lay, d_values, val_buf, idx_buf, s, counters);
        case 4: return build_levels<4, P>(lay, d_values, val_buf, idx_buf, s, counters);
        case 5: return build_levels<5, P>(lay, d_values, val_buf, idx_buf, s, counters);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_build(const Layout& lay, const float* d_values, float* val_buf,
                         uint32_t* idx_buf, cudaStream_t s, unsigned* counters) {
    return launch_build_p<uint32_t>(lay, d_values, val_buf, idx_buf, s, counters);
}

cudaError_t launch_build64(const Layout& lay, const float* d_values, float* val_buf,
                           uint64_t* idx_buf, cudaStream_t s, unsigned* counters) {
    return launch_build_p<uint64_t>(lay, d_values, val_buf, idx_buf, s, counters);
}

}  // namespace rmq
