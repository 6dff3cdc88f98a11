// rmq_build.cu — construction of the block-minimum hierarchy.
//
// Reference: xxx_build_step (src/xxx.h:91-120) reduces each aligned chunk of
// rf source entries to one minimum with a cooperative-groups tile, one launch
// per level (src/xxx.h:258-265).  Here each level step is a streaming kernel
// in which rf/8 lanes cooperate on one output block: every lane reads one
// 32-byte sector with a 256-bit load (a warp reads 1 KiB contiguous), keeps
// the first occurrence of its sector minimum, and the lanes combine by
// (value, position) so the stored block minimum is the first-occurring one and
// its level-0 index is recorded for argmin queries.
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

int build_launch_count(const Layout& lay) { return int(lay.num_levels) - 1; }

template <int R>
static cudaError_t build_levels(const Layout& lay, const float* d_values, float* val_buf,
                                uint32_t* idx_buf, cudaStream_t s) {
    constexpr uint32_t LPB = (1u << R) / 8u;
    for (uint32_t k = 0; k + 1 < lay.num_levels; ++k) {
        const float* src = k == 0 ? d_values : val_buf + lay.offset[k];
        const uint32_t* src_idx = (k == 0 || idx_buf == nullptr) ? nullptr : idx_buf + lay.offset[k];
        float* dst = val_buf + lay.offset[k + 1];
        uint32_t* dst_idx = idx_buf == nullptr ? nullptr : idx_buf + lay.offset[k + 1];
        const uint32_t dst_size = uint32_t(lay.size[k + 1]);
        const uint64_t threads = uint64_t(dst_size) * LPB;
        const uint32_t grid = uint32_t((threads + 255) / 256);
        build_step_kernel<R><<<grid, 256, 0, s>>>(src, src_idx, uint32_t(lay.size[k]), k > 0 ? 1 : 0,
                                                 dst, dst_idx, dst_size);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
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
