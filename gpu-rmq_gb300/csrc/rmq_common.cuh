// rmq_common.cuh — layout and device helpers shared by the build and query kernels.
//
// The structure is the reference's multi-level block-minimum hierarchy
// (metadata struct src/constants.cuh:34-39, layout loop src/xxx.h:225-243):
// level 0 is the caller's array; level k+1 holds, for every aligned chunk of
// rf = 2^R entries of level k, the chunk minimum.  The hierarchy here also stores,
// next to every block minimum, the level-0 index of its first occurrence so
// that argmin queries need one extra load instead of a second descent.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rmq {

// Bounds-checked builds (-DRMQ_DEBUG_BOUNDS=1: librmq_gb300_checked.so)
// check every level load of the query kernels before it is made; a load
// outside its level is counted and skipped (it reads +inf), so the checked
// build never touches memory out of bounds either.  compute-sanitizer is not
// available where this library is tested; this is the substitute.
#ifndef RMQ_DEBUG_BOUNDS
#define RMQ_DEBUG_BOUNDS 0
#endif
#if RMQ_DEBUG_BOUNDS
// One counter per translation unit (no relocatable device code); each unit
// that launches checked kernels reads its own through
// RMQ_BOUNDS_COUNTER_READER.
static __device__ unsigned int g_rmq_bounds_bad = 0;
__device__ __forceinline__ bool bounds_ok(bool ok) {
    if (!ok) atomicAdd(&g_rmq_bounds_bad, 1u);
    return ok;
}
#define RMQ_BOUNDS_COUNTER_READER(name)                                                 \
    unsigned int name() {                                                               \
        unsigned int v = 0, z = 0;                                                      \
        if (cudaMemcpyFromSymbol(&v, g_rmq_bounds_bad, sizeof(v)) != cudaSuccess) {     \
            cudaGetLastError();                                                         \
            return ~0u;                                                                 \
        }                                                                               \
        cudaMemcpyToSymbol(g_rmq_bounds_bad, &z, sizeof(z));                            \
        return v;                                                                       \
    }
#endif

constexpr int kMaxLevels = 20;            // XXX_MAX_LEVELS, src/constants.cuh:14
constexpr uint32_t kLevelAlign = 32;      // XXX_LEVEL_ALIGNMENT, src/constants.cuh:15 (entries)
constexpr uint32_t kNoPos = 0xFFFFFFFFu;  // "no candidate" / invalid-query argmin

// Host-side description of the hierarchy (sizes in entries).
struct Layout {
    uint32_t num_levels = 1;
    uint32_t rf_log = 3;
    uint64_t n = 0;
    uint64_t t = 0;
    uint64_t size[kMaxLevels] = {};
    uint64_t offset[kMaxLevels] = {};  // offset of level k >= 1 inside the level buffer
    uint64_t total = 0;                // entries in the level buffer incl. alignment padding
};

// Descriptor of one array inside packed buffers (batched and served modes).
struct ArrayDesc {
    uint64_t val_off;   // first value of the array, in floats from the values base
    uint64_t lvl_base;  // first entry of its coarse levels, from the level-value base
    uint64_t idx_base;  // first entry of its argmin arrays, from the argmin base
    uint32_t num_levels;
    uint32_t size[kMaxLevels];
    uint32_t off[kMaxLevels];  // level k >= 1 starts at lvl_base + off[k]
};

// Index width: 32-bit handles (the reference's default nType = uint32_t,
// uint2 queries) or 64-bit handles (its IS_LONG build: uint64_t, ulong2
// queries; src/main.cu:21-27).
template <typename I>
struct IdxTraits;
template <>
struct IdxTraits<uint32_t> {
    using Pair = uint2;
    using Count = uint32_t;  // query numbers (q <= 2^32 - 1 on 32-bit handles)
    static constexpr uint32_t none = 0xFFFFFFFFu;
};
template <>
struct IdxTraits<uint64_t> {
    using Pair = ulonglong2;
    using Count = uint64_t;
    static constexpr uint64_t none = ~uint64_t(0);
};

// Device-side view passed by value to the kernels (fits easily in the 32 KB
// parameter space).
template <typename I>
struct LevelsT {
    const float* val[kMaxLevels];  // val[0] = caller's array
    const I* idx[kMaxLevels];      // idx[k] (k >= 1): level-0 index of block k's first minimum
    I size[kMaxLevels];
    uint32_t num_levels;
};
using Levels = LevelsT<uint32_t>;
using Levels64 = LevelsT<uint64_t>;

// ---------------------------------------------------------------------------
// Memory access helpers (inline PTX; sm_100+ 256-bit global loads).  The
// loads read data that no kernel writes while queries run, so they are not
// volatile: the compiler may batch independent loads before their first use.
// ---------------------------------------------------------------------------

// 32-byte (one sector) load through the non-coherent path; the caller
// guarantees 32-byte alignment and that all 8 floats lie inside the buffer.
__device__ __forceinline__ void ld_sector(const float* p, float (&v)[8]) {
    asm(
        "ld.global.nc.L1::no_allocate.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]),
          "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p));
}

// Same load with an explicit L2 cache policy (createpolicy result).
__device__ __forceinline__ void ld_sector_policy(const float* p, float (&v)[8], uint64_t pol) {
    asm(
        "ld.global.nc.L1::no_allocate.L2::cache_hint.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]),
          "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p), "l"(pol));
}

// Eight consecutive uint32 (one 32-byte sector) with an L2 cache policy.
// The same load, allocating in L1 (for the small top levels, which every SM
// re-reads for many queries).
__device__ __forceinline__ void ld_sector_l1_policy(const float* p, float (&v)[8], uint64_t pol) {
    asm(
        "ld.global.nc.L2::cache_hint.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]),
          "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p), "l"(pol));
}

__device__ __forceinline__ void ld_sector_u32_l1_policy(const uint32_t* p, uint32_t (&v)[8], uint64_t pol) {
    asm(
        "ld.global.nc.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]),
          "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "l"(p), "l"(pol));
}

__device__ __forceinline__ void ld_sector_u32_policy(const uint32_t* p, uint32_t (&v)[8], uint64_t pol) {
    asm(
        "ld.global.nc.L1::no_allocate.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]),
          "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "l"(p), "l"(pol));
}

__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ void ld_quad(const float* p, float (&v)[4]) {
    asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
                 : "l"(p));
}

__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

#ifndef RMQ_Q_HINT
#define RMQ_Q_HINT 0  // query stream: 0 = evict_first, 1 = default
#endif
#ifndef RMQ_ST_HINT
#define RMQ_ST_HINT 0  // result stores: 0 = .cs (streaming), 1 = default
#endif

// Streaming query load of one {l, r} pair; the query array is read once, so
// it is marked evict-first in L2 to leave room for the coarse levels.
__device__ __forceinline__ uint2 ld_query(const uint2* p) {
    uint2 v;
#if RMQ_Q_HINT == 0
    asm(
        "{\n\t.reg .b64 pol;\n\t"
        "createpolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
        "ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0,%1}, [%2], pol;\n\t}"
        : "=r"(v.x), "=r"(v.y) : "l"(p));
#else
    v = __ldg(p);
#endif
    return v;
}

__device__ __forceinline__ ulonglong2 ld_query(const ulonglong2* p) {
    ulonglong2 v;
    asm(
        "{\n\t.reg .b64 pol;\n\t"
        "createpolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
        "ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u64 {%0,%1}, [%2], pol;\n\t}"
        : "=l"(v.x), "=l"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ void st_stream(uint64_t* p, uint64_t v) {
    asm volatile("st.global.cs.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void st_stream(float* p, float v) {
#if RMQ_ST_HINT == 0
    asm volatile("st.global.cs.f32 [%0], %1;" :: "l"(p), "f"(v) : "memory");
#else
    *p = v;
#endif
}
__device__ __forceinline__ void st_stream(uint32_t* p, uint32_t v) {
#if RMQ_ST_HINT == 0
    asm volatile("st.global.cs.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
#else
    *p = v;
#endif
}

// ---------------------------------------------------------------------------
// Candidate ordering.  A candidate is an entry of some level together with the
// level-0 position of its block start.  The pieces a query visits partition
// [l, r], so positions are unique and ordering candidates by (value, position)
// with IEEE "<" on the value reproduces the brute-force scan's
// "first occurrence of the minimum" (src/cpu_methods.h:42-53).
// ---------------------------------------------------------------------------
struct Cand {
    float v;
    uint32_t pos;   // level-0 position of the candidate's block start
    uint32_t lvl;   // level the candidate came from
};

__device__ __forceinline__ void cand_init(Cand& c) {
    c.v = __int_as_float(0x7f800000);  // +inf
    c.pos = kNoPos;
    c.lvl = 0;
}

__device__ __forceinline__ bool cand_better(float v, uint32_t pos, const Cand& c) {
    return (v < c.v) | ((v == c.v) & (pos < c.pos));
}

__device__ __forceinline__ void cand_update(Cand& c, float v, uint32_t pos, uint32_t lvl) {
    if (cand_better(v, pos, c)) {
        c.v = v;
        c.pos = pos;
        c.lvl = lvl;
    }
}

__device__ __forceinline__ float f_inf() { return __int_as_float(0x7f800000); }
__device__ __forceinline__ float f_nan() { return __int_as_float(0x7fc00000); }

}  // namespace rmq
