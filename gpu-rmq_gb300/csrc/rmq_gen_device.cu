// rmq_gen_device.cu — seeded device-side input generators
// (include/rmq_gb300_batch.h).  The batched and serving workloads hold up to
// ~2^31 values and ~2^31 queries; generating them on the host with the
// reference's sequential engines (src/rand.cuh:49-217) would take minutes, so
// they come from a counter-based hash (splitmix64 finaliser) instead: value i
// depends only on (seed, i), independent of launch shape and GPU.
#include <cmath>
#include <cstdint>

#include "../../include/rmq_gb300_batch.h"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__global__ void gen_values_kernel(float* __restrict__ out, uint64_t n, uint64_t seed) {
    const uint64_t key = mix64(seed);
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t h = mix64(key ^ i);
        out[i] = float(h >> 40) * (1.0f / 16777216.0f);  // 24 random bits -> [0, 1)
    }
}

__global__ void gen_queries_kernel(uint2* __restrict__ out, uint64_t q, uint32_t n, int law, float ln_median,
                                   float sigma, uint64_t seed) {
    const uint64_t key = mix64(seed ^ 0x5157455259ull);
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < q; i += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t h1 = mix64(key ^ (2 * i));
        const uint64_t h2 = mix64(key ^ (2 * i + 1));
        uint32_t len;
        if (law == 0) {
            len = 1u + uint32_t(((h1 >> 32) * uint64_t(n)) >> 32);  // uniform in [1, n]
        } else {
            // Box-Muller on two 24-bit uniforms; u1 in (0, 1].
            const float u1 = (float(h1 >> 40) + 1.0f) * (1.0f / 16777216.0f);
            const float u2 = float(h1 & 0xFFFFFFull) * (1.0f / 16777216.0f);
            const float z = sqrtf(-2.0f * logf(u1)) * cosf(6.283185307f * u2);
            const float x = rintf(expf(ln_median + sigma * z));
            len = !(x >= 1.0f) ? 1u : (x >= float(n) ? n : uint32_t(x));
        }
        const uint64_t range = uint64_t(n) - len + 1u;
        const uint32_t l = uint32_t(((h2 >> 32) * range) >> 32);  // uniform in [0, n - len]
        out[i] = make_uint2(l, l + len - 1u);
    }
}

int grid_for(uint64_t work) {
    uint64_t g = (work + 255) / 256;
    return int(g < 152ull * 32 ? (g == 0 ? 1 : g) : 152ull * 32);
}

}  // namespace

extern "C" int rmq_gen_values_device(float* d_out, uint64_t n, uint64_t seed, rmq_stream_t stream) {
    if (d_out == nullptr) return n == 0 ? RMQ_OK : RMQ_ERR_ARG;
    if (n == 0) return RMQ_OK;
    gen_values_kernel<<<grid_for(n), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(d_out, n, seed);
    return cudaGetLastError() == cudaSuccess ? RMQ_OK : RMQ_ERR_CUDA;
}

extern "C" int rmq_gen_queries_device(uint32_t* d_lr, uint64_t q, uint64_t n, int32_t law, double median,
                                      double sigma, uint64_t seed, rmq_stream_t stream) {
    if (q == 0) return RMQ_OK;
    if (d_lr == nullptr || n == 0 || n > 0xFFFFFF00ull || (law != 0 && law != 1)) return RMQ_ERR_ARG;
    if (law == 1 && !(median >= 1.0 && sigma >= 0.0)) return RMQ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d_lr) & 7u) != 0) return RMQ_ERR_ARG;
    gen_queries_kernel<<<grid_for(q), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<uint2*>(d_lr), q, uint32_t(n), law, float(std::log(median > 1.0 ? median : 1.0)),
        float(sigma), seed);
    return cudaGetLastError() == cudaSuccess ? RMQ_OK : RMQ_ERR_CUDA;
}
