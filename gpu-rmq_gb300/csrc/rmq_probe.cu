// rmq_probe.cu — the L2 read rate of this GPU, for the coarse levels' roofline.
//
// The query kernels read the coarse levels (levels >= 1) of a hierarchy as
// 32-byte sectors that stay in L2.  Their bound is therefore the rate at which
// the SMs can read L2-resident sectors, which no datasheet gives for GB300
// (two dies; half of the L2 lines live behind the die-to-die link for any
// SM).  This kernel measures it with the query kernels' own load form
// (256-bit, L1 bypassed): every thread reads sectors of a buffer that fits in
// L2, either in address order or at hashed (random) sector positions, and
// folds them into a minimum that one store keeps live.
#include "../../include/rmq_gb300.h"
#include "rmq_internal.h"

namespace {

__global__ void __launch_bounds__(256)
l2_read_kernel(const float* __restrict__ buf, uint64_t sectors, uint32_t passes, int random,
               float* __restrict__ sink) {
    const uint64_t tid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    float m = rmq::f_inf();
    for (uint32_t p = 0; p < passes; ++p) {
        for (uint64_t i = tid; i < sectors; i += stride) {
            // Multiplicative hash (odd multiplier) of the sector number, taken
            // modulo the sector count (a power of two): a permutation of the
            // sectors, so every pass reads each sector once either way.
            const uint64_t s = random ? ((i + p) * 0x9E3779B97F4A7C15ull) & (sectors - 1) : i;
            float v[8];
            rmq::ld_sector(buf + 8 * s, v);
            m = fminf(m, rmq::fmin3(rmq::fmin3(v[0], v[1], v[2]), rmq::fmin3(v[3], v[4], v[5]), fminf(v[6], v[7])));
        }
    }
    if (m < -1.0f) sink[tid & 1023] = m;  // never true for the probe's data; keeps the loads live
}

}  // namespace

extern "C" int rmq_measure_l2_read(const float* d_buf, uint64_t bytes, uint32_t passes, int32_t random,
                                   rmq_stream_t stream, float* ms_out) {
    if (d_buf == nullptr || ms_out == nullptr || passes == 0) return RMQ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d_buf) & 31u) != 0) return RMQ_ERR_ARG;
    const uint64_t sectors = bytes / 32;
    if (sectors < 1024 || (sectors & (sectors - 1)) != 0) return RMQ_ERR_ARG;  // a power of two
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // 8 CTAs of 256 threads per SM: 64 warps, the SM's limit, to keep as
    // many sector loads in flight as it allows.
    const uint32_t grid = uint32_t(sms > 0 ? sms : 1) * 8u;
    float* sink = const_cast<float*>(d_buf);  // written only if a value is below -1
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        l2_read_kernel<<<grid, 256, 0, s>>>(d_buf, sectors, 1u, random, sink);  // brings the buffer into L2
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) {
        l2_read_kernel<<<grid, 256, 0, s>>>(d_buf, sectors, passes, random, sink);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms_out, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return RMQ_ERR_CUDA;
    }
    return RMQ_OK;
}
