// ref_gpu_harness.cu — device-code build of the reference's own GPU kernels
// (TEST / BENCHMARK INFRASTRUCTURE ONLY).
//
// Compiled by oracle/build_ref.sh, where the reference sources exist, into
// oracle/_ref/rmq_ref_kernels.fatbin (device code only, so the file runs on
// any host architecture through the CUDA driver API; see oracle/ref_gpu.py).
// It instantiates, with the paper's chosen configurations, the reference's
// hierarchical kernels from src/xxx.h:
//   CL (alg 16): xxx_build_step<u32, uint2, 4, 1>, xxx_query<u32, uint2, 4, 1>
//                (16 lanes x 2 entries, rf 32)
//   VL (alg 20): xxx_build_step<u32, uint2, 2, 1>,
//                kernel_hierarchical_vector_load<u32, uint2, 1>   (rf 8)
// and the brute-force kernels of src/cuda_methods.cuh.  Nothing here is
// shipped or linked by the product.
#include <algorithm>
#include <bit>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <cuda_runtime.h>

#define ALG_CPU_BASE 0
#define ALG_CPU_HRMQ 1
#define ALG_GPU_BASE 2
#define ALG_GPU_RTX_BLOCKS 5
#define ALG_GPU_RTX_SER 10
#define ALG_XXX 16
#define ALG_INTERLEAVED 17
#define ALG_INTERLEAVED2 18
#define ALG_INTERLEAVED_IN_CUDA 19
#define ALG_HIERARCHICAL_VECTOR_LOAD 20
#define ALG_INTERLEAVED_IN_OPTIX 21
#define ALG_XXX_WITHOUT_SHUFFLES 23
#define ALG_XXX_MULTI_LOAD 24
#define ALG_CPU_BASE_IDX 100
#define ALG_CPU_HRMQ_IDX 101
#define ALG_GPU_BASE_IDX 102
#define ALG_GPU_RTX_BLOCKS_IDX 105
static const char* algStr[25] = {"cpu-base"};
static const char* algStrIdx[25] = {"cpu-base-idx"};
static std::string directory_save_aux_data = "";
void CPUPowerBegin(const char*, int, std::string);
void CPUPowerEnd();
void GPUPowerBegin(const char*, int, int, std::string);
void GPUPowerEnd();

#include "common/common.h"
#include "common/Timer.h"
#include "src/constants.cuh"
#include "src/tools.h"
#include "src/device_tools.cuh"
#include "src/cuda_methods.cuh"
#include "src/xxx.h"

using md_t = xxx_metadata_type<uint32_t, uint2>;
template __global__ void xxx_build_step<uint32_t, uint2, 4, 1>(const float*, float*, uint32_t, uint32_t);
template __global__ void xxx_query<uint32_t, uint2, 4, 1>(uint32_t, const uint2*, float*, const float*,
                                                          const float*, md_t, uint32_t);
template __global__ void xxx_build_step<uint32_t, uint2, 2, 1>(const float*, float*, uint32_t, uint32_t);
template __global__ void kernel_hierarchical_vector_load<uint32_t, uint2, 1>(const uint32_t, const uint32_t,
                                                                            const uint2*, float*, float4*,
                                                                            float4*, md_t, uint32_t);
template __global__ void kernel_rmq_basic<uint32_t, uint2>(uint32_t, int, float*, uint2*, float*);
template __global__ void kernel_rmq_basic_idx<uint32_t, uint2>(uint32_t, int, float*, uint2*, uint32_t*);
