// ref_harness.cu — pinning harness for the oracle (TEST INFRASTRUCTURE ONLY).
//
// Compiled by oracle/build_ref.sh, only where the reference sources are
// present, into oracle/_ref/librmq_ref.so.  It includes the reference's own
// generator (src/rand.cuh) and CPU brute-force RMQ (src/cpu_methods.h) from
// the reference tree and exposes them with C linkage so that the CPU tests can
// check the oracle restatement and the product's generators against them, and
// so that tests/golden/make_golden.py can write fixtures.  Nothing here is
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
#include <omp.h>

// Definitions the reference headers expect from src/main.cu and
// common/common.h (terminal colours are disabled).
#define AC_RESET ""
#define AC_RED ""
#define AC_GREEN ""
#define AC_YELLOW ""
#define AC_MAGENTA ""
#define AC_CYAN ""
#define AC_BOLDGREEN ""
#define AC_BOLDCYAN ""
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
static const char* algStr[25] = {"cpu-base", "cpu-hrmq", "gpu-base"};
static const char* algStrIdx[25] = {"cpu-base-idx", "cpu-hrmq-idx", "gpu-base-idx"};
static std::string directory_save_aux_data = "";
void CPUPowerBegin(const char*, int, std::string);
void CPUPowerEnd();
void GPUPowerBegin(const char*, int, int, std::string);
void GPUPowerEnd();

#include "common/Timer.h"
#include "src/rand.cuh"
#include "src/tools.h"
#include "src/cpu_methods.h"

extern "C" {

void ref_random_array(uint32_t n, int seed, float* out) {
    float* a = random_array_par_cpu<uint32_t>(n, seed);
    std::memcpy(out, a, sizeof(float) * n);
    delete[] a;
}

void ref_random_queries(uint32_t q, int lr, uint32_t n, int seed, int trivial, uint32_t* out) {
    uint2* qs = random_queries_par_cpu<uint32_t, uint2>(q, lr, n, 1, seed, trivial != 0);
    std::memcpy(out, qs, sizeof(uint2) * q);
    delete[] qs;
}

uint32_t ref_sample_indices(uint32_t original_size, uint32_t sample_size, int seed, uint32_t* out) {
    uint32_t* s = randomly_sample_indices<uint32_t>(original_size, sample_size, seed);
    const uint32_t m = original_size <= sample_size ? original_size : sample_size;
    std::memcpy(out, s, sizeof(uint32_t) * m);
    free(s);
    return m;
}

static CmdArgs quiet_args() {
    CmdArgs a{};
    a.reps = 1;
    a.save_time = 0;
    a.save_power = 0;
    return a;
}

void ref_cpu_rmq(uint32_t n, uint32_t q, float* A, const uint32_t* Q, int nt, float* out) {
    float* r = cpu_rmq<float, uint32_t, uint2>(n, int(q), A, (uint2*)Q, nt, quiet_args());
    std::memcpy(out, r, sizeof(float) * q);
    delete[] r;
}

void ref_cpu_rmq_idx(uint32_t n, uint32_t q, float* A, const uint32_t* Q, int nt, uint32_t* out) {
    uint32_t* r = cpu_rmq_idx<float, uint32_t, uint2>(n, int(q), A, (uint2*)Q, nt, quiet_args());
    std::memcpy(out, r, sizeof(uint32_t) * q);
    delete[] r;
}

}  // extern "C"
