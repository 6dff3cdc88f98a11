#!/usr/bin/env bash
# Builds oracle/_ref/librmq_ref.so from the reference's own sources (read in
# place, never copied) for pinning the oracle.  TEST INFRASTRUCTURE ONLY.
#
# Usage: oracle/build_ref.sh REFERENCE_ROOT
#    or: RMQ_REFERENCE_ROOT=<reference checkout> oracle/build_ref.sh
#
# The reference's CPU path (src/cpu_methods.h) #includes the header of an
# external CPU RMQ library that the reference does not vendor
# (../hrmq/includes/RMQRMM64.h); the functions used here never call it, so a
# declaration-only stand-in of that header is written into oracle/_ref/stub.
# src/tools.h reads cudaDeviceProp::memoryClockRate, which CUDA 13 removed; it
# is mapped onto an existing field for compilation (that code is never run).
set -euo pipefail
REF="${1:-${RMQ_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
    echo "build_ref: name the reference checkout (argument or RMQ_REFERENCE_ROOT); nothing built" >&2
    exit 0
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
    echo "build_ref: reference sources not found at $REF; nothing built" >&2
    exit 0
fi
mkdir -p "$OUT/stub/hrmq/includes" "$OUT/stub/inc" "$OUT/stub/x"
cat > "$OUT/stub/hrmq/includes/RMQRMM64.h" <<'H'
#pragma once
// Declaration-only stand-in: the pinned functions never construct it.
namespace rmqrmm {
class RMQRMM64 {
public:
    RMQRMM64(int*, unsigned long);
    unsigned int getSize();
    unsigned long queryRMQ(unsigned long, unsigned long);
};
}
H
# Declaration-only OptiX stand-in for parsing src/rtx_functions.h (host code
# that src/xxx.h includes; a device-code build never compiles or calls it).
cat > "$OUT/stub/inc/optix.h" <<'H'
#pragma once
#include <cstddef>
#include <cuda.h>
typedef struct OptixDeviceContext_t* OptixDeviceContext;
typedef struct OptixModule_t* OptixModule;
typedef struct OptixPipeline_t* OptixPipeline;
typedef struct OptixProgramGroup_t* OptixProgramGroup;
typedef unsigned long long OptixTraversableHandle;
enum OptixResult { OPTIX_SUCCESS = 0 };
enum { OPTIX_GEOMETRY_FLAG_NONE, OPTIX_EXCEPTION_FLAG_NONE, OPTIX_COMPILE_OPTIMIZATION_DEFAULT,
       OPTIX_COMPILE_DEFAULT_MAX_REGISTER_COUNT, OPTIX_COMPILE_DEBUG_LEVEL_NONE,
       OPTIX_TRAVERSABLE_GRAPH_FLAG_ALLOW_SINGLE_GAS, OPTIX_PROGRAM_GROUP_KIND_RAYGEN,
       OPTIX_PROGRAM_GROUP_KIND_MISS, OPTIX_PROGRAM_GROUP_KIND_HITGROUP, OPTIX_BUILD_INPUT_TYPE_TRIANGLES,
       OPTIX_VERTEX_FORMAT_FLOAT3, OPTIX_INDICES_FORMAT_UNSIGNED_INT3, OPTIX_BUILD_OPERATION_BUILD,
       OPTIX_BUILD_OPERATION_UPDATE, OPTIX_PROPERTY_TYPE_COMPACTED_SIZE, OPTIX_PROPERTY_TYPE_AABBS,
       OPTIX_BUILD_FLAG_ALLOW_COMPACTION = 1, OPTIX_BUILD_FLAG_ALLOW_UPDATE = 2,
       OPTIX_BUILD_FLAG_PREFER_FAST_TRACE = 4, OPTIX_BUILD_FLAG_ALLOW_RANDOM_VERTEX_ACCESS = 8 };
#define OPTIX_SBT_RECORD_HEADER_SIZE 32
#define OPTIX_SBT_RECORD_ALIGNMENT 16
typedef void (*OptixLogCallback)(unsigned int, const char*, const char*, void*);
struct OptixDeviceContextOptions { OptixLogCallback logCallbackFunction; void* logCallbackData; int logCallbackLevel; };
struct OptixModuleCompileOptions { int maxRegisterCount, optLevel, debugLevel; };
struct OptixPipelineCompileOptions { int usesMotionBlur; unsigned traversableGraphFlags; int numPayloadValues,
    numAttributeValues; unsigned exceptionFlags; const char* pipelineLaunchParamsVariableName; };
struct OptixProgramGroupOptions { int reserved; };
struct OptixPGEntry { OptixModule module; const char* entryFunctionName; };
struct OptixPGHit { OptixModule moduleCH; const char* entryFunctionNameCH; OptixModule moduleAH;
    const char* entryFunctionNameAH; OptixModule moduleIS; const char* entryFunctionNameIS; };
struct OptixProgramGroupDesc { int kind; unsigned flags; OptixPGEntry raygen, miss; OptixPGHit hitgroup; };
struct OptixPipelineLinkOptions { unsigned maxTraceDepth; };
struct OptixShaderBindingTable { CUdeviceptr raygenRecord, exceptionRecord, missRecordBase;
    unsigned missRecordStrideInBytes, missRecordCount; CUdeviceptr hitgroupRecordBase;
    unsigned hitgroupRecordStrideInBytes, hitgroupRecordCount; };
struct OptixTriangleArray { int vertexFormat; unsigned numVertices; const CUdeviceptr* vertexBuffers;
    const unsigned* flags; unsigned numSbtRecords; int indexFormat; unsigned numIndexTriplets;
    CUdeviceptr indexBuffer; };
struct OptixBuildInput { int type; OptixTriangleArray triangleArray; };
struct OptixAccelBuildOptions { unsigned buildFlags; int operation; };
struct OptixAccelEmitDesc { int type; CUdeviceptr result; };
struct OptixAccelBufferSizes { size_t outputSizeInBytes, tempSizeInBytes, tempUpdateSizeInBytes; };
template <typename... A> OptixResult optixInit(A...);
template <typename... A> OptixResult optixDeviceContextCreate(A...);
template <typename... A> OptixResult optixModuleCreate(A...);
template <typename... A> OptixResult optixModuleCreateFromPTX(A...);
template <typename... A> OptixResult optixProgramGroupCreate(A...);
template <typename... A> OptixResult optixPipelineCreate(A...);
template <typename... A> OptixResult optixSbtRecordPackHeader(A...);
template <typename... A> OptixResult optixAccelComputeMemoryUsage(A...);
template <typename... A> OptixResult optixAccelBuild(A...);
template <typename... A> OptixResult optixAccelCompact(A...);
template <typename... A> OptixResult optixLaunch(A...);
inline const char* optixGetErrorString(OptixResult) { return ""; }
H
# src/constants.cuh includes the CMake-configured constants_config.cuh; its
# four values are passed with -D below, so an empty file stands in for it.
echo "// configuration values are passed with -D" > "$OUT/stub/inc/constants_config.cuh"
# Device code of the reference's kernels (paper configurations), loadable on
# any host through the driver API.
nvcc -std=c++20 -O3 -w -fatbin \
    -DBSIZE=1024 -DIS_LONG=0 -DXXX_CG_SIZE_LOG=4 -DXXX_CG_AMOUNT_LOG=1 \
    -DTRIVCHECK_LOG_NUM_DIFFQ=10 -DRAND_TRIVCHECK_LOG_NUM_DIFFQ=15 \
    -DmemoryClockRate=memoryBusWidth \
    -I "$REF" -I "$REF/src" -I "$OUT/stub/inc" -I "$OUT/stub/x" \
    -gencode arch=compute_103a,code=sm_103a \
    "$HERE/ref_gpu_harness.cu" -o "$OUT/rmq_ref_kernels.fatbin"
nvcc -std=c++20 -O2 -w -shared -Xcompiler -fPIC,-fopenmp -lgomp \
    -DBSIZE=1024 -DIS_LONG=0 -DXXX_CG_SIZE_LOG=3 -DXXX_CG_AMOUNT_LOG=2 \
    -DTRIVCHECK_LOG_NUM_DIFFQ=10 -DRAND_TRIVCHECK_LOG_NUM_DIFFQ=15 \
    -DmemoryClockRate=memoryBusWidth \
    -I "$REF" -I "$REF/src" -I "$OUT/stub/inc" \
    -gencode arch=compute_103a,code=sm_103a \
    "$HERE/ref_harness.cu" -o "$OUT/librmq_ref.so"
echo "build_ref: wrote $OUT/librmq_ref.so and $OUT/rmq_ref_kernels.fatbin"
