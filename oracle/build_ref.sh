#!/usr/bin/env bash
# Builds oracle/_ref/librmq_ref.so from the reference's own sources (read in
# place, never copied) for pinning the oracle.  TEST INFRASTRUCTURE ONLY.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: /root/reference)
#
# The reference's CPU path (src/cpu_methods.h) #includes the header of an
# external CPU RMQ library that the reference does not vendor
# (../hrmq/includes/RMQRMM64.h); the functions used here never call it, so a
# declaration-only stand-in of that header is written into oracle/_ref/stub.
# src/tools.h reads cudaDeviceProp::memoryClockRate, which CUDA 13 removed; it
# is mapped onto an existing field for compilation (that code is never run).
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
    echo "build_ref: reference sources not found at $REF; nothing built" >&2
    exit 0
fi
mkdir -p "$OUT/stub/hrmq/includes" "$OUT/stub/inc"
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
nvcc -std=c++20 -O2 -w -shared -Xcompiler -fPIC,-fopenmp -lgomp \
    -DBSIZE=1024 -DIS_LONG=0 -DXXX_CG_SIZE_LOG=3 -DXXX_CG_AMOUNT_LOG=2 \
    -DTRIVCHECK_LOG_NUM_DIFFQ=10 -DRAND_TRIVCHECK_LOG_NUM_DIFFQ=15 \
    -DmemoryClockRate=memoryBusWidth \
    -I "$REF" -I "$REF/src" -I "$OUT/stub/inc" \
    -gencode arch=compute_103a,code=sm_103a \
    "$HERE/ref_harness.cu" -o "$OUT/librmq_ref.so"
echo "build_ref: wrote $OUT/librmq_ref.so"
