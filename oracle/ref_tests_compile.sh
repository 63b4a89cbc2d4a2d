#!/bin/sh
# Compiles and links the reference's own test programs (tests/test_qmckl_ao.cpp and
# tests/test_qmckl_mo.cpp of qmckl_sycl, read in place) against this library's C ABI through
# include/qmckl_gpu_sycl_compat.hpp, unmodified: their `#include "../include/qmckl_gpu.hpp"`
# is resolved to the compatibility header by searching only the -I directories for quoted
# includes (-I-). Besides the context, those programs run SYCL kernels of their own over the
# device arrays (checks of the getters); the host SYCL shim of oracle/sycl_shim stands in for
# a SYCL implementation so that they compile, which makes this a check of names, argument lists
# and linkage: the binaries in oracle/_ref/compat/ are not meant to run (their SYCL kernels
# would run on the host over device memory).
#
#   sh oracle/ref_tests_compile.sh [REFERENCE_DIR]
# (default: QMCKL_REFERENCE_DIR, else the location oracle/Makefile.ref uses)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-$(make -s -f "$HERE/Makefile.ref" print-reference)}
REPO=$(dirname "$HERE")
OUT=$HERE/_ref/compat
LIB=$REPO/qmckl_sycl_gb300/_lib
rm -rf "$OUT"
mkdir -p "$OUT/x" "$OUT/include" "$OUT/sys/sycl/ext/intel"
ln -s "$REPO/include/qmckl_gpu_sycl_compat.hpp" "$OUT/include/qmckl_gpu.hpp"
: > "$OUT/sys/sycl/ext/intel/fpga_extensions.hpp"
for t in test_qmckl_ao test_qmckl_mo; do
  g++ -std=c++17 -O1 -w -DQMCKL_COMPAT_EXTERNAL_SYCL -include "$HERE/sycl_shim/CL/sycl.hpp" \
      -I"$OUT/x" -I"$REPO/include" -I"$REF/tests" -I- -I"$OUT/sys" -I"$HERE/sycl_shim" \
      "$REF/tests/$t.cpp" -o "$OUT/$t" -L"$LIB" -lqmckl_gpu -Wl,-rpath,"$LIB"
done
echo "compiled: $OUT/test_qmckl_ao $OUT/test_qmckl_mo"
