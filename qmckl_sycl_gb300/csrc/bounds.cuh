// Opt-in bounds checks on the kernels' global stores, for the debug build of the library
// (compiled with -DQMCKL_BOUNDS_CHECK: `python -m qmckl_sycl_gb300.build --bounds` writes
// _lib/libqmckl_gpu_bounds.so). In that build every checked store first tests its element index
// against the extent of the array it writes; an index outside [0, extent) skips the store and
// the first such event is recorded (store site, index, extent) in a device word that the host
// reads with qmckl_bounds_check_status_device. Nothing traps or asserts: the kernel carries on
// and the caller decides. In the normal build QG_STORE_OK is the constant `true` and costs
// nothing.
//
// The library is compiled without relocatable device code, so each translation unit holds its
// own record; a static registrar hands its address to the status query (context.cpp).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace qg {

// Store sites (the value recorded with a violation).
enum BoundsSite : int {
  kSiteAoOut = 1,         // ao_vgl / ao_value rows written by the fused AO kernels
  kSiteAoPlanes = 2,      // BF16 planes written by the fused AO kernel (split-BF16 form)
  kSiteShellVgl = 3,      // shell_vgl
  kSitePointPerm = 4,     // processing order of the points
  kSiteSplitOut = 5,      // split-BF16 contraction output
  kSiteSplitPlanes = 6,   // split pass of an FP64 operand into BF16 planes
  kSiteDgemmOut = 7,      // FP64 DMMA contraction output
  kSiteSumParts = 8,      // split-K sums
  kSiteDistance = 9,      // e-n / e-e distances
  kSiteUtil = 10,         // transposes, strided copies, fills
  kSiteVjp = 11,          // adjoint kernels
};

#ifdef QMCKL_BOUNDS_CHECK
namespace dev {
struct BoundsRecord {
  int hit;           // 0 until the first violation
  int site;
  long long index;
  long long extent;
};
static __device__ BoundsRecord g_bounds;  // one per translation unit

__device__ __forceinline__ bool store_ok(int site, long long idx, long long extent) {
  if (idx >= 0 && idx < extent) return true;
  if (atomicCAS(&g_bounds.hit, 0, 1) == 0) {
    g_bounds.site = site;
    g_bounds.index = idx;
    g_bounds.extent = extent;
  }
  return false;
}
}  // namespace dev

// Registered by each translation unit at load time; returns the device address of its record.
void register_bounds_record(void* (*address)());

namespace {
void* bounds_record_address() {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, dev::g_bounds) != cudaSuccess) return nullptr;
  return p;
}
struct BoundsRegistrar {
  BoundsRegistrar() { register_bounds_record(&bounds_record_address); }
};
const BoundsRegistrar g_bounds_registrar;
}  // namespace

#define QG_STORE_OK(site, idx, extent) ::qg::dev::store_ok((site), (long long)(idx), (long long)(extent))
#else
#define QG_STORE_OK(site, idx, extent) true
#endif

}  // namespace qg
