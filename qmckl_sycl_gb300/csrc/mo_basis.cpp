// MO basis: setters/getters (src/qmckl_mo.cpp:459-583 of qmckl_sycl), finalize
// (coefficient transpose, src/qmckl_mo_sycl.cpp:137-189), select_mo (src/qmckl_mo.cpp:31-106)
// and the provide chain for mo_vgl / mo_value (src/qmckl_mo.cpp:114-453).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "internal.hpp"

using namespace qg;

namespace qg {
qmckl_exit_code_device provide_mo_split(Ctx* ctx, qmckl_context_device c, double* dst, bool value_only);
void invalidate_caches(Ctx* ctx);
}  // namespace qg

namespace {

Ctx* checked(qmckl_context_device c) {
  return qmckl_context_check_device(c) == QMCKL_NULL_CONTEXT_DEVICE ? nullptr : ctx_of(c);
}

}  // namespace

extern "C" {

qmckl_exit_code_device qmckl_finalize_mo_basis_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_finalize_mo_basis_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_finalize_mo_basis_device";
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  MoBasisData& mo = ctx->mo_basis;
  const int64_t A = ctx->ao_basis.ao_num, M = mo.mo_num;
  if (!mo.coefficient) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, "coefficients not set");
  double* ct = static_cast<double*>(dalloc(ctx, sizeof(double) * (size_t)(A * M)));
  if (!ct) return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  if (mo.coefficient_t) dfree(ctx, mo.coefficient_t);
  // coefficient is [M][A]; coefficient_t[i][j] = coefficient[j][i] (src/qmckl_mo_sycl.cpp:178-183)
  launch_transpose(ctx, mo.coefficient, M, A, ct);
  mo.coefficient_t = ct;
  if (mo.coef_split) {
    dfree(ctx, mo.coef_split);
    mo.coef_split = nullptr;
  }
  mo.mo_vgl_date = mo.mo_value_date = 0;
  return finish(ctx, context, fn);
}

bool qmckl_mo_basis_provided_device(qmckl_context_device context) {
  Ctx* ctx = checked(context);
  return ctx ? ctx->mo_basis.provided : false;
}

qmckl_exit_code_device qmckl_get_mo_basis_mo_num_device(qmckl_context_device context, int64_t* mo_num) {
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_get_mo_basis_mo_num", nullptr);
  if (ctx->mo_basis.uninitialized & 1)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_get_mo_basis_mo_num", nullptr);
  if (!mo_num) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_mo_basis_mo_num", "NULL pointer");
  *mo_num = ctx->mo_basis.mo_num;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_set_mo_basis_mo_num_device(qmckl_context_device context, int64_t mo_num) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  const int32_t mask = 1;
  if (!(ctx->mo_basis.uninitialized & mask))
    return qmckl_failwith_device(context, QMCKL_ALREADY_SET_DEVICE, "qmckl_set_mo_basis_mo_num_device", nullptr);
  if (mo_num <= 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_mo_basis_mo_num_device", "mo_num <= 0");
  ctx->mo_basis.mo_num = mo_num;
  ctx->mo_basis.uninitialized &= ~mask;
  ctx->mo_basis.provided = ctx->mo_basis.uninitialized == 0;
  if (ctx->mo_basis.provided) return qmckl_finalize_mo_basis_device(context);
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_set_mo_basis_coefficient_device(qmckl_context_device context, double* coefficient) {
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_set_mo_basis_coefficient_device";
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  const int32_t mask = 1 << 1;
  if (!(ctx->mo_basis.uninitialized & mask))
    return qmckl_failwith_device(context, QMCKL_ALREADY_SET_DEVICE, fn, nullptr);
  const int64_t A = ctx->ao_basis.ao_num, M = ctx->mo_basis.mo_num;
  if (A <= 0) return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, "ao_num is not set");
  if (M <= 0) return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, "mo_num is not set");
  if (!coefficient) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (!ensure_device(ctx)) return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, "no usable CUDA device");
  if (ctx->mo_basis.coefficient) {
    qmckl_exit_code_device rc = qmckl_free_device(context, ctx->mo_basis.coefficient);
    if (rc != QMCKL_SUCCESS_DEVICE) return qmckl_failwith_device(context, rc, fn, nullptr);
    ctx->mo_basis.coefficient = nullptr;
  }
  double* a = static_cast<double*>(dalloc(ctx, sizeof(double) * (size_t)(A * M)));
  if (!a) return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  qmckl_exit_code_device rc = copy(ctx, context, a, coefficient, sizeof(double) * (size_t)(A * M), fn, true);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  ctx->mo_basis.coefficient = a;
  ctx->mo_basis.uninitialized &= ~mask;
  ctx->mo_basis.provided = ctx->mo_basis.uninitialized == 0;
  if (ctx->mo_basis.provided) return qmckl_finalize_mo_basis_device(context);
  return QMCKL_SUCCESS_DEVICE;
}

// The reference declares this bool and returns exit codes through it (src/qmckl_mo.cpp:31);
// the ABI is kept: false on success, true on failure (details in the context's error).
bool qmckl_mo_basis_select_mo_device(qmckl_context_device context, int32_t* keep, int64_t size_max) {
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_get_mo_basis_select_mo_device";
  if (!ctx) return true;
  if (!ctx->mo_basis.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr) != 0;
  if (!keep) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer") != 0;
  MoBasisData& mo = ctx->mo_basis;
  const int64_t M = mo.mo_num, A = ctx->ao_basis.ao_num;
  if (size_max < M)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_mo_basis_select_mo",
                                 "Array too small: expected mo_num.") != 0;
  int64_t kept = 0;
  for (int64_t i = 0; i < M; ++i) kept += keep[i] != 0;
  if (kept == 0)
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, "no MO selected") != 0;
  double* c = static_cast<double*>(dalloc(ctx, sizeof(double) * (size_t)(A * kept)));
  if (!c) return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr) != 0;
  int64_t k = 0;
  for (int64_t i = 0; i < M; ++i)
    if (keep[i] != 0) {
      cudaMemcpyAsync(c + k * A, mo.coefficient + i * A, sizeof(double) * A, cudaMemcpyDeviceToDevice, ctx->stream);
      ++k;
    }
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, "copy failed") != 0;
  }
  dfree(ctx, mo.coefficient);
  mo.coefficient = c;
  mo.mo_num = kept;
  return qmckl_finalize_mo_basis_device(context) != QMCKL_SUCCESS_DEVICE;
}

// ---------------------------------------------------------------- provides
static qmckl_exit_code_device compute_mo_vgl(Ctx* ctx, qmckl_context_device context, double* dst) {
  const char* fn = "qmckl_provide_mo_basis_mo_vgl_device";
  if (!ctx->ao_basis.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_ao_basis", nullptr);
  // the split-BF16 form takes the AO operand straight from the fused AO kernel
  if (ctx->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE) return provide_mo_split(ctx, context, dst, false);
  qmckl_exit_code_device rc = qmckl_provide_ao_basis_ao_vgl_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_ao_basis", nullptr);
  launch_mo_vgl_fp64(ctx, ctx->ao_basis.ao_vgl, ctx->mo_basis.coefficient_t, ctx->point.num, ctx->ao_basis.ao_num,
                     ctx->mo_basis.mo_num, dst);
  return finish(ctx, context, fn);
}

static qmckl_exit_code_device compute_mo_value(Ctx* ctx, qmckl_context_device context, double* dst) {
  const char* fn = "qmckl_provide_mo_basis_mo_value_device";
  MoBasisData& mo = ctx->mo_basis;
  if (mo.mo_vgl_date == ctx->point.date && mo.mo_vgl) {
    // src/qmckl_mo.cpp:232-260: mo_vgl is current, copy its value rows
    launch_strided_copy(ctx, mo.mo_vgl, 5 * mo.mo_num, dst, mo.mo_num, ctx->point.num, mo.mo_num);
    return finish(ctx, context, fn);
  }
  qmckl_exit_code_device rc = qmckl_provide_ao_basis_ao_value_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_ao_basis_ao_value_device", nullptr);
  if (ctx->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE) return provide_mo_split(ctx, context, dst, true);
  launch_mo_value_fp64(ctx, ctx->ao_basis.ao_value, mo.coefficient_t, ctx->point.num, ctx->ao_basis.ao_num, mo.mo_num,
                       dst);
  return finish(ctx, context, fn);
}

qmckl_exit_code_device qmckl_provide_mo_basis_mo_vgl_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_provide_mo_basis_mo_vgl_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_provide_mo_basis_mo_vgl_device";
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  MoBasisData& mo = ctx->mo_basis;
  if (!mo.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  if (ctx->point.date > mo.mo_vgl_date) {
    if (!ensure(ctx, &mo.mo_vgl, &mo.mo_vgl_cap, sizeof(double) * 5 * mo.mo_num * ctx->point.num))
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_mo_basis_mo_vgl", nullptr);
    qmckl_exit_code_device rc = compute_mo_vgl(ctx, context, mo.mo_vgl);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    mo.mo_vgl_date = ctx->date;
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_provide_mo_basis_mo_value_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_provide_mo_basis_mo_value_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_provide_mo_basis_mo_value_device";
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  MoBasisData& mo = ctx->mo_basis;
  if (!mo.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  if (ctx->point.date > mo.mo_value_date) {
    if (!ensure(ctx, &mo.mo_value, &mo.mo_value_cap, sizeof(double) * mo.mo_num * ctx->point.num))
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_mo_basis_mo_value", nullptr);
    qmckl_exit_code_device rc = compute_mo_value(ctx, context, mo.mo_value);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    mo.mo_value_date = ctx->date;
  }
  return QMCKL_SUCCESS_DEVICE;
}

// Point ranges of the host-buffer path: by default sized by the contraction's waves (each range's
// tiles fill one wave of the SMs; chunks = 0), so that no range's contraction ends with idle SMs.
// All ranges are put in processing order by one pass before the first range computes, and small
// ranges take the AO kernel's finest tasks (pieces of nuclei), so the per-range cost is small and
// many ranges pay: the first range, whose compute the link waits for, stays short. Measured end
// to end on 40,960 points (set_point from and mo_vgl into page-locked host memory, ms per step; the
// link alone needs 2.55 ms) with equal ranges: 2.91 / 2.89 / 2.86 / 2.85 / 2.84 / 2.84 / 2.84 /
// 3.15 / 2.79 ms with 8 / 10 / 11 / 12 / 13 / 14 / 16 / 21 / 22 ranges: 22 ranges of 1888 points
// make 148 tiles each (one wave of 152 SMs), 21 of 1952 points 154 (a wave and 2 tiles).
constexpr int kHostChunks = 0;
constexpr double kHostChunkRatio = 1.0;

// QMCKL_GB300_HOST_CHUNKS="<ranges>[,<ratio>]" overrides the plan (for measurements).
static void host_chunk_plan_override(int* chunks, double* ratio) {
  const char* v = getenv("QMCKL_GB300_HOST_CHUNKS");
  if (!v || !*v) return;
  int n = 0;
  double r = 0.0;
  const int got = sscanf(v, "%d,%lf", &n, &r);
  if (got >= 1 && n >= 1 && n <= kMaxHostChunks) *chunks = n;
  if (got == 2 && r >= 0.25 && r <= 4.0) *ratio = r;
}

// True for host memory (page-locked or not): a destination the device reaches over the host link.
static bool host_memory(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeUnregistered;
}

qmckl_exit_code_device qmckl_get_mo_basis_mo_vgl_device(qmckl_context_device context, double* const mo_vgl,
                                                        const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_mo_basis_mo_vgl_device");
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  MoBasisData& mo = ctx->mo_basis;
  // split-BF16 results for a host buffer on a large point set: compute in chunks and overlap the
  // device-to-host copy of each chunk with the next chunk's compute
  if (mo.provided && ctx->ao_basis.provided && ctx->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE &&
      ctx->point.date > mo.mo_vgl_date && ctx->point.num >= 16384 && mo_vgl &&
      size_max >= 5 * ctx->point.num * mo.mo_num && ensure_device(ctx) && host_memory(mo_vgl)) {
    // point ranges sized by the contraction's waves (QMCKL_GB300_HOST_CHUNKS="<ranges>,<ratio>"
    // overrides the plan); the device-to-host link (~193 GB/s) needs 2.54 ms for the medium
    // workload's 491 MB of mo_vgl, the computation 1.53 ms
    int chunks = kHostChunks;
    double ratio = kHostChunkRatio;
    host_chunk_plan_override(&chunks, &ratio);
    qmckl_exit_code_device rc = split_mo_vgl_to_host(ctx, context, mo_vgl, chunks, ratio);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    mo.mo_vgl_date = ctx->date;
    return QMCKL_SUCCESS_DEVICE;
  }
  qmckl_exit_code_device rc = qmckl_provide_mo_basis_mo_vgl_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  const int64_t sze = 5 * ctx->point.num * ctx->mo_basis.mo_num;
  if (size_max < sze)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_mo_basis_mo_vgl", "input array too small");
  if (!mo_vgl) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_mo_basis_mo_vgl", "NULL pointer");
  return copy(ctx, context, mo_vgl, ctx->mo_basis.mo_vgl, sizeof(double) * (size_t)sze, "qmckl_get_mo_basis_mo_vgl", true);
}

qmckl_exit_code_device qmckl_get_mo_basis_mo_vgl_inplace_device(qmckl_context_device context, double* const mo_vgl,
                                                                const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_mo_basis_mo_vgl_inplace_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_get_mo_basis_mo_vgl_device";
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  const int64_t sze = 5 * ctx->mo_basis.mo_num * ctx->point.num;
  if (size_max < sze) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "input array too small");
  qmckl_exit_code_device rc = qmckl_context_touch_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!ctx->mo_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_provide_mo_basis_mo_vgl_device", nullptr);
  if (!mo_vgl) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (gpu_accessible(mo_vgl)) return compute_mo_vgl(ctx, context, mo_vgl);
  rc = qmckl_provide_mo_basis_mo_vgl_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  return copy(ctx, context, mo_vgl, ctx->mo_basis.mo_vgl, sizeof(double) * (size_t)sze, fn, true);
}

qmckl_exit_code_device qmckl_get_mo_basis_mo_value_device(qmckl_context_device context, double* const mo_value,
                                                          const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_mo_basis_mo_value_device");
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  qmckl_exit_code_device rc = qmckl_provide_mo_basis_mo_value_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  const int64_t sze = ctx->point.num * ctx->mo_basis.mo_num;
  if (size_max < sze)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_mo_basis_mo_value", "input array too small");
  if (!mo_value) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_mo_basis_mo_value", "NULL pointer");
  return copy(ctx, context, mo_value, ctx->mo_basis.mo_value, sizeof(double) * (size_t)sze,
              "qmckl_get_mo_basis_mo_value", true);
}

qmckl_exit_code_device qmckl_get_mo_basis_mo_value_inplace_device(qmckl_context_device context,
                                                                  double* const mo_value, const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_mo_basis_mo_value_inplace_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_get_mo_basis_mo_value_device";
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  const int64_t sze = ctx->mo_basis.mo_num * ctx->point.num;
  if (size_max < sze) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "input array too small");
  qmckl_exit_code_device rc = qmckl_context_touch_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!ctx->mo_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_provide_mo_basis_mo_value_device", nullptr);
  if (!mo_value) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (gpu_accessible(mo_value)) return compute_mo_value(ctx, context, mo_value);
  rc = qmckl_provide_mo_basis_mo_value_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  return copy(ctx, context, mo_value, ctx->mo_basis.mo_value, sizeof(double) * (size_t)sze, fn, true);
}

// ---------------------------------------------------------------- precision mode
qmckl_exit_code_device qmckl_set_precision_mode_device(qmckl_context_device context, int32_t mode) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (mode != QMCKL_PRECISION_FP64_DEVICE && mode != QMCKL_PRECISION_SPLIT_BF16_DEVICE)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_precision_mode_device",
                                 "mode must be QMCKL_PRECISION_FP64_DEVICE or QMCKL_PRECISION_SPLIT_BF16_DEVICE");
  if (ctx->precision != mode) {
    ctx->precision = mode;
    ctx->mo_basis.mo_vgl_date = ctx->mo_basis.mo_value_date = 0;
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_precision_mode_device(qmckl_context_device context, int32_t* mode) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!mode) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_precision_mode_device", "NULL pointer");
  *mode = ctx->precision;
  return QMCKL_SUCCESS_DEVICE;
}

}  // extern "C"
