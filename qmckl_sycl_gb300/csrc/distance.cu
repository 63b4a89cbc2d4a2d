// Electron-nucleus and electron-electron distances (reference: src/qmckl_electron.cpp:192-552 of
// qmckl_sycl). The reference's distance kernel lets every work-item take square roots of a whole
// column of C, racing with the work-items that are still writing it (:504-546); here each entry is
// formed once, sqrt((x*x + y*y) + z*z) with the reference's host rounding (no fused multiply-add),
// one thread per entry, the ee distances of all walkers in one launch.
#include <cstdint>

#include "internal.hpp"

namespace qg {
namespace {

// Coordinate d of point i of a matrix in 'N' ([i][3], leading dimension ld) or 'T' ([3][ld]) layout.
__device__ __forceinline__ double coord_of(const double* __restrict__ M, bool t, int64_t ld, int64_t i, int d) {
  return t ? M[i + d * ld] : M[d + i * ld];
}

// C[w][i + j * ldc] = |A_i - B_j| for walker w (A, B offset by w * a_step / b_step points); one
// thread per entry, entries numbered i fastest.
__global__ void distance_kernel(const double* __restrict__ A, bool ta, int64_t lda, int64_t a_step,
                                const double* __restrict__ B, bool tb, int64_t ldb, int64_t b_step, int64_t m,
                                int64_t n, int64_t total, double* __restrict__ C, int64_t ldc, int64_t c_step) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total) return;
  const int64_t i = e % m;
  const int64_t j = (e / m) % n;
  const int64_t w = e / (m * n);
  const double x = __dsub_rn(coord_of(A, ta, lda, w * a_step + i, 0), coord_of(B, tb, ldb, w * b_step + j, 0));
  const double y = __dsub_rn(coord_of(A, ta, lda, w * a_step + i, 1), coord_of(B, tb, ldb, w * b_step + j, 1));
  const double z = __dsub_rn(coord_of(A, ta, lda, w * a_step + i, 2), coord_of(B, tb, ldb, w * b_step + j, 2));
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
  if (QG_STORE_OK(kSiteDistance, w * c_step + i + j * ldc, (total / (m * n) - 1) * c_step + (n - 1) * ldc + m))
    C[w * c_step + i + j * ldc] = __dsqrt_rn(r2);
}

// The reference's argument checks (src/qmckl_electron.cpp:380-488), with lda checked against transa
// and ldb against transb.
qmckl_exit_code_device check_distance_args(char transa, char transb, int64_t m, int64_t n, int64_t lda, int64_t ldb,
                                           int64_t ldc, bool* ta, bool* tb) {
  if (m <= 0) return QMCKL_INVALID_ARG_4_DEVICE;
  if (n <= 0) return QMCKL_INVALID_ARG_5_DEVICE;
  const bool an = transa == 'N' || transa == 'n', at = transa == 'T' || transa == 't';
  const bool bn = transb == 'N' || transb == 'n', bt = transb == 'T' || transb == 't';
  if (!(an || at) || !(bn || bt)) return QMCKL_INVALID_ARG_1_DEVICE;
  if ((an && lda < 3) || (at && lda < m)) return QMCKL_INVALID_ARG_7_DEVICE;
  if ((bn && ldb < 3) || (bt && ldb < n)) return QMCKL_INVALID_ARG_9_DEVICE;
  if (ldc < m) return QMCKL_INVALID_ARG_11_DEVICE;
  *ta = at;
  *tb = bt;
  return QMCKL_SUCCESS_DEVICE;
}

cudaError_t launch_distance(Ctx* ctx, const double* A, bool ta, int64_t lda, int64_t a_step, const double* B, bool tb,
                            int64_t ldb, int64_t b_step, int64_t m, int64_t n, double* C, int64_t ldc, int64_t c_step,
                            int64_t walkers) {
  const int64_t total = m * n * walkers;
  if (total <= 0) return cudaSuccess;
  LaunchScope scope(ctx, "distance");
  distance_kernel<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(A, ta, lda, a_step, B, tb, ldb, b_step, m,
                                                                            n, total, C, ldc, c_step);
  return cudaGetLastError();
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

qmckl_exit_code_device qmckl_distance_device(const qmckl_context_device context, const char transa, const char transb,
                                             const int64_t m, const int64_t n, const double* A, const int64_t lda,
                                             const double* B, const int64_t ldb, double* const C, const int64_t ldc) {
  QG_NVTX_RANGE("qmckl_distance_device");
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  bool ta = false, tb = false;
  qmckl_exit_code_device rc = check_distance_args(transa, transb, m, n, lda, ldb, ldc, &ta, &tb);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!A || !B || !C) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_6_DEVICE, "qmckl_distance_device", "NULL pointer");
  Ctx* ctx = ctx_of(context);
  if (!ensure_device(ctx)) return fail(context, QMCKL_FAILURE_DEVICE, "qmckl_distance_device", "no usable CUDA device");
  if (launch_distance(ctx, A, ta, lda, 0, B, tb, ldb, 0, m, n, C, ldc, 0, 1) != cudaSuccess) {
    cudaGetLastError();
    return fail(context, QMCKL_FAILURE_DEVICE, "qmckl_distance_device", "launch failed");
  }
  return finish(ctx, context, "qmckl_distance_device");
}

qmckl_exit_code_device qmckl_compute_en_distance_device(const qmckl_context_device context, const int64_t point_num,
                                                        const int64_t nucl_num, const double* elec_coord,
                                                        const double* nucl_coord, double* const en_distance) {
  QG_NVTX_RANGE("qmckl_compute_en_distance_device");
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (point_num <= 0) return QMCKL_INVALID_ARG_2_DEVICE;
  if (nucl_num <= 0) return QMCKL_INVALID_ARG_3_DEVICE;
  // src/qmckl_electron.cpp:326-328: distance('T', 'T', nucl_num, point_num, nucl_coord, nucl_num,
  // elec_coord, point_num, en_distance, nucl_num)
  return qmckl_distance_device(context, 'T', 'T', nucl_num, point_num, nucl_coord, nucl_num, elec_coord, point_num,
                               en_distance, nucl_num);
}

qmckl_exit_code_device qmckl_compute_ee_distance_device(const qmckl_context_device context, const int64_t elec_num,
                                                        const int64_t walk_num, const double* coord,
                                                        double* const ee_distance) {
  QG_NVTX_RANGE("qmckl_compute_ee_distance_device");
  const char* fn = "qmckl_compute_ee_distance_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (elec_num <= 0) return QMCKL_INVALID_ARG_2_DEVICE;
  if (walk_num <= 0) return QMCKL_INVALID_ARG_3_DEVICE;
  if (!coord || !ee_distance) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, fn, "NULL pointer");
  Ctx* ctx = ctx_of(context);
  if (!ensure_device(ctx)) return fail(context, QMCKL_FAILURE_DEVICE, fn, "no usable CUDA device");
  // src/qmckl_electron.cpp:359-367: per walker k, distance('T', 'T', elec_num, elec_num,
  // coord + k * elec_num, elec_num * walk_num, (same), ee_distance + k * elec_num^2, elec_num)
  const int64_t ld = elec_num * walk_num;
  if (launch_distance(ctx, coord, true, ld, elec_num, coord, true, ld, elec_num, elec_num, elec_num, ee_distance,
                      elec_num, elec_num * elec_num, walk_num) != cudaSuccess) {
    cudaGetLastError();
    return fail(context, QMCKL_FAILURE_DEVICE, fn, "launch failed");
  }
  return finish(ctx, context, fn);
}

qmckl_exit_code_device qmckl_provide_en_distance_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_provide_en_distance_device");
  const char* fn = "qmckl_provide_en_distance_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (!ctx->nucleus.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  ElectronData& el = ctx->electron;
  if (ctx->point.date > el.en_distance_date || !el.en_distance) {
    const int64_t P = ctx->point.num, N = ctx->nucleus.num;
    if (P <= 0) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, "no points");
    if (!ensure(ctx, &el.en_distance, &el.en_distance_cap, sizeof(double) * P * N))
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_en_distance_device", nullptr);
    qmckl_exit_code_device rc =
        qmckl_compute_en_distance_device(context, P, N, ctx->point.coord, ctx->nucleus.coord, el.en_distance);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    el.en_distance_date = ctx->date;
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_provide_ee_distance_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_provide_ee_distance_device");
  const char* fn = "qmckl_provide_ee_distance_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  ElectronData& el = ctx->electron;
  if (!el.provided || el.walker.num <= 0)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, "electron coordinates are not set");
  if (ctx->point.date > el.ee_distance_date || !el.ee_distance) {
    const int64_t E = el.num, W = el.walker.num;
    if (ctx->point.num != E * W)
      return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, "points are not the electrons of the walkers");
    if (!ensure(ctx, &el.ee_distance, &el.ee_distance_cap, sizeof(double) * E * E * W))
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_ee_distance_device", nullptr);
    qmckl_exit_code_device rc = qmckl_compute_ee_distance_device(context, E, W, ctx->point.coord, el.ee_distance);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    el.ee_distance_date = ctx->date;
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_electron_en_distance_device(qmckl_context_device context, double* distance,
                                                             int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_electron_en_distance_device");
  const char* fn = "qmckl_get_electron_en_distance_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!distance) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  qmckl_exit_code_device rc = qmckl_provide_en_distance_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  Ctx* ctx = ctx_of(context);
  const int64_t sze = ctx->point.num * ctx->nucleus.num;
  if (size_max < sze) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "array too small");
  return copy(ctx, context, distance, ctx->electron.en_distance, sizeof(double) * (size_t)sze, fn, true);
}

qmckl_exit_code_device qmckl_get_electron_ee_distance_device(qmckl_context_device context, double* distance,
                                                             int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_electron_ee_distance_device");
  const char* fn = "qmckl_get_electron_ee_distance_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!distance) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  qmckl_exit_code_device rc = qmckl_provide_ee_distance_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  Ctx* ctx = ctx_of(context);
  const int64_t sze = ctx->electron.num * ctx->electron.num * ctx->electron.walker.num;
  if (size_max < sze) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "array too small");
  return copy(ctx, context, distance, ctx->electron.ee_distance, sizeof(double) * (size_t)sze, fn, true);
}

}  // extern "C"
