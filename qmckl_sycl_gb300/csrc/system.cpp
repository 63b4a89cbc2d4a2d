// Points, nuclei and electrons: setters and getters with the reference's argument checks
// and exit codes (src/qmckl_point.cpp, src/qmckl_nucleus.cpp:359-663,
// src/qmckl_electron.cpp:8-190 of qmckl_sycl). Coordinates are kept structure-of-arrays,
// [3][num], as the reference stores them, so the kernels read each axis coalesced.
#include <cstring>

#include "internal.hpp"

using namespace qg;

namespace {

bool referenced_by_walkers(Ctx* ctx, double* p) {
  return p && (ctx->electron.walker.point.coord == p || ctx->electron.walker_old.point.coord == p);
}

// in[num][3] (device or host memory) -> out[3][num] on the device.
qmckl_exit_code_device aos_to_soa(Ctx* ctx, qmckl_context_device c, const double* in, int64_t num, double* out,
                                  const char* fn) {
  if (num == 0) return QMCKL_SUCCESS_DEVICE;
  const double* src = in;
  if (!gpu_accessible(in)) {
    double* st = static_cast<double*>(staging(ctx, sizeof(double) * 3 * num));
    if (!st) return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
    qmckl_exit_code_device rc = copy(ctx, c, st, in, sizeof(double) * 3 * num, fn);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    src = st;
  }
  launch_point_aos_to_soa(ctx, src, num, out);
  return finish(ctx, c, fn);
}

// in[3][num] on the device -> out[num][3] (device or host memory).
qmckl_exit_code_device soa_to_aos(Ctx* ctx, qmckl_context_device c, const double* in, int64_t num, double* out,
                                  const char* fn) {
  if (num == 0) return QMCKL_SUCCESS_DEVICE;
  if (gpu_accessible(out)) {
    launch_transpose(ctx, in, 3, num, out);
    return finish(ctx, c, fn);
  }
  double* st = static_cast<double*>(staging(ctx, sizeof(double) * 3 * num));
  if (!st) return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  launch_transpose(ctx, in, 3, num, st);
  qmckl_exit_code_device rc = finish(ctx, c, fn);
  if (rc == QMCKL_SUCCESS_DEVICE) rc = copy(ctx, c, out, st, sizeof(double) * 3 * num, fn, true);
  return rc;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- points
qmckl_exit_code_device qmckl_set_point_device(qmckl_context_device context, char transp, int64_t num, double* coord,
                                              int64_t size_max) {
  QG_NVTX_RANGE("qmckl_set_point_device");
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (size_max < 3 * num)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_set_point_device", "Array too small");
  if (transp != 'N' && transp != 'T')
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_point_device",
                                 "transp should be 'N' or 'T'");
  if (coord == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_set_point_device",
                                 "coord is a NULL pointer");
  if (num < 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_set_point_device", "num < 0");
  Ctx* ctx = ctx_of(context);
  if (!ensure_device(ctx))
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_set_point_device", "no usable CUDA device");
  if (num != ctx->point.num || (num > 0 && !ctx->point.coord)) {
    // src/qmckl_point.cpp:96-109; a buffer still referenced by the other walker set is kept
    if (ctx->point.coord && !referenced_by_walkers(ctx, ctx->point.coord)) dfree(ctx, ctx->point.coord);
    ctx->point.coord = nullptr;
    if (num > 0) {
      ctx->point.coord = static_cast<double*>(dalloc(ctx, sizeof(double) * 3 * num));
      if (!ctx->point.coord)
        return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_set_point", nullptr);
    }
  }
  ctx->point.num = num;
  qmckl_exit_code_device rc;
  if (transp == 'T')
    rc = copy(ctx, context, ctx->point.coord, coord, sizeof(double) * 3 * num, "qmckl_set_point_device");
  else
    rc = aos_to_soa(ctx, context, coord, num, ctx->point.coord, "qmckl_set_point_device");
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  return qmckl_context_touch_device(context);
}

qmckl_exit_code_device qmckl_get_point_device(const qmckl_context_device context, const char transp,
                                              double* const coord, const int64_t size_max) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (coord == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_point_coord",
                                 "coord is a null pointer");
  Ctx* ctx = ctx_of(context);
  const int64_t num = ctx->point.num;
  if (num == 0) return QMCKL_NOT_PROVIDED_DEVICE;
  if (size_max < 3 * num)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_point_coord_device",
                                 "size_max too small");
  if (transp == 'N') return soa_to_aos(ctx, context, ctx->point.coord, num, coord, "qmckl_get_point_device");
  return copy(ctx, context, coord, ctx->point.coord, sizeof(double) * 3 * num, "qmckl_get_point_device", true);
}

// ---------------------------------------------------------------- nucleus
bool qmckl_nucleus_provided_device(qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return false;
  return ctx_of(context)->nucleus.provided;
}

qmckl_exit_code_device qmckl_get_nucleus_num_device(qmckl_context_device context, int64_t* num) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (num == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_nucleus_num", "num is a null pointer");
  Ctx* ctx = ctx_of(context);
  if (ctx->nucleus.uninitialized & 1) {
    *num = 0;
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_get_nucleus_num",
                                 "nucleus data is not provided");
  }
  *num = ctx->nucleus.num;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_set_nucleus_num_device(qmckl_context_device context, int64_t num) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  const int32_t mask = 1 << 0;
  if (!(ctx->nucleus.uninitialized & mask))
    return qmckl_failwith_device(context, QMCKL_ALREADY_SET_DEVICE, "qmckl_set_nucleus_*", nullptr);
  if (num <= 0) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_nucleus_num", "num <= 0");
  ctx->nucleus.num = num;
  ctx->nucleus.uninitialized &= ~mask;
  ctx->nucleus.provided = ctx->nucleus.uninitialized == 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_set_nucleus_coord_device(qmckl_context_device context, char transp, double* coord,
                                                      int64_t size_max) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  const int32_t mask = 1 << 2;
  if (!(ctx->nucleus.uninitialized & mask))
    return qmckl_failwith_device(context, QMCKL_ALREADY_SET_DEVICE, "qmckl_set_nucleus_*", nullptr);
  const int64_t nucl_num = ctx->nucleus.num;
  if (nucl_num <= 0)
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_set_nucleus_coord", "nucl_num is not set");
  if (size_max < 3 * nucl_num)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_set_nucleus_coord", "Array too small");
  if (coord == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_set_nucleus_coord", "NULL pointer");
  if (!ensure_device(ctx))
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_set_nucleus_coord", "no usable CUDA device");
  if (!ctx->nucleus.coord) {
    ctx->nucleus.coord = static_cast<double*>(dalloc(ctx, sizeof(double) * 3 * nucl_num));
    if (!ctx->nucleus.coord)
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_set_nucleus_coord", nullptr);
  }
  // src/qmckl_nucleus.cpp:589-602: 'N' is [num][3] and is transposed; anything else is [3][num]
  qmckl_exit_code_device rc =
      transp == 'N' ? aos_to_soa(ctx, context, coord, nucl_num, ctx->nucleus.coord, "qmckl_set_nucleus_coord")
                    : copy(ctx, context, ctx->nucleus.coord, coord, sizeof(double) * 3 * nucl_num,
                           "qmckl_set_nucleus_coord", true);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  ctx->ao_basis.tables.valid = false;  // the kernel tables embed nucleus coordinates
  ctx->nucleus.uninitialized &= ~mask;
  ctx->nucleus.provided = ctx->nucleus.uninitialized == 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_set_nucleus_charge_device(qmckl_context_device context, double* charge,
                                                       int64_t size_max) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (charge == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_nucleus_charge_device",
                                 "charge is a null pointer");
  int64_t num = 0;
  qmckl_exit_code_device rc = qmckl_get_nucleus_num_device(context, &num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (num > size_max)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_set_nucleus_charge_device",
                                 "Array too small");
  if (!ensure_device(ctx))
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_set_nucleus_charge_device", "no device");
  if (!ctx->nucleus.charge) {
    ctx->nucleus.charge = static_cast<double*>(dalloc(ctx, sizeof(double) * num));
    if (!ctx->nucleus.charge)
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_set_nucleus_charge_device",
                                   nullptr);
  }
  rc = copy(ctx, context, ctx->nucleus.charge, charge, sizeof(double) * num, "qmckl_set_nucleus_charge_device", true);
  if (rc != QMCKL_SUCCESS_DEVICE)
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_set_nucleus_charge_device",
                                 "Error in vector->double* conversion");
  ctx->nucleus.uninitialized &= ~(1 << 1);
  ctx->nucleus.provided = ctx->nucleus.uninitialized == 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_nucleus_coord_device(const qmckl_context_device context, const char transp,
                                                      double* const coord, const int64_t size_max) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (transp != 'N' && transp != 'T')
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_nucleus_coord_device",
                                 "transp should be 'N' or 'T'");
  if (coord == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_nucleus_coord_device",
                                 "coord is a null pointer");
  Ctx* ctx = ctx_of(context);
  if (ctx->nucleus.uninitialized & (1 << 2))
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_get_nucleus_coord_device",
                                 "nucleus data is not provided");
  const int64_t n = ctx->nucleus.num;
  if (size_max < 3 * n)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_get_nucleus_coord_device",
                                 "Array too small");
  if (transp == 'N') return soa_to_aos(ctx, context, ctx->nucleus.coord, n, coord, "qmckl_get_nucleus_coord_device");
  return copy(ctx, context, coord, ctx->nucleus.coord, sizeof(double) * 3 * n, "qmckl_get_nucleus_coord_device", true);
}

qmckl_exit_code_device qmckl_get_nucleus_charge_device(const qmckl_context_device context, double* const charge,
                                                       const int64_t size_max) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (charge == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_nucleus_charge",
                                 "charge is a null pointer");
  Ctx* ctx = ctx_of(context);
  if (ctx->nucleus.uninitialized & (1 << 1))
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_get_nucleus_charge_device",
                                 "nucleus data is not provided");
  if (ctx->nucleus.num > size_max)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_nucleus_charge", "Array too small");
  return copy(ctx, context, charge, ctx->nucleus.charge, sizeof(double) * ctx->nucleus.num,
              "qmckl_get_nucleus_charge_device", true);
}

// ---------------------------------------------------------------- electrons
bool qmckl_electron_provided_device(qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return false;
  return ctx_of(context)->electron.provided;
}

qmckl_exit_code_device qmckl_set_electron_num_device(qmckl_context_device context, int64_t up_num, int64_t down_num) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  const int32_t mask = 1 << 0;
  if (!(ctx->electron.uninitialized & mask))
    return qmckl_failwith_device(context, QMCKL_ALREADY_SET_DEVICE, "qmckl_set_electron_*", nullptr);
  if (up_num <= 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_electron_num_device", "up_num <= 0");
  if (down_num < 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_set_electron_num_device",
                                 "down_num < 0");
  ctx->electron.up_num = up_num;
  ctx->electron.down_num = down_num;
  ctx->electron.num = up_num + down_num;
  ctx->electron.uninitialized &= ~mask;
  ctx->electron.provided = ctx->electron.uninitialized == 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_set_electron_coord_device(qmckl_context_device context, char transp, int64_t walk_num,
                                                       double* coord, int64_t size_max) {
  QG_NVTX_RANGE("qmckl_set_electron_coord_device");
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  const int64_t elec_num = ctx->electron.num;
  if (elec_num == 0)
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_set_electron_coord_device",
                                 "elec_num is not set");
  // src/qmckl_electron.cpp:74-87: swap the walker sets, then set the points
  WalkerData tmp = ctx->electron.walker_old;
  ctx->electron.walker_old = ctx->electron.walker;
  ctx->electron.walker = tmp;
  ctx->point = ctx->electron.walker.point;
  qmckl_exit_code_device rc = qmckl_set_point_device(context, transp, walk_num * elec_num, coord, size_max);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  ctx->electron.walker.num = walk_num;
  ctx->electron.walker.point = ctx->point;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_electron_num_device(const qmckl_context_device context, int64_t* const num) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (num == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_electron_num", "num is a null pointer");
  Ctx* ctx = ctx_of(context);
  if (ctx->electron.uninitialized & 1) return QMCKL_NOT_PROVIDED_DEVICE;
  *num = ctx->electron.num;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_electron_coord_device(const qmckl_context_device context, const char transp,
                                                       double* const coord, const int64_t size_max) {
  if (transp != 'N' && transp != 'T')
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_electron_coord_device",
                                 "transp should be 'N' or 'T'");
  if (coord == nullptr)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_electron_coord_device",
                                 "coord is a null pointer");
  if (size_max <= 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_get_electron_coord_device",
                                 "size_max should be > 0");
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (!ctx->electron.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_get_electron_coord_device", nullptr);
  return qmckl_get_point_device(context, transp, coord, size_max);
}

}  // extern "C"
