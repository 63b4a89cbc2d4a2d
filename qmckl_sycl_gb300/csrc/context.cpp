// Context, error and memory runtime of the GB300 QMCkl library.
//
// Mirrors the reference's runtime layer (src/qmckl_context.cpp, src/qmckl_basic_functions.cpp,
// src/qmckl_memory.cpp, src/qmckl_blas.cpp): an opaque int64 handle validated by a tag, a
// recursive lock around the error record and the allocation registry, date-stamped caches,
// and a registry that frees every device allocation at destroy. One CUDA stream per
// context replaces the sycl::queue; it is created on first use, so a context (and all of
// its host-side argument checks) can be exercised on a machine without a GPU.
#include <cstdio>
#include <cstring>
#include <new>

#include "internal.hpp"

using namespace qg;

namespace qg {

static bool activate(Ctx* ctx) {
  if (cudaSetDevice(ctx->device_id) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (!ctx->stream) {
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    ctx->stream = s;
    ctx->own_stream = true;
  }
  return true;
}

qmckl_exit_code_device fail(qmckl_context_device c, qmckl_exit_code_device code, const char* fn, const char* msg) {
  return qmckl_failwith_device(c, code, fn, msg);
}

void* dalloc(Ctx* ctx, size_t bytes) { return qmckl_malloc_device(reinterpret_cast<qmckl_context_device>(ctx), bytes); }

void dfree(Ctx* ctx, void* p) {
  if (p) qmckl_free_device(reinterpret_cast<qmckl_context_device>(ctx), p);
}

bool ensure_raw(Ctx* ctx, void** buf, size_t* cap, size_t bytes) {
  if (*buf && *cap >= bytes) return true;
  if (*buf) {
    dfree(ctx, *buf);
    *buf = nullptr;
    *cap = 0;
  }
  void* p = dalloc(ctx, bytes ? bytes : 8);
  if (!p) return false;
  *buf = p;
  *cap = bytes;
  return true;
}

bool ensure(Ctx* ctx, double** buf, size_t* cap, size_t bytes) {
  void* b = *buf;
  bool ok = ensure_raw(ctx, &b, cap, bytes);
  *buf = static_cast<double*>(b);
  return ok;
}

static void harvest(Ctx* ctx, bool wait) {
  size_t keep = 0;
  for (size_t i = 0; i < ctx->pending.size(); ++i) {
    PendingEvent& e = ctx->pending[i];
    cudaError_t q = wait ? cudaEventSynchronize(e.stop) : cudaEventQuery(e.stop);
    if (q == cudaSuccess) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, e.start, e.stop) == cudaSuccess) ctx->stats[e.slot].total_ms += ms;
      ctx->event_pool.push_back(e.start);
      ctx->event_pool.push_back(e.stop);
    } else {
      if (q != cudaErrorNotReady) cudaGetLastError();
      ctx->pending[keep++] = e;
    }
  }
  ctx->pending.resize(keep);
}

static cudaEvent_t pooled_event(Ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

LaunchScope::LaunchScope(Ctx* c, const char* name) : ctx(c), slot(-1) {
  ctx->launch_count += 1;
  int s = -1;
  for (size_t i = 0; i < ctx->stats.size(); ++i)
    if (ctx->stats[i].name == name) s = (int)i;
  if (s < 0) {
    ctx->stats.push_back(KernelStat{name, 0, 0.0});
    s = (int)ctx->stats.size() - 1;
  }
  slot = s;
  ctx->stats[s].launches += 1;
  if (ctx->profiling) {
    start = pooled_event(ctx);
    stop = pooled_event(ctx);
    if (start) cudaEventRecord(start, ctx->stream);
  }
}

LaunchScope::~LaunchScope() {
  if (ctx->profiling && start && stop) {
    cudaEventRecord(stop, ctx->stream);
    ctx->pending.push_back(PendingEvent{slot, start, stop});
    if (ctx->pending.size() > 4096) harvest(ctx, true);
  }
}

qmckl_exit_code_device finish(Ctx* ctx, qmckl_context_device c, const char* fn) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !ctx->async) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof msg, "CUDA error: %s", cudaGetErrorString(e));
    return fail(c, QMCKL_FAILURE_DEVICE, fn, msg);
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device copy(Ctx* ctx, qmckl_context_device c, void* dst, const void* src, size_t bytes,
                            const char* fn, bool force_sync) {
  if (bytes == 0) return QMCKL_SUCCESS_DEVICE;
  if (!activate(ctx)) return fail(c, QMCKL_FAILURE_DEVICE, fn, "no usable CUDA device");
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream);
  if (e == cudaSuccess && (force_sync || !ctx->async)) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    char msg[256];
    snprintf(msg, sizeof msg, "cudaMemcpyAsync failed: %s", cudaGetErrorString(e));
    return fail(c, QMCKL_FAILURE_DEVICE, fn, msg);
  }
  return QMCKL_SUCCESS_DEVICE;
}

bool ensure_device(Ctx* ctx) { return activate(ctx); }

bool gpu_accessible(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeHost;
}

void* staging(Ctx* ctx, size_t bytes) {
  if (!ensure_raw(ctx, &ctx->staging, &ctx->staging_cap, bytes)) return nullptr;
  return ctx->staging;
}

// The bounds-check records of the translation units (bounds-checked build only).
static std::vector<void* (*)()>& bounds_records() {
  static std::vector<void* (*)()> v;
  return v;
}

void register_bounds_record(void* (*address)()) { bounds_records().push_back(address); }

int32_t bounds_check_status(bool reset, int64_t* site, int64_t* index, int64_t* extent) {
#ifndef QMCKL_BOUNDS_CHECK
  (void)reset;
  (void)site;
  (void)index;
  (void)extent;
  return -1;
#else
  struct Rec {
    int hit, site;
    long long index, extent;
  };
  // the records are read once every kernel of every stream (contexts' streams do not
  // synchronise with the legacy stream that cudaMemcpy uses) has finished
  if (cudaDeviceSynchronize() != cudaSuccess) return -2;
  int32_t found = 0;
  for (auto address : bounds_records()) {
    void* p = address();
    if (!p) return -2;
    Rec r{};
    if (cudaMemcpy(&r, p, sizeof r, cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
    if (r.hit && !found) {
      found = 1;
      if (site) *site = r.site;
      if (index) *index = r.index;
      if (extent) *extent = r.extent;
    }
    if (reset && cudaMemset(p, 0, sizeof r) != cudaSuccess) return -2;
  }
  return found;
#endif
}

}  // namespace qg

extern "C" {

// ---------------------------------------------------------------- context
static qmckl_context_device create(int32_t device_id, void* stream) {
  Ctx* ctx = new (std::nothrow) Ctx();
  if (!ctx) return QMCKL_NULL_CONTEXT_DEVICE;
  ctx->device_id = device_id;
  if (stream) {
    ctx->stream = static_cast<cudaStream_t>(stream);
    ctx->own_stream = false;
  }
  // initial masks, src/qmckl_context.cpp:21,37,143 and src/qmckl_ao.cpp:18
  ctx->electron.uninitialized = (1 << 1) - 1;
  ctx->nucleus.uninitialized = (1 << 3) - 1;
  ctx->ao_basis.uninitialized = (1 << 14) - 1;
  ctx->mo_basis.uninitialized = (1 << 2) - 1;
  return reinterpret_cast<qmckl_context_device>(ctx);
}

qmckl_context_device qmckl_context_create_device(int32_t device_id) { return create(device_id, nullptr); }

qmckl_context_device qmckl_context_create_with_stream_device(int32_t device_id, void* cuda_stream) {
  return create(device_id, cuda_stream);
}

qmckl_context_device qmckl_context_check_device(const qmckl_context_device context) {
  if (context == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_NULL_CONTEXT_DEVICE;
  const Ctx* ctx = ctx_of(context);
  if (ctx->tag != kValidTag) return QMCKL_NULL_CONTEXT_DEVICE;
  return context;
}

qmckl_exit_code_device qmckl_context_destroy_device(const qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (ctx->stream) {
    cudaSetDevice(ctx->device_id);
    cudaStreamSynchronize(ctx->stream);
  }
  for (auto& kv : ctx->device_allocs) cudaFree(kv.first);
  ctx->device_allocs.clear();
  for (auto& kv : ctx->host_allocs) free(kv.first);
  ctx->host_allocs.clear();
  for (auto& e : ctx->pending) {
    cudaEventDestroy(e.start);
    cudaEventDestroy(e.stop);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  for (auto e : ctx->chunk_done)
    if (e) cudaEventDestroy(e);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  cudaGetLastError();
  ctx->tag = kInvalidTag;
  delete ctx;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_context_touch_device(const qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE)
    return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_context_touch_device", nullptr);
  Ctx* ctx = ctx_of(context);
  ctx->electron.walker_old = ctx->electron.walker;  // src/qmckl_context.cpp:58
  ctx->date += 1;
  ctx->point.date = ctx->date;
  return QMCKL_SUCCESS_DEVICE;
}

void qmckl_lock_device(qmckl_context_device context) {
  if (context == QMCKL_NULL_CONTEXT_DEVICE) return;
  Ctx* ctx = ctx_of(context);
  ctx->mutex.lock();
  ctx->lock_count += 1;
}

void qmckl_unlock_device(qmckl_context_device context) {
  if (context == QMCKL_NULL_CONTEXT_DEVICE) return;
  Ctx* ctx = ctx_of(context);
  ctx->lock_count -= 1;
  ctx->mutex.unlock();
}

// ---------------------------------------------------------------- errors
const char* qmckl_string_of_error_device(const qmckl_exit_code_device error) {
  switch (error) {
    case QMCKL_SUCCESS_DEVICE: return "Success";
    case QMCKL_INVALID_ARG_1_DEVICE: return "Invalid argument 1";
    case QMCKL_INVALID_ARG_2_DEVICE: return "Invalid argument 2";
    case QMCKL_INVALID_ARG_3_DEVICE: return "Invalid argument 3";
    case QMCKL_INVALID_ARG_4_DEVICE: return "Invalid argument 4";
    case QMCKL_INVALID_ARG_5_DEVICE: return "Invalid argument 5";
    case QMCKL_INVALID_ARG_6_DEVICE: return "Invalid argument 6";
    case QMCKL_INVALID_ARG_7_DEVICE: return "Invalid argument 7";
    case QMCKL_INVALID_ARG_8_DEVICE: return "Invalid argument 8";
    case QMCKL_INVALID_ARG_9_DEVICE: return "Invalid argument 9";
    case QMCKL_INVALID_ARG_10_DEVICE: return "Invalid argument 10";
    case QMCKL_INVALID_ARG_11_DEVICE: return "Invalid argument 11";
    case QMCKL_INVALID_ARG_12_DEVICE: return "Invalid argument 12";
    case QMCKL_INVALID_ARG_13_DEVICE: return "Invalid argument 13";
    case QMCKL_INVALID_ARG_14_DEVICE: return "Invalid argument 14";
    case QMCKL_INVALID_ARG_15_DEVICE: return "Invalid argument 15";
    case QMCKL_INVALID_ARG_16_DEVICE: return "Invalid argument 16";
    case QMCKL_INVALID_ARG_17_DEVICE: return "Invalid argument 17";
    case QMCKL_INVALID_ARG_18_DEVICE: return "Invalid argument 18";
    case QMCKL_INVALID_ARG_19_DEVICE: return "Invalid argument 19";
    case QMCKL_INVALID_ARG_20_DEVICE: return "Invalid argument 20";
    case QMCKL_FAILURE_DEVICE: return "Failure";
    case QMCKL_ERRNO_DEVICE: return "Error (errno)";
    case QMCKL_INVALID_CONTEXT_DEVICE: return "Invalid context";
    case QMCKL_ALLOCATION_FAILED_DEVICE: return "Allocation failed";
    case QMCKL_DEALLOCATION_FAILED_DEVICE: return "De-allocation failed";
    case QMCKL_NOT_PROVIDED_DEVICE: return "Not provided";
    case QMCKL_OUT_OF_BOUNDS_DEVICE: return "Index out of bounds";
    case QMCKL_ALREADY_SET_DEVICE: return "Already set";
    case QMCKL_INVALID_EXIT_CODE_DEVICE: return "Invalid exit code";
    default: break;
  }
  if (error > 0 && error <= 20) return "Invalid argument";
  return "Unknown error";
}

qmckl_exit_code_device qmckl_set_error_device(qmckl_context_device context, const qmckl_exit_code_device exit_code,
                                              const char* function_name, const char* message) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (exit_code <= 0 || exit_code >= QMCKL_INVALID_EXIT_CODE_DEVICE) return QMCKL_INVALID_ARG_2_DEVICE;
  Ctx* ctx = ctx_of(context);
  qmckl_lock_device(context);
  ctx->error.exit_code = exit_code;
  strncpy(ctx->error.function, function_name ? function_name : "", QMCKL_MAX_FUN_LEN_DEVICE - 1);
  ctx->error.function[QMCKL_MAX_FUN_LEN_DEVICE - 1] = 0;
  strncpy(ctx->error.message, message ? message : "", QMCKL_MAX_MSG_LEN_DEVICE - 1);
  ctx->error.message[QMCKL_MAX_MSG_LEN_DEVICE - 1] = 0;
  qmckl_unlock_device(context);
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_failwith_device(qmckl_context_device context, const qmckl_exit_code_device exit_code,
                                             const char* function, const char* message) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  qmckl_set_error_device(context, exit_code, function ? function : "",
                         message ? message : qmckl_string_of_error_device(exit_code));
  return exit_code;
}

qmckl_exit_code_device qmckl_get_error_device(qmckl_context_device context, qmckl_exit_code_device* exit_code,
                                              char* function, int64_t function_size, char* message,
                                              int64_t message_size) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  qmckl_lock_device(context);
  if (exit_code) *exit_code = ctx->error.exit_code;
  if (function && function_size > 0) {
    strncpy(function, ctx->error.function, (size_t)function_size - 1);
    function[function_size - 1] = 0;
  }
  if (message && message_size > 0) {
    strncpy(message, ctx->error.message, (size_t)message_size - 1);
    message[message_size - 1] = 0;
  }
  qmckl_unlock_device(context);
  return QMCKL_SUCCESS_DEVICE;
}

// ---------------------------------------------------------------- memory
void* qmckl_malloc_host(qmckl_context_device context, const qmckl_memory_info_struct_device info) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return nullptr;
  Ctx* ctx = ctx_of(context);
  void* p = calloc(info.size ? info.size : 1, 1);
  if (!p) return nullptr;
  qmckl_lock_device(context);
  ctx->host_allocs[p] = info.size;
  qmckl_unlock_device(context);
  return p;
}

qmckl_exit_code_device qmckl_free_host(qmckl_context_device context, void* const ptr) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE)
    return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_free_host", nullptr);
  if (!ptr) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_free_host", "NULL pointer");
  Ctx* ctx = ctx_of(context);
  qmckl_lock_device(context);
  auto it = ctx->host_allocs.find(ptr);
  if (it == ctx->host_allocs.end()) {
    qmckl_unlock_device(context);
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_free_host",
                                 "Pointer not found in context");
  }
  free(ptr);
  ctx->host_allocs.erase(it);
  qmckl_unlock_device(context);
  return QMCKL_SUCCESS_DEVICE;
}

void* qmckl_malloc_device(qmckl_context_device context, size_t size) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return nullptr;
  Ctx* ctx = ctx_of(context);
  if (!activate(ctx)) return nullptr;
  qmckl_lock_device(context);
  if (ctx->fail_alloc_countdown > 0) {
    ctx->fail_alloc_countdown -= 1;
    if (ctx->fail_alloc_countdown == 0) {
      qmckl_unlock_device(context);
      return nullptr;
    }
  }
  qmckl_unlock_device(context);
  void* p = nullptr;
  if (cudaMalloc(&p, size ? size : 1) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  // The reference's comment promises zeroed memory (src/qmckl_memory.cpp:78); do it.
  if (cudaMemsetAsync(p, 0, size ? size : 1, ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(p);
    return nullptr;
  }
  qmckl_lock_device(context);
  ctx->device_allocs[p] = size;
  qmckl_unlock_device(context);
  return p;
}

qmckl_exit_code_device qmckl_free_device(qmckl_context_device context, void* const ptr) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE)
    return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_free_device", nullptr);
  if (!ptr) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_free_device", "NULL pointer");
  Ctx* ctx = ctx_of(context);
  qmckl_lock_device(context);
  auto it = ctx->device_allocs.find(ptr);
  if (it == ctx->device_allocs.end()) {
    qmckl_unlock_device(context);
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_free_device", "Pointer not found in context");
  }
  ctx->device_allocs.erase(it);
  qmckl_unlock_device(context);
  cudaSetDevice(ctx->device_id);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (cudaFree(ptr) != cudaSuccess) {
    cudaGetLastError();
    return qmckl_failwith_device(context, QMCKL_DEALLOCATION_FAILED_DEVICE, "qmckl_free_device", "cudaFree failed");
  }
  return QMCKL_SUCCESS_DEVICE;
}

static qmckl_exit_code_device memcpy_checked(qmckl_context_device context, void* dest, void* src, size_t size,
                                             const char* fn) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE)
    return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  if (!dest) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL dest pointer");
  if (!src) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "NULL src pointer");
  Ctx* ctx = ctx_of(context);
  qmckl_lock_device(context);
  qmckl_exit_code_device rc = copy(ctx, context, dest, src, size, fn, true);
  qmckl_unlock_device(context);
  return rc;
}

qmckl_exit_code_device qmckl_memcpy_H2D(qmckl_context_device context, void* const dest, void* const src, size_t size) {
  return memcpy_checked(context, dest, src, size, "qmckl_memcpy_H2D");
}
qmckl_exit_code_device qmckl_memcpy_D2H(qmckl_context_device context, void* const dest, void* const src, size_t size) {
  return memcpy_checked(context, dest, src, size, "qmckl_memcpy_D2H");
}
qmckl_exit_code_device qmckl_memcpy_D2D(qmckl_context_device context, void* const dest, void* const src, size_t size) {
  return memcpy_checked(context, dest, src, size, "qmckl_memcpy_D2D");
}

// ---------------------------------------------------------------- containers
qmckl_vector_device qmckl_vector_alloc_device(qmckl_context_device context, const int64_t size) {
  qmckl_vector_device v{nullptr, 0};
  if (size <= 0) return v;
  v.data = static_cast<double*>(qmckl_malloc_device(context, (size_t)size * sizeof(double)));
  v.size = v.data ? size : 0;
  return v;
}

qmckl_exit_code_device qmckl_vector_free_device(qmckl_context_device context, qmckl_vector_device* vector) {
  if (!vector || !vector->data)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_vector_free_device", "NULL vector");
  qmckl_exit_code_device rc = qmckl_free_device(context, vector->data);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  vector->data = nullptr;
  vector->size = 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_vector_of_double_device(const qmckl_context_device context, const double* target,
                                                     const int64_t size_max, qmckl_vector_device* vector_out) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!vector_out || vector_out->size == 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_vector_device_of_double",
                                 "Vector not allocated");
  if (vector_out->size != size_max)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_vector_device_of_double",
                                 "Wrong vector size");
  return copy(ctx_of(context), context, vector_out->data, target, (size_t)size_max * sizeof(double),
              "qmckl_vector_device_of_double", true);
}

qmckl_matrix_device qmckl_matrix_alloc_device(qmckl_context_device context, const int64_t size1, const int64_t size2) {
  qmckl_matrix_device m{nullptr, {0, 0}};
  if (size1 <= 0 || size2 <= 0) return m;
  m.data = static_cast<double*>(qmckl_malloc_device(context, (size_t)(size1 * size2) * sizeof(double)));
  if (m.data) {
    m.size[0] = size1;
    m.size[1] = size2;
  }
  return m;
}

qmckl_exit_code_device qmckl_matrix_free_device(qmckl_context_device context, qmckl_matrix_device* matrix) {
  if (!matrix || !matrix->data)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_matrix_free_device", "NULL matrix");
  qmckl_exit_code_device rc = qmckl_free_device(context, matrix->data);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  matrix->data = nullptr;
  matrix->size[0] = matrix->size[1] = 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_matrix_of_double_device(const qmckl_context_device context, const double* target,
                                                     const int64_t size_max, qmckl_matrix_device* matrix_out) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!matrix_out || matrix_out->size[0] * matrix_out->size[1] == 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_matrix_device_of_double_device",
                                 "Matrix not allocated");
  if (matrix_out->size[0] * matrix_out->size[1] > size_max)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_matrix_device_of_double_device",
                                 "Wrong vector size");
  // The reference copies size_max doubles without waiting (src/qmckl_blas.cpp:177);
  // this copies the matrix's own size and waits.
  return copy(ctx_of(context), context, matrix_out->data, target,
              (size_t)(matrix_out->size[0] * matrix_out->size[1]) * sizeof(double),
              "qmckl_matrix_device_of_double_device", true);
}

qmckl_exit_code_device qmckl_transpose_device(qmckl_context_device context, const qmckl_matrix_device A,
                                              qmckl_matrix_device At) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (A.size[0] < 1)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_transpose_device", "Invalid size for A");
  if (!At.data)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_transpose_device",
                                 "Output matrix not allocated");
  if (At.size[0] != A.size[1] || At.size[1] != A.size[0])
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_transpose_device",
                                 "Invalid size for At");
  Ctx* ctx = ctx_of(context);
  if (!activate(ctx)) return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_transpose_device", "no device");
  // Fortran (s0, s1) is C [s1][s0]; At(i, j) = A(j, i).
  launch_transpose(ctx, A.data, A.size[1], A.size[0], At.data);
  return finish(ctx, context, "qmckl_transpose_device");
}

qmckl_tensor_device qmckl_tensor_alloc_device(qmckl_context_device context, const int64_t order, const int64_t* size) {
  qmckl_tensor_device t;
  memset(&t, 0, sizeof t);
  if (order <= 0 || order > QMCKL_TENSOR_ORDER_MAX_DEVICE || !size) return t;
  int64_t n = 1;
  for (int64_t i = 0; i < order; ++i) {
    if (size[i] <= 0) return t;
    n *= size[i];
  }
  t.data = static_cast<double*>(qmckl_malloc_device(context, (size_t)n * sizeof(double)));
  if (!t.data) return t;
  t.order = order;
  for (int64_t i = 0; i < order; ++i) t.size[i] = size[i];
  return t;
}

qmckl_exit_code_device qmckl_tensor_free_device(qmckl_context_device context, qmckl_tensor_device* tensor) {
  if (!tensor || !tensor->data)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_tensor_free_device", "NULL tensor");
  qmckl_exit_code_device rc = qmckl_free_device(context, tensor->data);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  memset(tensor, 0, sizeof *tensor);
  return QMCKL_SUCCESS_DEVICE;
}

// ---------------------------------------------------------------- GB300 extensions
qmckl_exit_code_device qmckl_set_async_device(qmckl_context_device context, int32_t async) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  ctx_of(context)->async = async != 0;
  return QMCKL_SUCCESS_DEVICE;
}

void* qmckl_get_stream_device(qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return nullptr;
  Ctx* ctx = ctx_of(context);
  if (!activate(ctx)) return nullptr;
  return ctx->stream;
}

qmckl_exit_code_device qmckl_synchronize_device(qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (!ctx->stream) return QMCKL_SUCCESS_DEVICE;
  cudaSetDevice(ctx->device_id);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_synchronize_device", cudaGetErrorString(e));
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_set_profiling_device(qmckl_context_device context, int32_t enable) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  ctx_of(context)->profiling = enable != 0;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_reset_kernel_stats_device(qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (ctx->stream) {
    cudaSetDevice(ctx->device_id);
    harvest(ctx, true);
  }
  for (auto& s : ctx->stats) {
    s.launches = 0;
    s.total_ms = 0.0;
  }
  ctx->launch_count = 0;
  return QMCKL_SUCCESS_DEVICE;
}

int32_t qmckl_get_kernel_stats_device(qmckl_context_device context, int32_t which, char* name, int64_t name_size,
                                      int64_t* launches, double* total_ms) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return -1;
  Ctx* ctx = ctx_of(context);
  if (ctx->stream) {
    cudaSetDevice(ctx->device_id);
    harvest(ctx, true);
  }
  if (which < 0) return (int32_t)ctx->stats.size();
  if (which >= (int32_t)ctx->stats.size()) return -1;
  const KernelStat& s = ctx->stats[which];
  if (name && name_size > 0) {
    strncpy(name, s.name.c_str(), (size_t)name_size - 1);
    name[name_size - 1] = 0;
  }
  if (launches) *launches = s.launches;
  if (total_ms) *total_ms = s.total_ms;
  return (int32_t)ctx->stats.size();
}

int64_t qmckl_get_launch_count_device(qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return -1;
  return ctx_of(context)->launch_count;
}

qmckl_exit_code_device qmckl_set_allocation_failure_device(qmckl_context_device context, int64_t n) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (n < 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_allocation_failure_device",
                                 "n must be >= 0");
  ctx_of(context)->fail_alloc_countdown = n;
  return QMCKL_SUCCESS_DEVICE;
}

int32_t qmckl_bounds_check_status_device(int32_t reset, int64_t* site, int64_t* index, int64_t* extent) {
  return qg::bounds_check_status(reset != 0, site, index, extent);
}

int32_t qmckl_bounds_check_selftest_device(int64_t index, int64_t extent) {
#ifndef QMCKL_BOUNDS_CHECK
  (void)index;
  (void)extent;
  return -1;
#else
  return qg::bounds_selftest(index, extent) == cudaSuccess ? 0 : -2;
#endif
}

qmckl_exit_code_device qmckl_set_split_wait_test_device(qmckl_context_device context, int64_t wait_cycles,
                                                        int32_t withhold_loads) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (wait_cycles < 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_split_wait_test_device",
                                 "wait_cycles must be >= 0");
  if (withhold_loads != 0 && withhold_loads != 1)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_set_split_wait_test_device",
                                 "withhold_loads must be 0 or 1");
  Ctx* ctx = ctx_of(context);
  ctx->split_wait_cycles = wait_cycles;
  ctx->split_withhold_loads = withhold_loads;
  return QMCKL_SUCCESS_DEVICE;
}

const char* qmckl_gb300_build_info(void) {
#ifdef QMCKL_BOUNDS_CHECK
  return "qmckl-gb300 sm_103a fp64+split-bf16 bounds-check";
#else
  return "qmckl-gb300 sm_103a fp64+split-bf16";
#endif
}

}  // extern "C"
