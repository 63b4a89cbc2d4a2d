// Measurement helpers exported by the library: stream-ordered CUDA-event timing, host
// buffer page-locking, and an FP64 tensor-pipe (DMMA) throughput probe used as the
// roofline denominator of the FP64 MO contraction.
#include "internal.hpp"

namespace {

// Each warp issues `iters` x 4 independent m16n8k4 DMMAs on register operands; the four
// accumulator sets keep the pipe busy. The result is written once per thread so that
// nothing is optimised away; out has gridDim.x * blockDim.x elements.
__global__ void dmma_peak_kernel(double* out, int iters) {
  const double a0 = threadIdx.x * 1e-3, a1 = a0 + 1.0, b = 1.0 - threadIdx.x * 1e-4;
  double c[4][4] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
                   : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
                   : "d"(a0), "d"(a1), "d"(b));
  }
  double s = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

struct TimerEvents {
  cudaEvent_t a = nullptr, b = nullptr;
};

TimerEvents& timer_of(qg::Ctx* ctx) {
  static thread_local std::unordered_map<qg::Ctx*, TimerEvents> m;
  return m[ctx];
}

}  // namespace

extern "C" {

qmckl_exit_code_device qmckl_timer_start_device(qmckl_context_device context) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  qg::Ctx* ctx = qg::ctx_of(context);
  if (!qg::ensure_device(ctx))
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_timer_start_device", "no usable CUDA device");
  TimerEvents& t = timer_of(ctx);
  if (!t.a) cudaEventCreate(&t.a);
  if (!t.b) cudaEventCreate(&t.b);
  if (cudaEventRecord(t.a, ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_timer_start_device", "cudaEventRecord failed");
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_timer_stop_device(qmckl_context_device context, double* elapsed_ms) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  qg::Ctx* ctx = qg::ctx_of(context);
  TimerEvents& t = timer_of(ctx);
  if (!t.a || !t.b || !elapsed_ms)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_timer_stop_device", "timer not started");
  float ms = 0.f;
  if (cudaEventRecord(t.b, ctx->stream) != cudaSuccess || cudaEventSynchronize(t.b) != cudaSuccess ||
      cudaEventElapsedTime(&ms, t.a, t.b) != cudaSuccess) {
    cudaGetLastError();
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_timer_stop_device", "event timing failed");
  }
  *elapsed_ms = ms;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_host_register_device(qmckl_context_device context, void* ptr, size_t size) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!ptr) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_host_register_device", "NULL pointer");
  qg::Ctx* ctx = qg::ctx_of(context);
  if (!qg::ensure_device(ctx) || cudaHostRegister(ptr, size, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_host_register_device", "cudaHostRegister failed");
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_host_unregister_device(qmckl_context_device context, void* ptr) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!ptr) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_host_unregister_device", "NULL pointer");
  if (cudaHostUnregister(ptr) != cudaSuccess) {
    cudaGetLastError();
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_host_unregister_device", "cudaHostUnregister failed");
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_exp_check_device(qmckl_context_device context, const double* x, int64_t n, double* out) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  qg::Ctx* ctx = qg::ctx_of(context);
  if (!ctx->ao_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_exp_check_device", nullptr);
  qmckl_exit_code_device rc = qg::ensure_tables(ctx, context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!x || !out || n < 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_exp_check_device", "bad arguments");
  qg::launch_exp_check(ctx, ctx->ao_basis.tables.exp_table, x, n, out);
  return qg::finish(ctx, context, "qmckl_exp_check_device");
}

qmckl_exit_code_device qmckl_prim_value_check_device(qmckl_context_device context, const double* r2, int64_t n,
                                                     double* out, int64_t size_max) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  qg::Ctx* ctx = qg::ctx_of(context);
  if (!ctx->ao_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_prim_value_check_device", nullptr);
  qmckl_exit_code_device rc = qg::ensure_tables(ctx, context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!r2 || n < 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_prim_value_check_device", "bad arguments");
  if (!out)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_4_DEVICE, "qmckl_prim_value_check_device", "NULL");
  if (size_max < n * ctx->ao_basis.prim_num)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_5_DEVICE, "qmckl_prim_value_check_device",
                                 "size_max < n * prim_num");
  qg::launch_prim_check(ctx, ctx->ao_basis.tables, r2, n, ctx->ao_basis.prim_num, out);
  return qg::finish(ctx, context, "qmckl_prim_value_check_device");
}

qmckl_exit_code_device qmckl_measure_fp64_peak_device(qmckl_context_device context, double* tflops) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!tflops) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_measure_fp64_peak_device", "NULL");
  qg::Ctx* ctx = qg::ctx_of(context);
  if (!qg::ensure_device(ctx))
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_measure_fp64_peak_device", "no device");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 256;
  double* out = static_cast<double*>(qg::dalloc(ctx, sizeof(double) * blocks * threads));
  if (!out) return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_measure_fp64_peak_device", nullptr);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, ctx->stream);
    dmma_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, iters);
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    const double flops = (double)blocks * threads / 32.0 * iters * 4 * (16.0 * 8 * 4 * 2);
    if (ms > 0 && rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  qg::dfree(ctx, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_measure_fp64_peak_device", cudaGetErrorString(e));
  *tflops = best;
  return QMCKL_SUCCESS_DEVICE;
}

}  // extern "C"
