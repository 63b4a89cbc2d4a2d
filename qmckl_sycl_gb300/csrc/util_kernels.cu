// Small data-movement kernels: tiled transpose (MO coefficients, coordinate layouts),
// strided row copies (value component of a vgl array), fill.
//
// Reference counterparts: coefficient transpose src/qmckl_mo_sycl.cpp:178-183, point
// AoS->SoA src/qmckl_point.cpp:124-129, value copies src/qmckl_ao_sycl.cpp:801-807 (a serial
// single_task there) and src/qmckl_mo.cpp:243-257.
#include <cstdint>

#include "internal.hpp"

namespace qg {
namespace {

// out[c][r] = in[r][c]; in is rows x cols, C order. CTA (x, y) transposes column block x of row
// blocks y, y + gridDim.y, ... (gridDim.y is capped at 65535).
__global__ void transpose_kernel(const double* __restrict__ in, int64_t rows, int64_t cols, double* __restrict__ out) {
  __shared__ double tile[32][33];
  const int64_t bx = (int64_t)blockIdx.x * 32;
  for (int64_t by = (int64_t)blockIdx.y * 32; by < rows; by += (int64_t)gridDim.y * 32) {
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const int64_t r = by + i, c = bx + threadIdx.x;
      if (r < rows && c < cols) tile[i][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const int64_t c = bx + i, r = by + threadIdx.x;
      if (c < cols && r < rows && QG_STORE_OK(kSiteUtil, c * rows + r, rows * cols))
        out[c * rows + r] = tile[threadIdx.x][i];
    }
    __syncthreads();
  }
}

__global__ void strided_copy_kernel(const double* __restrict__ in, int64_t in_stride, double* __restrict__ out,
                                    int64_t out_stride, int64_t rows, int64_t cols) {
  const int64_t n = rows * cols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / cols, c = i - r * cols;
    out[r * out_stride + c] = in[r * in_stride + c];
  }
}

__global__ void fill_kernel(double* __restrict__ p, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// Self-test of the bounds-checked build's recording: evaluates the check for element `index` of
// an array of `extent` elements and stores nothing (there is no array).
__global__ void bounds_selftest_kernel(long long index, long long extent) {
  if (QG_STORE_OK(kSiteUtil, index, extent)) return;
}

unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t launch_transpose(Ctx* ctx, const double* in, int64_t rows, int64_t cols, double* out) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const int64_t row_blocks = (rows + 31) / 32;
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)(row_blocks < 65535 ? row_blocks : 65535));
  LaunchScope scope(ctx, "transpose");
  transpose_kernel<<<grid, dim3(32, 8), 0, ctx->stream>>>(in, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t launch_strided_copy(Ctx* ctx, const double* in, int64_t in_stride, double* out, int64_t out_stride,
                                int64_t rows, int64_t cols) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  LaunchScope scope(ctx, "strided_copy");
  strided_copy_kernel<<<grid_for(rows * cols), 256, 0, ctx->stream>>>(in, in_stride, out, out_stride, rows, cols);
  return cudaGetLastError();
}

cudaError_t launch_fill(Ctx* ctx, double* p, int64_t n, double v) {
  if (n <= 0) return cudaSuccess;
  LaunchScope scope(ctx, "fill");
  fill_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(p, n, v);
  return cudaGetLastError();
}

// Launches the self-test on the current device and waits for it (bounds-checked build; the
// normal build's check is the constant `true`, so the kernel then does nothing).
cudaError_t bounds_selftest(int64_t index, int64_t extent) {
  bounds_selftest_kernel<<<1, 1>>>((long long)index, (long long)extent);
  cudaError_t e = cudaGetLastError();
  return e != cudaSuccess ? e : cudaDeviceSynchronize();
}

// in[num][3] -> out[3][num]
cudaError_t launch_point_aos_to_soa(Ctx* ctx, const double* in, int64_t num, double* out) {
  return launch_transpose(ctx, in, num, 3, out);
}

}  // namespace qg
