// FP64 MO contraction on the FP64 tensor pipe (DMMA, mma.sync m16n8k4 .f64) for sm_103a.
//
//   mo_vgl[5P][M] = ao_vgl[5P][A] * coef_t[A][M]        (rows r = 5*point + component)
//   mo_value[P][M] = ao_value[P][A] * coef_t[A][M]
//
// Reference: src/qmckl_mo_sycl.cpp:24-50 (one work-item per point, serial triple loop) and
// :77-129 (value only). The reference skips AO k of a point, for every component, when that
// AO's *value* is exactly zero (:40). For the value row the skip changes nothing; for the
// gradient and Laplacian rows it drops the term, so this kernel applies the same mask: an
// element (5p + c, k) with c > 0 is read as zero when ao_vgl[5p][k] == 0.
//
// On GB300 the FP64 pipe (DFMA and DMMA alike) delivers ~1.05 TFLOP/s, so this GEMM is
// bound by DMMA issue, with arithmetic intensity ~2M/(8(1+M/A)) FLOP/byte: no shared-memory
// staging is needed to feed it. Each warp owns a 32x32 output tile (2 x 4 m16n8 fragments)
// and reads its A and B fragments straight from L1/L2; a CTA of 4 warps covers 64 rows x
// 64 columns so that neighbouring warps share A rows in L1.
#include <cstdint>

#include "internal.hpp"

namespace qg {
namespace {

constexpr int kWM = 32, kWN = 32;     // warp tile
constexpr int kCM = 64, kCN = 64;     // CTA tile (2 x 2 warps)

__device__ __forceinline__ void dmma_16x8x4(double (&d)[4], double a0, double a1, double b0) {
  asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
               : "+d"(d[0]), "+d"(d[1]), "+d"(d[2]), "+d"(d[3])
               : "d"(a0), "d"(a1), "d"(b0));
}

// Element (r, k) of A (row-major, ld = K) with bounds and, when MASK, the reference's
// zero-value skip for rows whose component (r % 5) is not 0.
template <bool MASK>
__device__ __forceinline__ double load_a(const double* __restrict__ A, int64_t lda, int64_t R, int64_t K, int64_t r,
                                         int64_t k) {
  if (r >= R || k >= K) return 0.0;
  double v = __ldg(A + r * lda + k);
  if constexpr (MASK) {
    const int comp = (int)(r % 5);
    if (comp != 0) {
      const double v0 = __ldg(A + (r - comp) * lda + k);
      if (v0 == 0.0) v = 0.0;
    }
  }
  return v;
}

// One warp's 32x32 tile of C at (r0, c0), if it starts inside C. A is R x K with leading
// dimension lda (lda > K for a K-slice of a wider matrix), B is K x N, C is R x N.
template <bool MASK>
__device__ __forceinline__ void dgemm_warp_tile(const double* __restrict__ A, int64_t lda,
                                                const double* __restrict__ B, double* __restrict__ C, int64_t R,
                                                int64_t K, int64_t N, int64_t r0, int64_t c0, int lane) {
  if (r0 >= R || c0 >= N) return;  // warp-uniform
  const int g = lane >> 2, t = lane & 3;
  double acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0;

  bool colok[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) colok[j] = c0 + 8 * j + g < N;

#pragma unroll 2
  for (int64_t k = 0; k < K; k += 4) {
    double a[2][2], b[4];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      a[i][0] = load_a<MASK>(A, lda, R, K, r0 + 16 * i + g, k + t);
      a[i][1] = load_a<MASK>(A, lda, R, K, r0 + 16 * i + g + 8, k + t);
    }
    const bool kok = k + t < K;
#pragma unroll
    for (int j = 0; j < 4; ++j) b[j] = (kok && colok[j]) ? __ldg(B + (k + t) * N + c0 + 8 * j + g) : 0.0;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) dmma_16x8x4(acc[i][j], a[i][0], a[i][1], b[j]);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t col = c0 + 8 * j + 2 * t;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t row = r0 + 16 * i + g + 8 * h;
        if (row < R) {
          if (col < N && QG_STORE_OK(kSiteDgemmOut, row * N + col, R * N)) C[row * N + col] = acc[i][j][2 * h];
          if (col + 1 < N && QG_STORE_OK(kSiteDgemmOut, row * N + col + 1, R * N))
            C[row * N + col + 1] = acc[i][j][2 * h + 1];
        }
      }
    }
}

// CTA (x, y) covers column block x and row blocks y, y + gridDim.y, ... (gridDim.y is capped at
// 65535, so more row blocks are walked in turn).
template <bool MASK>
__global__ void __launch_bounds__(128) dgemm_dmma_kernel(const double* __restrict__ A, const double* __restrict__ B,
                                                         double* __restrict__ C, int64_t R, int64_t K, int64_t N) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c0 = (int64_t)blockIdx.x * kCN + (warp & 1) * kWN;
  for (int64_t rb = blockIdx.y; rb * kCM < R; rb += gridDim.y) {
    const int64_t r0 = rb * kCM + (warp >> 1) * kWM;
    dgemm_warp_tile<MASK>(A, K, B, C, R, K, N, r0, c0, lane);
  }
}

// Split-K: CTA z computes the K-slice [z*kc, min(K, (z+1)*kc)) of A*B into parts[z] (R x N).
__global__ void __launch_bounds__(128) dgemm_splitk_kernel(const double* __restrict__ A, const double* __restrict__ B,
                                                           double* __restrict__ parts, int64_t R, int64_t K,
                                                           int64_t N, int64_t kc) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t k0 = (int64_t)blockIdx.z * kc;
  const int64_t kn = (K - k0) < kc ? (K - k0) : kc;
  const int64_t c0 = (int64_t)blockIdx.x * kCN + (warp & 1) * kWN;
  for (int64_t rb = blockIdx.y; rb * kCM < R; rb += gridDim.y) {
    const int64_t r0 = rb * kCM + (warp >> 1) * kWM;
    dgemm_warp_tile<false>(A + k0, K, B + k0 * N, parts + (int64_t)blockIdx.z * R * N, R, kn, N, r0, c0, lane);
  }
}

// out[i] = sum over z (in order) of parts[z][i].
__global__ void sum_parts_kernel(const double* __restrict__ parts, int nparts, int64_t n, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int z = 0; z < nparts; ++z) s += parts[(int64_t)z * n + i];
  if (QG_STORE_OK(kSiteSumParts, i, n)) out[i] = s;
}

// Several contractions, persistent: a CTA of WR x WC warps owns (32 WR) x (32 WC) tiles of C,
// taken from *counter in job order (the host lists the jobs with the longest K first).
template <bool MASK, int WR, int WC>
__global__ void __launch_bounds__(32 * WR * WC) dgemm_batch_kernel(const GemmJob* __restrict__ jobs,
                                                                    const int32_t* __restrict__ tile_begin, int njobs,
                                                                    int total_tiles, unsigned int* counter) {
  __shared__ int s_tile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= total_tiles) break;
    int lo = 0, hi = njobs - 1;  // last job whose first tile is <= tile
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tile_begin[mid] <= tile) lo = mid;
      else hi = mid - 1;
    }
    const GemmJob& jb = jobs[lo];
    const int local = tile - tile_begin[lo];
    const int64_t r0 = (int64_t)(local / jb.col_tiles) * (32 * WR) + (warp / WC) * 32;
    const int64_t c0 = (int64_t)(local % jb.col_tiles) * (32 * WC) + (warp % WC) * 32;
    dgemm_warp_tile<MASK>(jb.a, jb.k, jb.b, jb.c, jb.rows, jb.k, jb.cols, r0, c0, lane);
  }
}

template <bool MASK, int WR, int WC>
cudaError_t launch_batch_shape(cudaStream_t stream, const GemmJob* jobs, const int32_t* tile_begin, int njobs,
                               int total_tiles, unsigned int* counter) {
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dgemm_batch_kernel<MASK, WR, WC>, 32 * WR * WC, 0);
  int grid = sms * (per_sm > 0 ? per_sm : 1);
  if (grid > total_tiles) grid = total_tiles;
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream);
  if (e != cudaSuccess) return e;
  dgemm_batch_kernel<MASK, WR, WC><<<grid, 32 * WR * WC, 0, stream>>>(jobs, tile_begin, njobs, total_tiles, counter);
  return cudaGetLastError();
}

// Row blocks of R rows for gridDim.y (at most 65535; the kernels walk the rest).
int64_t grid_rows(int64_t R) {
  const int64_t rb = (R + kCM - 1) / kCM;
  return rb < 65535 ? rb : 65535;
}

template <bool MASK>
cudaError_t launch_dgemm(Ctx* ctx, const double* A, const double* B, double* C, int64_t R, int64_t K, int64_t N,
                         const char* name) {
  if (R <= 0 || N <= 0) return cudaSuccess;
  if (K <= 0) return cudaMemsetAsync(C, 0, sizeof(double) * R * N, ctx->stream);
  dim3 grid((unsigned)((N + kCN - 1) / kCN), (unsigned)grid_rows(R));
  LaunchScope scope(ctx, name);
  dgemm_dmma_kernel<MASK><<<grid, 128, 0, ctx->stream>>>(A, B, C, R, K, N);
  return cudaGetLastError();
}

}  // namespace

void gemm_shape_tile(int shape, int* rows, int* cols) {
  *rows = shape == 1 ? 128 : 64;
  *cols = shape == 2 ? 128 : 64;
}

cudaError_t launch_dgemm_batch(cudaStream_t stream, int shape, bool mask5, const GemmJob* jobs,
                               const int32_t* tile_begin, int njobs, int total_tiles, unsigned int* counter) {
  if (njobs <= 0 || total_tiles <= 0) return cudaSuccess;
  switch (shape * 2 + (mask5 ? 1 : 0)) {
    case 0: return launch_batch_shape<false, 2, 2>(stream, jobs, tile_begin, njobs, total_tiles, counter);
    case 1: return launch_batch_shape<true, 2, 2>(stream, jobs, tile_begin, njobs, total_tiles, counter);
    case 2: return launch_batch_shape<false, 4, 2>(stream, jobs, tile_begin, njobs, total_tiles, counter);
    case 3: return launch_batch_shape<true, 4, 2>(stream, jobs, tile_begin, njobs, total_tiles, counter);
    case 4: return launch_batch_shape<false, 2, 4>(stream, jobs, tile_begin, njobs, total_tiles, counter);
    case 5: return launch_batch_shape<true, 2, 4>(stream, jobs, tile_begin, njobs, total_tiles, counter);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_dgemm_rm(Ctx* ctx, const double* A, const double* B, double* C, int64_t R, int64_t K, int64_t N,
                            const char* name) {
  return launch_dgemm<false>(ctx, A, B, C, R, K, N, name);
}

int64_t dgemm_splitk_parts(int64_t R, int64_t K, int64_t N, int sms) {
  const int64_t tiles = ((R + kCM - 1) / kCM) * ((N + kCN - 1) / kCN);
  int64_t z = (4 * (int64_t)sms + tiles - 1) / tiles;  // about four CTAs per SM
  const int64_t max_by_k = (K + 63) / 64;               // slices of at least 64
  if (z > max_by_k) z = max_by_k;
  return z < 1 ? 1 : z;
}

cudaError_t launch_dgemm_splitk(Ctx* ctx, const double* A, const double* B, double* parts, int64_t nparts, double* C,
                                int64_t R, int64_t K, int64_t N, const char* name) {
  if (R <= 0 || N <= 0) return cudaSuccess;
  if (K <= 0 || nparts < 1) return cudaMemsetAsync(C, 0, sizeof(double) * R * N, ctx->stream);
  int64_t kc = (K + nparts - 1) / nparts;
  kc = (kc + 3) / 4 * 4;
  const int64_t z = (K + kc - 1) / kc;
  dim3 grid((unsigned)((N + kCN - 1) / kCN), (unsigned)grid_rows(R), (unsigned)z);
  {
    LaunchScope scope(ctx, name);
    dgemm_splitk_kernel<<<grid, 128, 0, ctx->stream>>>(A, B, parts, R, K, N, kc);
  }
  LaunchScope scope(ctx, "sum_parts");
  sum_parts_kernel<<<(unsigned)((R * N + 255) / 256), 256, 0, ctx->stream>>>(parts, (int)z, R * N, C);
  return cudaGetLastError();
}

cudaError_t launch_mo_vgl_fp64(Ctx* ctx, const double* ao_vgl, const double* coef_t, int64_t point_num,
                               int64_t ao_num, int64_t mo_num, double* mo_vgl) {
  return launch_dgemm<true>(ctx, ao_vgl, coef_t, mo_vgl, 5 * point_num, ao_num, mo_num, "mo_vgl_dgemm");
}

cudaError_t launch_mo_value_fp64(Ctx* ctx, const double* ao_value, const double* coef_t, int64_t point_num,
                                 int64_t ao_num, int64_t mo_num, double* mo_value) {
  return launch_dgemm<false>(ctx, ao_value, coef_t, mo_value, point_num, ao_num, mo_num, "mo_value_dgemm");
}

}  // namespace qg
