// Split-BF16 MO contraction on the tcgen05 tensor cores (the precision form).
//
//   mo[r][m] = sum_k ao[r][k] * coef[m][k],   r = 5*point + component (or point, value only)
//
// Each FP64 operand x is split into three BF16 terms x ~ x_hi + x_mid + x_lo (24 significant
// bits), and the product is formed from the six terms whose order is above 2^-24:
//   hi*hi + hi*mid + mid*hi + hi*lo + mid*mid + lo*hi
// on tcgen05.mma kind::f16 (BF16 x BF16 -> FP32 in tensor memory). Distances, exponentials,
// screening and the AO Laplacian assembly stay FP64 (the AO kernel); only this contraction
// runs on the BF16 tensor cores. The reference computes it in FP64 with one work-item per
// point (src/qmckl_mo_sycl.cpp:24-50); the AO-value-is-zero skip of its line 40 is applied
// when the AO operand is split.
//
// The split avoids the FP64 pipe entirely (on GB300 it issues at ~1/66 of the FP32 rate):
// the double is rounded to float with integer instructions on its bit pattern, and the
// three BF16 terms are peeled off in FP32, where every subtraction is exact.
//
// Accumulation. The tensor core adds each MMA's products into the FP32 accumulator with a
// truncating alignment, so every MMA costs an error of order 2^-24 of the accumulator (and of
// its largest product). The five correction products (all ~2^-8 of the result or smaller)
// go into their own accumulator; the main hi*hi product is accumulated for two 64-wide K
// blocks at a time (eight MMAs) in one of two alternating tensor-memory buffers, and the fold
// warps add each finished block sum into a running FP32 sum held in registers (rounded, not
// truncated) while the next blocks are multiplied, so the truncation error does not grow with K.
// The result is that sum + corrections, rounded once to FP32 and widened exactly to FP64. (A
// compensated FP32 two-sum (hi, lo) for the running sum, QMCKL_SPLIT_TWO_SUM=1, lowers the
// medium workload's worst normwise error from 5.1e-7 to 4.9e-7 and costs 5 % of the contraction
// there, 16 % on the 64-molecule batch: measured 0.655 / 0.691 ms and 1.627 / 1.946 ms.)
//
// GEMM structure (persistent, one CTA per SM, 128 x N output tiles with N <= 160): warp 0
// issues TMA loads of the six operand planes per 64-wide K block into a two-stage ring of
// 128B-swizzled shared-memory buffers; warp 1 owns tensor memory and issues the MMAs (24 per K
// block: six products x four K=16 steps); eight fold warps, two per 32-lane quarter of tensor
// memory (one row per thread, one column half per warp), fold the main product and write the
// tile's FP64 results from registers (32-byte stores of each thread's row segment, or, for rows
// not 32-byte aligned, through a small per-warp transposition buffer). An MMA costs nearly the
// same time for N = 32 to 160 (its A operand fetch dominates), so the widest tile that tensor
// memory and shared memory allow sets the rate: 160 columns halve the MMA count of 80-column
// tiles. Every
// mbarrier wait is bounded (~1 s); on expiry the kernel records an error code, drains what it
// issued, releases its tensor memory and exits, and the host reports QMCKL_FAILURE_DEVICE.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <vector>

#include "internal.hpp"

namespace qg {
namespace {

constexpr int kBM = 128;        // rows per tile (UMMA M)
constexpr int kBK = 64;         // K per stage: 64 BF16 = 128 bytes = one swizzle row
constexpr int kStages = 2;
constexpr int kMaxN = 160;      // columns per tile: two halves of <= 80, each fold thread holds 2 x 80 sums
constexpr int kHalfN = kMaxN / 2;
constexpr int kThreads = 384;   // 12 warps = 3 warpgroups: {TMA, MMA, 2 idle}, 8 fold warps
constexpr int kBufs = 2;         // main-product TMEM buffers: the MMAs run up to one fold group ahead
constexpr int kFold = 2;         // K blocks (of 64) per main-product block sum folded into the running sum
// Tensor memory (512 columns): corrections [0, kMaxN), main buffer b at kMaxN * (1 + b).
static_assert(kMaxN * (1 + kBufs) <= 512, "tensor memory holds the corrections and the main buffers");
// registers per thread after setmaxnreg: warpgroup 0 (TMA, MMA), warpgroups 1 and 2 (fold);
// launched with 168 per thread: 384 x 168 = 64512 = 128 x 56 + 256 x 224
constexpr int kRegsIssue = 56;
constexpr int kRegsFold = 224;
static_assert(128 * kRegsIssue + 256 * kRegsFold <= kThreads * 168, "register split exceeds the launch's registers");
constexpr uint32_t kPlaneA = kBM * kBK * 2;  // 16 KB per A plane and stage
constexpr uint32_t kMaxStage = 3 * kPlaneA + 3 * (uint32_t)kMaxN * kBK * 2;  // 108 KB
constexpr int kTPitch = 9;                   // transposition buffer: 32 rows x 8 floats, row pitch 9
constexpr uint32_t kTBuf = 32 * kTPitch * 4;  // bytes per fold warp
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s at GB300 clocks
#ifndef QMCKL_SPLIT_TWO_SUM
#define QMCKL_SPLIT_TWO_SUM 0
#endif
// The fold keeps the running main product as one FP32 sum, or (QMCKL_SPLIT_TWO_SUM=1) as an FP32
// two-sum (hi, lo).
constexpr bool kTwoSum = QMCKL_SPLIT_TWO_SUM != 0;

// Launch controls of the contraction kernel: the limit of every mbarrier wait (clock cycles),
// and, for the failure-handling test only, a producer that issues no loads, so that the
// consumers' first wait is one that nothing completes and runs out (no load is in flight then).
struct SplitCtl {
  long long wait_cycles = kWaitCycles;
  int32_t withhold_loads = 0;
};

// ------------------------------------------------------------------ split helpers
// Double -> float, round to nearest even, by integer operations on the bit pattern (no FP64
// instruction). Values below the float normal range flush to a signed zero; AO and MO
// coefficients are far inside the float range.
__device__ __forceinline__ float f64_to_f32_int(double a) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
  const unsigned long long frac = b & 0xFFFFFFFFFFFFFull;
  unsigned int m = (unsigned int)(frac >> 29);
  const unsigned long long rem = frac & 0x1FFFFFFFull;
  unsigned int bits = ((unsigned int)e << 23) | m;
  if (rem > 0x10000000ull || (rem == 0x10000000ull && (m & 1u))) bits += 1u;  // carry may bump the exponent
  return __uint_as_float(sign | bits);
}

// Float -> double exactly, by integer operations only, for every input (normal, zero,
// subnormal, infinity, NaN): a conversion instruction would run on the FP64 pipe, which issues at
// 1/64 of the FP32 rate on this GPU (the epilogue converts every output element).
__device__ __forceinline__ double f32_to_f64_int(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned int e = (u >> 23) & 0xFF, m = u & 0x7FFFFF;
  unsigned long long bits;
  if (e == 0) {
    // zero, or the subnormal m 2^-149: its leading bit at position p becomes the implicit one
    const int p = 31 - __clz(m);
    bits = m == 0 ? 0ull
                  : ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
  } else {
    const unsigned long long ee = e == 0xFF ? 0x7FFull : (unsigned long long)(e + 896);
    bits = (ee << 52) | ((unsigned long long)m << 29);
  }
  return __longlong_as_double((long long)(sign | bits));
}

// The same for normal numbers and zeros only, in six integer instructions: the double's upper word
// is the float's with the exponent re-biased (+896) and the mantissa shifted right by 3, its lower
// word the mantissa's last 3 bits. f32_special() tells which inputs need f32_to_f64_int instead.
__device__ __forceinline__ double f32_to_f64_normal(float f) {
  const unsigned int u = __float_as_uint(f), a = u & 0x7FFFFFFFu;
  const unsigned int hi = (u & 0x80000000u) | (a == 0 ? 0u : (a >> 3) + 0x38000000u);
  double d;
  asm("mov.b64 %0, {%1, %2};" : "=d"(d) : "r"(a << 29), "r"(hi));
  return d;
}
// Subnormal, infinite or NaN.
__device__ __forceinline__ bool f32_special(float f) {
  const unsigned int a = __float_as_uint(f) & 0x7FFFFFFFu;
  return a != 0 && a - 0x00800000u >= 0x7F000000u;
}

__device__ __forceinline__ void split3(double a, __nv_bfloat16& hi, __nv_bfloat16& mid, __nv_bfloat16& lo) {
  const float f = f64_to_f32_int(a);
  hi = __float2bfloat16_rn(f);
  const float r1 = f - __bfloat162float(hi);
  mid = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(mid);
  lo = __float2bfloat16_rn(r2);
}

// src [rows][ld_src] FP64 -> planes [3][rows][kp] BF16, zero in columns [k, kp). With
// mask5, an element of a row whose component (row % 5) is not 0 is zeroed when the value
// row of the same point has a zero in that column (src/qmckl_mo_sycl.cpp:40).
__global__ void split_planes_kernel(const double* __restrict__ src, int64_t rows, int64_t k, int64_t ld_src,
                                    int64_t kp, int mask5, __nv_bfloat16* __restrict__ planes) {
  const int64_t n = rows * kp;
  const int64_t plane = rows * kp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / kp, c = i - r * kp;
    double a = 0.0;
    if (c < k) {
      a = src[r * ld_src + c];
      if (mask5) {
        const int comp = (int)(r % 5);
        if (comp != 0 && src[(r - comp) * ld_src + c] == 0.0) a = 0.0;
      }
    }
    __nv_bfloat16 h, m, l;
    split3(a, h, m, l);
    if (!QG_STORE_OK(kSiteSplitPlanes, 2 * plane + i, 3 * plane)) continue;
    planes[i] = h;
    planes[plane + i] = m;
    planes[2 * plane + i] = l;
  }
}

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: true when the phase completed, false after `limit` cycles (~1 s by default).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (clock64() - t0 > limit) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor for a K-major operand in the 128B-swizzled layout that
// TMA writes: rows of 128 bytes, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;            // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

// Shared-memory descriptor of an M-major ("MN-major") operand tile with 128-byte swizzle, the
// layout TMA writes for boxes of 64 M x 64 K: K rows of 128 bytes (64 consecutive M), 8-row
// groups 1024 bytes apart (stride byte offset), and the second 64-wide M half 8 KB further
// (leading byte offset).
__device__ __forceinline__ uint64_t sdesc_mn(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(8192 >> 4) << 16;  // leading byte offset: next 64-element M block
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: next 8-row K group
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// The six MMAs of one K step, issued together: hi.hi into the main buffer d0 (accumulate flag
// am), then hi.mid, mid.hi, hi.lo, mid.mid, lo.hi into the correction accumulator d1 (flag ac for
// the first, accumulate for the rest). Descriptors come precomputed: the issuing thread's
// instruction count per MMA sets its issue rate.
__device__ __forceinline__ void umma_six(uint32_t d0, uint32_t d1, uint64_t a0, uint64_t b0, uint64_t a1, uint64_t b1,
                                         uint64_t a2, uint64_t b2, uint64_t a3, uint64_t b3, uint64_t a4, uint64_t b4,
                                         uint64_t a5, uint64_t b5, uint32_t idesc, uint32_t am, uint32_t ac) {
  asm volatile(
      "{\n .reg .pred pm, pc, pt;\n setp.ne.b32 pm, %15, 0;\n setp.ne.b32 pc, %16, 0;\n setp.eq.b32 pt, 0, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %2, %3, %14, pm;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%1], %4, %5, %14, pc;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%1], %6, %7, %14, pt;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%1], %8, %9, %14, pt;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%1], %10, %11, %14, pt;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%1], %12, %13, %14, pt;\n}\n" ::"r"(d0),
      "r"(d1), "l"(a0), "l"(b0), "l"(a1), "l"(b1), "l"(a2), "l"(b2), "l"(a3), "l"(b3), "l"(a4), "l"(b4), "l"(a5),
      "l"(b5), "r"(idesc), "r"(am), "r"(ac));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// tcgen05.ld of 16 consecutive columns (32 lanes x 32 bit), not yet waited for.
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// Waits for every outstanding tcgen05.ld of the thread; r is passed through so that its uses
// cannot be scheduled before the wait (call it for each array loaded; only the first waits).
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15])
               :
               : "memory");
}

// One contraction (one molecule): its six operand tensor maps and output. Jobs live in
// global memory so that one persistent launch can work through the tiles of many of them;
// tile t of the launch belongs to the job with the largest tile_begin <= t.
struct alignas(64) SplitJob {
  CUtensorMap ta[3];  // A planes: [3][rows][kp] (K-major) or [3][kp][rows] (M-major)
  CUtensorMap tb[3];  // B planes [3][cols][kp]
  double* out;        // [rows][ldo]
  int64_t rows;       // valid rows
  int64_t cols;       // valid columns (MO count)
  int64_t ldo;
  int32_t kblocks;    // kp / 64
  int32_t n_tile;     // columns per tile (multiple of 16, <= kMaxN)
  int32_t col_tiles;  // tiles along the columns
  int32_t tile_begin; // index of this job's first tile in the launch
  // M-major A (the fused AO kernel's 64-point blocks): operand row r = (5 g + c) 64 + j is
  // component c of the point at processing slot s = 64 g + j; it lands in output row
  // 5 * perm[s] + c (s < npts).
  int32_t a_mn;
  int32_t pp;         // points padded to a multiple of 64 (rows = 5 pp)
  int64_t npts;
  const int32_t* perm;  // processing order (null: identity)
};


// Two FP32 values in one 64-bit register (column 2i in the low half, 2i + 1 in the high half) for
// the packed FP32x2 instructions: two columns per instruction, each lane rounded exactly as the
// scalar instruction would round it.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pack2(uint32_t lo, uint32_t hi) {
  f32x2 d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "r"(lo), "r"(hi));
  return d;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ float lo_f(f32x2 v) { return __uint_as_float((uint32_t)v); }
__device__ __forceinline__ float hi_f(f32x2 v) { return __uint_as_float((uint32_t)(v >> 32)); }

// Knuth's TwoSum on two columns at once: s = fl(a + b) and the exact rounding error e.
__device__ __forceinline__ void two_sum2(f32x2 a, f32x2 b, f32x2& s, f32x2& e) {
  s = add2(a, b);
  const f32x2 bp = sub2(s, a);
  e = add2(sub2(a, sub2(s, bp)), sub2(b, bp));
}

// One 32-byte store (four doubles) to a 32-byte aligned global address.
__device__ __forceinline__ void st_global_v4(double* p, double a, double b, double c, double d) {
  asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(p), "d"(a), "d"(b), "d"(c), "d"(d) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait that also gives up once another role has aborted.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                              long long limit) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (*abort_flag || clock64() - t0 > limit) return false;
  }
  return true;
}

__device__ __forceinline__ void set_abort(volatile int* abort_flag, int* error, int code) {
  *abort_flag = 1;
  atomicExch(error, code);
}

// Tile geometry of launch tile `tile`: its job and the job-local row / column origins.
struct TileRef {
  const SplitJob* job;
  int m0, n0;
};
__device__ __forceinline__ TileRef tile_ref(const SplitJob* __restrict__ jobs, int njobs, int tile) {
  int j = 0, hi = njobs - 1;  // last job whose first tile is <= tile
  while (j < hi) {
    const int mid = (j + hi + 1) >> 1;
    if (jobs[mid].tile_begin <= tile) j = mid;
    else hi = mid - 1;
  }
  const SplitJob* job = &jobs[j];
  const int local = tile - job->tile_begin;
  TileRef t;
  t.job = job;
  t.m0 = (local / job->col_tiles) * kBM;
  t.n0 = (local % job->col_tiles) * job->n_tile;
  return t;
}

template <int R>
__device__ __forceinline__ void reg_dec() {
  asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(R));
}
__device__ __forceinline__ void reg_inc() { asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kRegsFold)); }

// What the fold warps of a CTA share across tiles.
struct FoldCtx {
  uint32_t lb;                       // TMEM address of this warp's 32 lanes, column 0
  float* tb;                         // this warp's transposition buffer (32 rows x kTPitch)
  uint64_t *accf, *acce, *tmem_free;
  volatile int* abort_flag;
  int* error;
  long long wait_cycles;
  int lane, quarter, half;
};

// Starts reading 16 (full16) or 8 consecutive columns of the warp's 32 lanes from tensor memory
// into r[o..o+15] (the rest of the 16 zeroed); tmem_wait_ld32 completes it.
__device__ __forceinline__ void tmem_ld_async(uint32_t taddr, bool full16, uint32_t (&r)[32], int o) {
  if (full16) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[o + 0]), "=r"(r[o + 1]), "=r"(r[o + 2]), "=r"(r[o + 3]), "=r"(r[o + 4]), "=r"(r[o + 5]),
          "=r"(r[o + 6]), "=r"(r[o + 7]), "=r"(r[o + 8]), "=r"(r[o + 9]), "=r"(r[o + 10]), "=r"(r[o + 11]),
          "=r"(r[o + 12]), "=r"(r[o + 13]), "=r"(r[o + 14]), "=r"(r[o + 15])
        : "r"(taddr));
  } else {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[o + 0]), "=r"(r[o + 1]), "=r"(r[o + 2]), "=r"(r[o + 3]), "=r"(r[o + 4]), "=r"(r[o + 5]),
                   "=r"(r[o + 6]), "=r"(r[o + 7])
                 : "r"(taddr));
#pragma unroll
    for (int q = 8; q < 16; ++q) r[o + q] = 0u;
  }
}
// Waits for every outstanding tcgen05.ld of the thread; the 32 registers pass through it so that
// their uses cannot be scheduled before the wait.
__device__ __forceinline__ void tmem_wait_ld32(uint32_t (&r)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                 "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                 "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
               :
               : "memory");
}

// Reads n (16 or 8) consecutive columns of the warp's 32 lanes from tensor memory and waits.
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, bool full16, uint32_t (&r)[16]) {
  if (full16) {
    tmem_ld16_async(taddr, r);
  } else {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int q = 8; q < 16; ++q) r[q] = 0u;
  }
  tmem_wait_ld(r);
}

// One fold warp's work on one tile (one row per thread, this warp's half of the N columns):
// after every kFold K blocks, the main product's FP32 block sum is read out of tensor memory and
// added into a running sum held in registers (tensor-memory traffic slows the MMAs that share it,
// so the sum does not live there); at the end sum + corrections is formed, tensor memory is released to the next tile, and the warp writes its 32 x N/2 block of
// the output: with 32-byte stores of each lane's own row where the rows allow it, otherwise eight
// columns at a time through the transposition buffer (each store instruction then writes four
// rows x 64 contiguous bytes). it: the running fold-group index (advanced). Returns false when a
// wait gave up.
__device__ __forceinline__ bool fold_tile(const FoldCtx& f, const SplitJob& job, const TileRef& tr, uint32_t& it) {
  // running sum of the main product, two columns per register, in h2 (and its two-sum's low part
  // in l2 when kTwoSum)
  f32x2 h2[kHalfN / 2], l2[kHalfN / 2];
  const int nh = job.n_tile >> 1;             // columns of this warp: [hc, hc + nh)
  const uint32_t hc = (uint32_t)(f.half * nh);
  // Output row of this thread's tile row (lane = row), looked up before the folds so that the
  // point order's load latency is hidden.
  const int64_t row = (int64_t)tr.m0 + f.quarter * 32 + f.lane;
  int64_t orow = row < job.rows ? row : -1;
  if (job.a_mn && orow >= 0) {
    const int64_t q = orow / 64, g = q / 5, comp = q - 5 * g, slot = 64 * g + (orow - 64 * q);
    orow = slot < job.npts ? 5 * (job.perm ? (int64_t)job.perm[slot] : slot) + comp : -1;
  }
  const int groups = (job.kblocks + kFold - 1) / kFold;
  for (int kb = 0; kb < groups; ++kb, ++it) {
    const uint32_t b = it % kBufs, use = it / kBufs;
    // warp-uniform decision: the tcgen05.ld below are .sync.aligned
    if (!__all_sync(0xffffffffu, wait_or_abort(&f.accf[b], use & 1u, f.abort_flag, f.wait_cycles))) {
      if (f.lane == 0) set_abort(f.abort_flag, f.error, 4);
      return false;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t mcol = (uint32_t)kMaxN * (1 + b) + hc;
    // 32 columns per wait: two loads in flight halve the tensor-memory round trips
#pragma unroll
    for (int c0 = 0; c0 < kHalfN; c0 += 32) {
      if (c0 < nh) {
        const bool fa = c0 + 16 <= nh, hb = c0 + 16 < nh, fb = c0 + 32 <= nh;
        uint32_t rv[32];
        tmem_ld_async(f.lb + mcol + (uint32_t)c0, fa, rv, 0);
        if (hb) tmem_ld_async(f.lb + mcol + (uint32_t)c0 + 16, fb, rv, 16);
        tmem_wait_ld32(rv);
#pragma unroll
        for (int q = 0; q < 32; q += 2) {
          if (c0 + q < kHalfN && (q < 8 || (q < 16 && fa) || (q >= 16 && hb && (q < 24 || fb)))) {
            const int i = (c0 + q) >> 1;
            const f32x2 v = pack2(rv[q], rv[q + 1]);
            if (kb == 0) {
              h2[i] = v;
              if constexpr (kTwoSum) l2[i] = 0ull;
            } else if constexpr (kTwoSum) {
              f32x2 s2, e2;
              two_sum2(h2[i], v, s2, e2);
              h2[i] = s2;
              l2[i] = add2(l2[i], e2);
            } else {
              h2[i] = add2(h2[i], v);
            }
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncwarp();
    if (f.lane == 0) mbar_arrive(&f.acce[b]);
  }
  // The last accf phase covered every MMA of the tile, corrections included.
#pragma unroll
  for (int c0 = 0; c0 < kHalfN; c0 += 16) {
    if (c0 < nh) {
      const bool full16 = c0 + 16 <= nh;
      uint32_t rc[16];
      tmem_ld_cols(f.lb + hc + (uint32_t)c0, full16, rc);
#pragma unroll
      for (int q = 0; q < 16; q += 2) {
        if (q < 8 || full16) {
          const int i = (c0 + q) >> 1;
          if constexpr (kTwoSum) {
            f32x2 s2, e2;
            two_sum2(h2[i], pack2(rc[q], rc[q + 1]), s2, e2);
            h2[i] = add2(s2, add2(l2[i], e2));  // hi + (lo + e) rounded once to FP32 (2^-24 relative)
          } else {
            h2[i] = add2(h2[i], pack2(rc[q], rc[q + 1]));
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncwarp();
  if (f.lane == 0) mbar_arrive(f.tmem_free);  // the next tile's MMAs may overwrite tensor memory

  const int64_t c_first = (int64_t)tr.n0 + hc;  // first output column of this warp
  const int ncol = (int)(job.cols - c_first < nh ? job.cols - c_first : nh);  // valid columns (may be <= 0)
  // elements of the output (bounds-checked build): 5 npts rows (M-major A) or rows
  const int64_t out_extent = (job.a_mn ? 5 * job.npts : job.rows) * job.ldo;
  if ((reinterpret_cast<uintptr_t>(job.out) & 31) == 0 && (job.ldo & 3) == 0 && (c_first & 3) == 0) {
    // 32-byte aligned row segments: each lane writes its own row, four columns per 32-byte
    // store, straight from registers (shared memory is busy with the MMAs' operand reads and
    // the TMA fills at this point, and waiting for it costs more than the scattered sectors).
    if (orow >= 0) {
      double* __restrict__ const p = job.out + orow * job.ldo + c_first;
#pragma unroll
      for (int c0 = 0; c0 < kHalfN; c0 += 4) {
        if (c0 + 4 <= ncol) {
          if (!QG_STORE_OK(kSiteSplitOut, orow * job.ldo + c_first + c0 + 3, out_extent)) continue;
          const float v0 = lo_f(h2[c0 >> 1]), v1 = hi_f(h2[c0 >> 1]), v2 = lo_f(h2[(c0 >> 1) + 1]),
                      v3 = hi_f(h2[(c0 >> 1) + 1]);
          if (f32_special(v0) || f32_special(v1) || f32_special(v2) || f32_special(v3))
            st_global_v4(p + c0, f32_to_f64_int(v0), f32_to_f64_int(v1), f32_to_f64_int(v2), f32_to_f64_int(v3));
          else
            st_global_v4(p + c0, f32_to_f64_normal(v0), f32_to_f64_normal(v1), f32_to_f64_normal(v2),
                         f32_to_f64_normal(v3));
        } else if (c0 < ncol) {
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (c0 + j < ncol && QG_STORE_OK(kSiteSplitOut, orow * job.ldo + c_first + c0 + j, out_extent))
              p[c0 + j] = f32_to_f64_int(j & 1 ? hi_f(h2[(c0 + j) >> 1]) : lo_f(h2[(c0 + j) >> 1]));
        }
      }
    }
    return true;
  }
  // Otherwise (unaligned rows): eight columns at a time through the transposition buffer.
  const int rr = f.lane >> 3, cc = f.lane & 7;  // read-back: rows rr + 4 i, column cc of the 8
  // The job's fields in registers: the stores below could alias them for the compiler, which
  // would otherwise reload them from global memory after every store.
  double* __restrict__ const out = job.out + c_first + cc;
  const int64_t ldo = job.ldo;
  float* __restrict__ const tb = f.tb;
  int64_t orows[8];  // output row of each read-back row, -1 where there is none
#pragma unroll
  for (int i = 0; i < 8; ++i) orows[i] = __shfl_sync(0xffffffffu, orow, 4 * i + rr);
#pragma unroll
  for (int c0 = 0; c0 < kHalfN; c0 += 8) {
    if (c0 < ncol) {
#pragma unroll
      for (int j = 0; j < 8; ++j) tb[f.lane * kTPitch + j] = j & 1 ? hi_f(h2[(c0 + j) >> 1]) : lo_f(h2[(c0 + j) >> 1]);
      __syncwarp();
      const bool col_ok = c0 + cc < ncol;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float v = tb[(4 * i + rr) * kTPitch + cc];
        if (orows[i] >= 0 && col_ok &&
            QG_STORE_OK(kSiteSplitOut, orows[i] * ldo + c_first + cc + c0, out_extent))
          out[orows[i] * ldo + c0] = f32_to_f64_int(v);
      }
      __syncwarp();
    }
  }
  return true;
}

// Persistent and continuous: CTA b processes tiles b, b + gridDim.x, ... of the launch (tiles
// of one job are ordered column tile fastest, so CTAs running at the same time share A rows in
// L2). The three roles walk the same sequence of (tile, K block) steps with running barrier
// phases, so the producer prefetches the next tile while the fold warps finish the current one;
// the only hand-over between tiles is `tmem_free`: the MMA issuer starts a tile once the fold
// warps have read the previous tile's corrections out of tensor memory (they then write that
// tile's output while the next tile computes).
__global__ void __launch_bounds__(kThreads, 1)
    split_gemm_kernel(const SplitJob* __restrict__ jobs, int njobs, int total_tiles, int* error, const SplitCtl ctl) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* tbuf = (float*)(base + kStages * kMaxStage);
  uint64_t* full = (uint64_t*)(base + kStages * kMaxStage + 8 * kTBuf);
  uint64_t* empty = full + kStages;
  uint64_t* accf = empty + kStages;  // [kBufs] main buffer filled (MMA -> fold warps)
  uint64_t* acce = accf + kBufs;     // [kBufs] main buffer folded (fold warps -> MMA)
  uint64_t* tmem_free = acce + kBufs;  // accumulators of the last tile read out (fold warps -> MMA)
  uint64_t* mma_done = tmem_free + 1;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  const uint32_t tmem_cols = 512;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    *abort_flag = 0;
    for (int s2 = 0; s2 < kStages; ++s2) {
      mbar_init(&full[s2], 1);
      mbar_init(&empty[s2], 1);
    }
    for (int b = 0; b < kBufs; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 8);
    }
    mbar_init(tmem_free, 8);
    mbar_init(mma_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // Registers move from the producer/MMA warpgroup to the two fold warpgroups; each role
  // adjusts its warpgroup's allocation on entry (all four warps of a warpgroup do the same).
  if (warp == 0) {
    reg_dec<kRegsIssue>();
    if (lane == 0) {
      // ---------------- TMA producer
      uint32_t it = 0;  // running K-block index over the CTA's tiles
      bool ok = true;
      for (int tile = blockIdx.x; ok && tile < total_tiles; tile += gridDim.x) {
        const TileRef tr = tile_ref(jobs, njobs, tile);
        const SplitJob& job = *tr.job;
        const uint32_t plane_b = (uint32_t)job.n_tile * kBK * 2;
        const uint32_t stage_bytes = 3 * kPlaneA + 3 * plane_b;
        for (int kb = 0; kb < job.kblocks; ++kb, ++it) {
          const uint32_t s2 = it % kStages, ph = (it / kStages) & 1u;
          if (!wait_or_abort(&empty[s2], ph ^ 1u, abort_flag, ctl.wait_cycles)) {
            set_abort(abort_flag, error, 1);
            ok = false;
            break;
          }
          if (ctl.withhold_loads) continue;  // failure-handling test: nothing completes `full`
          unsigned char* st = base + s2 * kMaxStage;
          mbar_expect_tx(&full[s2], stage_bytes);
          if (job.a_mn) {
            // two 64(M) x 64(K) boxes per plane: M rows m0..m0+63, then m0+64..m0+127
            for (int i = 0; i < 3; ++i) {
              tma_load_2d(st + i * kPlaneA, &job.ta[i], tr.m0, kb * kBK, &full[s2]);
              tma_load_2d(st + i * kPlaneA + kPlaneA / 2, &job.ta[i], tr.m0 + 64, kb * kBK, &full[s2]);
            }
          } else {
            for (int i = 0; i < 3; ++i) tma_load_2d(st + i * kPlaneA, &job.ta[i], kb * kBK, tr.m0, &full[s2]);
          }
          for (int i = 0; i < 3; ++i)
            tma_load_2d(st + 3 * kPlaneA + i * plane_b, &job.tb[i], kb * kBK, tr.n0, &full[s2]);
        }
      }
      // the loads still in flight must land before the shared memory is released
      const uint32_t first = it > (uint32_t)kStages ? it - kStages : 0;
      if (!ctl.withhold_loads)
        for (uint32_t q = first; q < it; ++q) mbar_wait(&full[q % kStages], (q / kStages) & 1u, ctl.wait_cycles);
    }
  } else if (warp == 1) {
    reg_dec<kRegsIssue>();
    if (lane == 0) {
      // ---------------- MMA issuer
      uint32_t it = 0, tl = 0, gi = 0;  // running K block, tile and fold-group indices
      bool ok = true;
      for (int tile = blockIdx.x; ok && tile < total_tiles; tile += gridDim.x, ++tl) {
        const TileRef tr = tile_ref(jobs, njobs, tile);
        const SplitJob& job = *tr.job;
        const int N = job.n_tile;
        const uint32_t plane_b = (uint32_t)N * kBK * 2;
        // D = F32 (bit 4), A = B = BF16 (bits 7, 10), A M-major (bit 15) when a_mn, N >> 3, M >> 4
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((job.a_mn ? 1u : 0u) << 15) |
                               ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
        const bool amn = job.a_mn != 0;
        const uint64_t ka = amn ? 128u : 2u, pa = kPlaneA >> 4, pb = plane_b >> 4;
        // the correction accumulator is read out before reuse
        if (tl > 0 && !wait_or_abort(tmem_free, (tl - 1) & 1u, abort_flag, ctl.wait_cycles)) {
          set_abort(abort_flag, error, 6);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int kb = 0; kb < job.kblocks; ++kb, ++it) {
          const uint32_t s2 = it % kStages, ph = (it / kStages) & 1u, b = gi % kBufs, use = gi / kBufs;
          const bool first = kb % kFold == 0, last = kb % kFold == kFold - 1 || kb == job.kblocks - 1;
          if (first && use > 0 && !wait_or_abort(&acce[b], (use - 1) & 1u, abort_flag, ctl.wait_cycles)) {
            set_abort(abort_flag, error, 2);
            ok = false;
            break;
          }
          if (!wait_or_abort(&full[s2], ph, abort_flag, ctl.wait_cycles)) {
            set_abort(abort_flag, error, 3);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // descriptors in 16-byte units: a K step is 2 (32 bytes along a K-major row) or 128
          // (16 rows of 128 bytes, M-major); planes are kPlaneA / plane_b bytes apart
          const uint32_t sa = smem_u32(base + s2 * kMaxStage);
          const uint64_t da = amn ? sdesc_mn(sa) : sdesc(sa);
          const uint64_t db = sdesc(sa + 3 * kPlaneA);
          const uint32_t main_acc = tmem + (uint32_t)kMaxN * (1 + b);
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk) {
            const uint64_t a = da + kk * ka, bb = db + kk * 2u;
            // (A plane, B plane): main (0,0); corrections (0,1) (1,0) (0,2) (1,1) (2,0)
            umma_six(main_acc, tmem, a, bb, a, bb + pb, a + pa, bb, a, bb + 2 * pb, a + pa, bb + pb, a + 2 * pa, bb, idesc,
                     (first && kk == 0) ? 0u : 1u, (kb | kk) != 0 ? 1u : 0u);
          }
          umma_commit(&empty[s2]);  // frees the stage once these MMAs have read it
          if (last) {
            umma_commit(&accf[b]);  // main buffer b holds this group's product
            ++gi;
          }
        }
      }
      umma_commit(mma_done);  // every MMA issued has completed
      if (!mbar_wait(mma_done, 0, ctl.wait_cycles)) set_abort(abort_flag, error, 5);
    }
  } else if (warp < 4) {
    reg_dec<kRegsIssue>();  // warps 2 and 3: no role (they complete warpgroup 0)
  } else {
    reg_inc();
    // ---------------- fold warps: warp w owns TMEM lanes 32*(w % 4) .. +31 (one row per thread)
    // and column half (w - 4) / 4 of each tile
    const int quarter = warp & 3, half = (warp - 4) >> 2;
    FoldCtx f{tmem + ((uint32_t)(quarter * 32) << 16), tbuf + (size_t)(warp - 4) * 32 * kTPitch, accf, acce,
              tmem_free, abort_flag, error, ctl.wait_cycles, lane, quarter, half};
    uint32_t it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; ok && tile < total_tiles; tile += gridDim.x) {
      const TileRef tr = tile_ref(jobs, njobs, tile);
      ok = fold_tile(f, *tr.job, tr, it);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
  }
}

// ------------------------------------------------------------------ host side
// cuTensorMapEncodeTiled is resolved through the runtime at first use, so the library does not
// link the driver library and still loads on machines without a GPU driver.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Resolved once per process; the initialisation of a function-local static is thread-safe, so
// first calls from several host threads (one per device, say) all see the resolved pointer.
EncodeTiledFn encode_tiled_fn() {
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<EncodeTiledFn>(p);
    cudaGetLastError();
    return nullptr;
  }();
  return fn;
}

bool encode_map(CUtensorMap* map, const void* base, int64_t rows, int64_t kp, int box_rows) {
  EncodeTiledFn encode = encode_tiled_fn();
  if (!encode) return false;
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// M-major A plane [kp][rows]: boxes of 64 rows (inner, 128 bytes) x 64 K.
bool encode_map_mn(CUtensorMap* map, const void* base, int64_t rows, int64_t kp) {
  EncodeTiledFn encode = encode_tiled_fn();
  if (!encode) return false;
  cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)kp};
  cuuint64_t strides[1] = {(cuuint64_t)rows * 2};
  cuuint32_t box[2] = {64, (cuuint32_t)kBK};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// Column tiling of an M-column contraction: the fewest tiles of at most kMaxN columns,
// as equal as multiples of 16 allow.
int tile_cols(int64_t M, int cap = kMaxN) {
  cap = cap < 16 ? 16 : (cap > kMaxN ? kMaxN : cap / 16 * 16);
  const int ntiles = (int)((M + cap - 1) / cap);
  return (int)round_up((M + ntiles - 1) / ntiles, 16);
}

// Describes out[rows][M] = A planes (ap, [3][rows][kp]) x B planes (bp, [3][M][kp])^T as a
// job whose tiles start at tile_begin; returns its tile count, or -1 if a map fails.
int make_job(SplitJob& job, const __nv_bfloat16* ap, int64_t rows, const __nv_bfloat16* bp, int64_t M, int64_t kp,
             double* out, int tile_begin, int n_cap = kMaxN) {
  memset(&job, 0, sizeof job);
  const int n_tile = tile_cols(M, n_cap);
  for (int i = 0; i < 3; ++i)
    if (!encode_map(&job.ta[i], ap + (size_t)i * rows * kp, rows, kp, kBM) ||
        !encode_map(&job.tb[i], bp + (size_t)i * M * kp, M, kp, n_tile))
      return -1;
  job.out = out;
  job.rows = rows;
  job.cols = M;
  job.ldo = M;
  job.kblocks = (int32_t)(kp / kBK);
  job.n_tile = n_tile;
  job.col_tiles = (int32_t)((M + n_tile - 1) / n_tile);
  job.tile_begin = tile_begin;
  return (int)((rows + kBM - 1) / kBM) * job.col_tiles;
}

// The mo_vgl contraction from the fused AO kernel's M-major planes ap ([3][kp][5 pp], pp a
// multiple of 64; operand row (5 g + c) 64 + j = component c of processing slot 64 g + j) into
// out[5 npts][M] (rows 5 perm[s] + c).
int make_job_mn(SplitJob& job, const __nv_bfloat16* ap, int64_t pp, int64_t npts, const int32_t* perm,
                const __nv_bfloat16* bp, int64_t M, int64_t kp, double* out, int tile_begin, int n_cap = kMaxN) {
  memset(&job, 0, sizeof job);
  if (pp % 64 != 0) return -1;
  const int n_tile = tile_cols(M, n_cap);
  const int64_t rows = 5 * pp;
  for (int i = 0; i < 3; ++i)
    if (!encode_map_mn(&job.ta[i], ap + (size_t)i * kp * rows, rows, kp) ||
        !encode_map(&job.tb[i], bp + (size_t)i * M * kp, M, kp, n_tile))
      return -1;
  job.out = out;
  job.rows = rows;
  job.cols = M;
  job.ldo = M;
  job.kblocks = (int32_t)(kp / kBK);
  job.n_tile = n_tile;
  job.col_tiles = (int32_t)((M + n_tile - 1) / n_tile);
  job.tile_begin = tile_begin;
  job.a_mn = 1;
  job.pp = (int32_t)pp;
  job.npts = npts;
  job.perm = perm;
  return (int)((rows + kBM - 1) / kBM) * job.col_tiles;
}

size_t split_smem_bytes() { return 1024 + kStages * (size_t)kMaxStage + 8 * (size_t)kTBuf + 256; }

// One persistent launch over every tile of the njobs jobs at d_jobs (device memory). Returns
// the launch's own status (cudaLaunchKernel), not an earlier error pending in the runtime.
cudaError_t launch_split_jobs(cudaStream_t stream, const SplitJob* d_jobs, int njobs, int total_tiles, int* err,
                              const SplitCtl& ctl = SplitCtl{}) {
  if (total_tiles <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = split_smem_bytes();
  cudaFuncSetAttribute(split_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int grid = total_tiles < sms ? total_tiles : sms;
  void* args[] = {(void*)&d_jobs, (void*)&njobs, (void*)&total_tiles, (void*)&err, (void*)&ctl};
  return cudaLaunchKernel((const void*)split_gemm_kernel, dim3(grid), dim3(kThreads), args, smem, stream);
}

cudaError_t launch_split(Ctx* ctx, const double* src, int64_t rows, int64_t k, int64_t ld, int64_t kp, bool mask5,
                         __nv_bfloat16* planes) {
  const int64_t n = rows * kp;
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  LaunchScope scope(ctx, mask5 ? "split_ao_planes" : "split_planes");
  split_planes_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(src, rows, k, ld, kp, mask5 ? 1 : 0, planes);
  return cudaGetLastError();
}

// The context's launch controls (the failure-handling test hook, when set).
SplitCtl ctl_of(const Ctx* ctx) {
  SplitCtl c;
  if (ctx->split_wait_cycles > 0) c.wait_cycles = ctx->split_wait_cycles;
  c.withhold_loads = ctx->split_withhold_loads;
  return c;
}

}  // namespace

// Splits (once per coefficient set) the MO coefficients [mo][ao] into BF16 planes.
static qmckl_exit_code_device ensure_coef_planes(Ctx* ctx, qmckl_context_device c, int64_t kp) {
  MoBasisData& mo = ctx->mo_basis;
  if (mo.coef_split && mo.split_ao_pad == kp && mo.split_mo_pad == mo.mo_num) return QMCKL_SUCCESS_DEVICE;
  if (mo.coef_split) dfree(ctx, mo.coef_split);
  mo.coef_split = dalloc(ctx, sizeof(__nv_bfloat16) * 3 * mo.mo_num * kp);
  if (!mo.coef_split) return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_provide_mo_basis_mo_vgl_device", nullptr);
  mo.split_ao_pad = kp;
  mo.split_mo_pad = mo.mo_num;
  launch_split(ctx, mo.coefficient, mo.mo_num, ctx->ao_basis.ao_num, ctx->ao_basis.ao_num, kp, false,
               static_cast<__nv_bfloat16*>(mo.coef_split));
  return finish(ctx, c, "qmckl_provide_mo_basis_mo_vgl_device");
}

// Uploads one job and runs its tiles on the context's stream.
static qmckl_exit_code_device run_job(Ctx* ctx, qmckl_context_device c, const SplitJob& job, int tiles, int* err,
                                      const char* name) {
  const char* fn = "qmckl_provide_mo_basis_mo_vgl_device";
  MoBasisData& mo = ctx->mo_basis;
  if (tiles < 0) return fail(c, QMCKL_FAILURE_DEVICE, fn, "cuTensorMapEncodeTiled failed");
  if (!ensure_raw(ctx, &mo.split_job, &mo.split_job_cap, sizeof(SplitJob)))
    return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "split job descriptor");
  if (cudaMemcpyAsync(mo.split_job, &job, sizeof job, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, QMCKL_FAILURE_DEVICE, fn, "job upload failed");
  }
  {
    LaunchScope scope(ctx, name);
    launch_split_jobs(ctx->stream, static_cast<const SplitJob*>(mo.split_job), 1, tiles, err, ctl_of(ctx));
  }
  qmckl_exit_code_device rc = finish(ctx, c, fn);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!ctx->async) {
    int h = 0;
    cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    if (h) return fail(c, QMCKL_FAILURE_DEVICE, fn, "split-BF16 GEMM: a pipeline wait timed out");
  }
  return QMCKL_SUCCESS_DEVICE;
}

// out[rows][M] = split-BF16 product of the A planes ap ([3][rows][kp]) and the coefficients.
static qmckl_exit_code_device contract_planes(Ctx* ctx, qmckl_context_device c, const __nv_bfloat16* ap, int64_t rows,
                                              int64_t kp, int* err, double* out, const char* name) {
  MoBasisData& mo = ctx->mo_basis;
  SplitJob job;
  const int tiles =
      make_job(job, ap, rows, static_cast<const __nv_bfloat16*>(mo.coef_split), mo.mo_num, kp, out, 0);
  return run_job(ctx, c, job, tiles, err, name);
}

// Ensures the A-plane buffer holds rows x kp planes plus the error word; returns the error word.
static int* ensure_a_planes(Ctx* ctx, int64_t rows, int64_t kp) {
  MoBasisData& mo = ctx->mo_basis;
  const size_t need = sizeof(__nv_bfloat16) * 3 * (size_t)rows * (size_t)kp + 256;
  if (!ensure_raw(ctx, &mo.ao_split, &mo.ao_split_cap, need)) return nullptr;
  int* err = reinterpret_cast<int*>(reinterpret_cast<char*>(mo.ao_split) + need - 256);
  cudaMemsetAsync(err, 0, sizeof(int), ctx->stream);
  return err;
}

// out[rows][M] = split-BF16 product of src[rows][A] (FP64, ld = A) and the coefficients.
qmckl_exit_code_device split_contract(Ctx* ctx, qmckl_context_device c, const double* src, int64_t rows, bool mask5,
                                      double* out) {
  const char* fn = "qmckl_provide_mo_basis_mo_vgl_device";
  MoBasisData& mo = ctx->mo_basis;
  const int64_t A = ctx->ao_basis.ao_num, M = mo.mo_num;
  if (rows <= 0 || M <= 0) return QMCKL_SUCCESS_DEVICE;
  const int64_t kp = round_up(A, kBK);
  if (kp / kBK > (int64_t)INT32_MAX || rows > (int64_t)INT32_MAX - kBM)
    return fail(c, QMCKL_FAILURE_DEVICE, fn, "problem too large for the split-BF16 form");
  qmckl_exit_code_device rc = ensure_coef_planes(ctx, c, kp);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  int* err = ensure_a_planes(ctx, rows, kp);
  if (!err) return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "split AO planes");
  __nv_bfloat16* ap = static_cast<__nv_bfloat16*>(mo.ao_split);
  launch_split(ctx, src, rows, A, A, kp, mask5, ap);
  return contract_planes(ctx, c, ap, rows, kp, err, out, mask5 ? "mo_vgl_split_bf16" : "mo_value_split_bf16");
}

// mo_vgl for the current points: the fused AO kernel writes the BF16 planes of the AO
// operand directly (no FP64 ao_vgl round trip), then the tensor-core contraction.
static qmckl_exit_code_device split_mo_vgl(Ctx* ctx, qmckl_context_device c, double* out) {
  const char* fn = "qmckl_provide_mo_basis_mo_vgl_device";
  const int64_t P = ctx->point.num, A = ctx->ao_basis.ao_num, M = ctx->mo_basis.mo_num;
  if (P <= 0 || M <= 0) return QMCKL_SUCCESS_DEVICE;
  const int64_t pp = round_up(P, 64), rows = 5 * pp, kp = round_up(A, kBK);
  if (rows > (int64_t)INT32_MAX - kBM) return fail(c, QMCKL_FAILURE_DEVICE, fn, "problem too large for the split-BF16 form");
  qmckl_exit_code_device rc = ensure_tables(ctx, c);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rc = ensure_coef_planes(ctx, c, kp);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  int* err = ensure_a_planes(ctx, rows, kp);
  if (!err) return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "split AO planes");
  __nv_bfloat16* ap = static_cast<__nv_bfloat16*>(ctx->mo_basis.ao_split);
  const int32_t* perm = point_order(ctx);
  launch_ao_planes(ctx, ctx->ao_basis.tables, ctx->point.coord, P, perm, P, kp, ap);
  SplitJob job;
  const int tiles = make_job_mn(job, ap, pp, P, perm, static_cast<const __nv_bfloat16*>(ctx->mo_basis.coef_split),
                                M, kp, out, 0);
  return run_job(ctx, c, job, tiles, err, "mo_vgl_split_bf16");
}

size_t split_job_bytes() { return sizeof(SplitJob); }

int split_make_job(void* job_host, const void* a_planes, int64_t rows, const void* b_planes, int64_t M, int64_t kp,
                   double* out, int tile_begin, int n_cap) {
  return make_job(*static_cast<SplitJob*>(job_host), static_cast<const __nv_bfloat16*>(a_planes), rows,
                  static_cast<const __nv_bfloat16*>(b_planes), M, kp, out, tile_begin, n_cap);
}

int split_make_job_mn(void* job_host, const void* a_planes, int64_t pp, int64_t npts, const int32_t* perm,
                      const void* b_planes, int64_t M, int64_t kp, double* out, int tile_begin, int n_cap) {
  return make_job_mn(*static_cast<SplitJob*>(job_host), static_cast<const __nv_bfloat16*>(a_planes), pp, npts, perm,
                     static_cast<const __nv_bfloat16*>(b_planes), M, kp, out, tile_begin, n_cap);
}

cudaError_t split_launch_jobs(cudaStream_t stream, const void* jobs, int njobs, int total_tiles, int* err) {
  return launch_split_jobs(stream, static_cast<const SplitJob*>(jobs), njobs, total_tiles, err);
}

int64_t split_k_pad(int64_t ao_num) { return round_up(ao_num, kBK); }

qmckl_exit_code_device split_prepare_coef(Ctx* ctx, qmckl_context_device c, int64_t kp) {
  return ensure_coef_planes(ctx, c, kp);
}

void* split_a_planes(Ctx* ctx, int64_t rows, int64_t kp) {
  return ensure_a_planes(ctx, rows, kp) ? ctx->mo_basis.ao_split : nullptr;
}

// Point ranges of the host-buffer path: sizes in the ratio 1 : ratio : ratio^2 ... (ratio 1: equal
// ranges), multiples of 64 points (the AO planes' block), the last range taking the rest.
// Ranges sized by the contraction's waves: each range but the last has the most points (a
// multiple of 64) whose tiles fill `waves` waves of one tile per SM, with waves = 1 unless that
// needs more than max_ranges ranges; the last range takes the rest. A range whose tiles end a
// wave exactly leaves no SM idle at its end: on the medium workload (M = 300, two column tiles
// of 150) ranges of 1920 points, 150 tiles each.
std::vector<int64_t> wave_plan(int64_t P, int64_t M, int sms, int max_ranges) {
  const int64_t col_tiles = (M + tile_cols(M) - 1) / tile_cols(M);
  int64_t n = 64;
  for (int64_t waves = 1;; ++waves) {
    const int64_t row_tiles = waves * sms / col_tiles;  // rows 5 n <= row_tiles * kBM
    n = row_tiles * kBM / 5 / 64 * 64;
    if (n >= 64 && (P + n - 1) / n <= max_ranges) break;
    if (row_tiles * kBM / 5 >= P) break;
  }
  if (n < 64) n = 64;
  std::vector<int64_t> sizes;
  for (int64_t done = 0; done < P; done += n) sizes.push_back(n < P - done ? n : P - done);
  return sizes;
}

std::vector<int64_t> chunk_plan(int64_t P, int chunks, double ratio) {
  std::vector<int64_t> sizes;
  double total = 0.0, w = 1.0;
  for (int k = 0; k < chunks; ++k, w *= ratio) total += w;
  int64_t done = 0;
  w = 1.0;
  for (int k = 0; k < chunks && done < P; ++k, w *= ratio) {
    int64_t n = k == chunks - 1 ? P - done : round_up((int64_t)(P * (w / total)), 64);
    if (n < 64) n = 64;
    if (n > P - done) n = P - done;
    sizes.push_back(n);
    done += n;
  }
  return sizes;
}

// mo_vgl of the split-BF16 form for a caller's host buffer: the points are processed in ranges
// (contiguous, each ordered on its own) whose rows of the cached mo_vgl are copied to the host on
// a second stream while the next range computes, so the device-to-host transfer (~193 GB/s over
// the host link here, 2.54 ms for the medium workload's 491.5 MB, the same for every buffer kind
// and copy method measured) overlaps the compute. The ranges' contraction jobs are encoded and
// uploaded once per shape and buffer set, and reused while those stay the same.
qmckl_exit_code_device split_mo_vgl_to_host(Ctx* ctx, qmckl_context_device c, double* host_dst, int chunks,
                                            double ratio) {
  const char* fn = "qmckl_get_mo_basis_mo_vgl_device";
  const int64_t P = ctx->point.num, A = ctx->ao_basis.ao_num, M = ctx->mo_basis.mo_num;
  MoBasisData& mo = ctx->mo_basis;
  AoBasisData& ao = ctx->ao_basis;
  const int64_t kp = round_up(A, kBK);
  std::vector<int64_t> sizes;
  if (chunks > 0) {
    chunks = chunks > kMaxHostChunks ? kMaxHostChunks : chunks;
    sizes = chunk_plan(P, chunks, ratio);
  } else {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    sizes = wave_plan(P, M, sms, kMaxHostChunks);
    ratio = 0.0;
  }
  const int nc = (int)sizes.size();
  int64_t pc = 0;  // points of the largest range
  for (int64_t n : sizes) pc = n > pc ? n : pc;
  pc = round_up(pc, 64);
  const int64_t pp = round_up(P, 64);
  if (5 * pc > (int64_t)INT32_MAX - kBM) return fail(c, QMCKL_FAILURE_DEVICE, fn, "problem too large for the split-BF16 form");
  qmckl_exit_code_device rc = ensure_tables(ctx, c);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rc = ensure_coef_planes(ctx, c, kp);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!ensure(ctx, &mo.mo_vgl, &mo.mo_vgl_cap, sizeof(double) * 5 * M * P))
    return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "mo_vgl");
  int* err = ensure_a_planes(ctx, 5 * pc, kp);
  if (!err) return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "split AO planes");
  void* perm = ao.point_perm;
  void* keys = ao.point_keys;
  void* counts = ao.cell_counts;
  const bool ok = ensure_raw(ctx, &perm, &ao.perm_cap, sizeof(int32_t) * pp) &&
                  ensure_raw(ctx, &keys, &ao.keys_cap, sizeof(int32_t) * pp) &&
                  ensure_raw(ctx, &counts, &ao.counts_cap, sizeof(int32_t) * kOrderCells * (size_t)nc);
  ao.point_perm = static_cast<int32_t*>(perm);
  ao.point_keys = static_cast<int32_t*>(keys);
  ao.cell_counts = static_cast<int32_t*>(counts);
  ao.perm_date = 0;  // the buffer holds chunk-local orders from here on
  if (!ok) return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "point order buffers");
  if (!ctx->copy_stream && cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, QMCKL_FAILURE_DEVICE, fn, "stream creation failed");
  }
  for (int k = 0; k < nc; ++k)
    if (!ctx->chunk_done[k] && cudaEventCreateWithFlags(&ctx->chunk_done[k], cudaEventDisableTiming) != cudaSuccess) {
      ctx->chunk_done[k] = nullptr;
      cudaGetLastError();
      return fail(c, QMCKL_FAILURE_DEVICE, fn, "event creation failed");
    }
  __nv_bfloat16* ap = static_cast<__nv_bfloat16*>(mo.ao_split);
  // the ranges' jobs and first points, encoded and uploaded once for this shape and these buffers
  // (range k's processing order lives at point_perm + its first point)
  HostChunkJobs& hj = mo.host_jobs;
  const HostChunkKey key{P, M, kp, nc, ratio, ap, mo.coef_split, mo.mo_vgl, ao.point_perm};
  const size_t job_bytes = sizeof(SplitJob) * (size_t)nc;
  if (!(hj.key == key) || !hj.jobs) {
    hj.key = HostChunkKey{};
    if (!ensure_raw(ctx, &hj.jobs, &hj.jobs_cap, job_bytes + sizeof(int64_t) * (size_t)(nc + 1)))
      return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "split job descriptors");
    std::vector<SplitJob> jobs((size_t)nc);
    std::vector<int64_t> bounds((size_t)nc + 1);
    int64_t off = 0;
    for (int k = 0; k < nc; ++k) {
      const int64_t n = sizes[k];
      bounds[k] = off;
      hj.tiles[k] = make_job_mn(jobs[k], ap, round_up(n, 64), n, ao.point_perm + off,
                                static_cast<const __nv_bfloat16*>(mo.coef_split), M, kp, mo.mo_vgl + 5 * off * M, 0);
      if (hj.tiles[k] < 0) return fail(c, QMCKL_FAILURE_DEVICE, fn, "cuTensorMapEncodeTiled failed");
      off += n;
    }
    bounds[nc] = off;
    unsigned char* dst = static_cast<unsigned char*>(hj.jobs);
    if (cudaMemcpy(dst, jobs.data(), job_bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dst + job_bytes, bounds.data(), sizeof(int64_t) * bounds.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      cudaGetLastError();
      return fail(c, QMCKL_FAILURE_DEVICE, fn, "job upload failed");
    }
    hj.key = key;
  }
  const SplitJob* d_jobs = static_cast<const SplitJob*>(hj.jobs);
  const int64_t* d_bounds = reinterpret_cast<const int64_t*>(static_cast<const unsigned char*>(hj.jobs) + job_bytes);
  // every range's processing order in one pass (three launches instead of three per range)
  cudaError_t e = launch_point_order_ranges(ctx, ao.tables, ctx->point.coord, P, d_bounds, nc, ao.point_keys,
                                            ao.cell_counts, ao.point_perm);
  int64_t off = 0;
  for (int k = 0; k < nc && e == cudaSuccess; ++k) {
    const int64_t n = sizes[k];
    const double* coord = ctx->point.coord + off;  // rows of [3][P], slice of n points
    e = launch_ao_planes(ctx, ao.tables, coord, P, ao.point_perm + off, n, kp, ap);
    if (e != cudaSuccess) break;
    {
      LaunchScope scope(ctx, "mo_vgl_split_bf16");
      e = launch_split_jobs(ctx->stream, d_jobs + k, 1, hj.tiles[k], err, ctl_of(ctx));
    }
    if (e == cudaSuccess) e = cudaEventRecord(ctx->chunk_done[k], ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->chunk_done[k], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(host_dst + 5 * off * M, mo.mo_vgl + 5 * off * M, sizeof(double) * 5 * n * M,
                          cudaMemcpyDeviceToHost, ctx->copy_stream);
    off += n;
  }
  cudaError_t e2 = cudaStreamSynchronize(ctx->copy_stream);
  cudaError_t e3 = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = e2 != cudaSuccess ? e2 : e3;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, QMCKL_FAILURE_DEVICE, fn, cudaGetErrorString(e));
  }
  int h = 0;
  cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  if (h) return fail(c, QMCKL_FAILURE_DEVICE, fn, "split-BF16 GEMM: a pipeline wait timed out");
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device provide_mo_split(Ctx* ctx, qmckl_context_device c, double* dst, bool value_only) {
  if (value_only) return split_contract(ctx, c, ctx->ao_basis.ao_value, ctx->point.num, false, dst);
  return split_mo_vgl(ctx, c, dst);
}

}  // namespace qg

// ======================================================================================
// Split-BF16 contraction that allocates nothing.
//
// Some callers cannot let a library allocate device memory: codes that hand all device
// memory to their own pool allocator at start-up (a cudaMalloc from a library then fails or
// fragments the pool), hosts that load this library as a plug-in and forbid it to allocate
// on its own, and latency-critical loops where cudaMalloc/cudaFree would synchronise the
// device and stall other streams. For them this entry point keeps its scratch memory (the
// BF16 operand planes and an error word) in the file-scope device array below, which every
// GPU that loads the library holds until the process exits. Its size bounds the problem:
// ao_num <= 2048 and mo_num <= 1024; any number of rows is accepted (rows are processed in
// chunks of kNoAllocChunkRows that reuse the array in stream order).
// ======================================================================================
namespace qg {
namespace {

constexpr int64_t kNoAllocMaxAo = 2048;
constexpr int64_t kNoAllocMaxMo = 1024;
constexpr int64_t kNoAllocChunkRows = 1280;  // a multiple of 128 (tile rows) and of 5 (vgl rows of a point)
constexpr size_t kNoAllocBytes =
    sizeof(__nv_bfloat16) * 3 * (size_t)(kNoAllocMaxMo + kNoAllocChunkRows) * (size_t)kNoAllocMaxAo + 2048;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];
// Layout of the array: B planes [3][mo_num][kp], A planes [3][chunk rows][kp] (together at most
// kNoAllocBytes - 2048 bytes), the job descriptor at kNoAllocBytes - 2048, the error word at
// kNoAllocBytes - 256.
static_assert(sizeof(SplitJob) <= 2048 - 256, "the job descriptor must end below the error word");

// Host-side device addresses of the array, one per device, resolved on each device's first
// call (with that device current). A host pointer to the symbol is not a device address.
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

}  // namespace

}  // namespace qg

extern "C" qmckl_exit_code_device qmckl_mo_contract_split_bf16_noalloc_device(const double* ao, int64_t rows,
                                                                              int64_t ao_num,
                                                                              const double* coefficient,
                                                                              int64_t mo_num, int32_t vgl_mask,
                                                                              double* out, void* cuda_stream) {
  using namespace qg;
  if (!ao) return QMCKL_INVALID_ARG_1_DEVICE;
  if (rows < 0 || (vgl_mask && rows % 5 != 0)) return QMCKL_INVALID_ARG_2_DEVICE;
  if (ao_num < 1 || ao_num > kNoAllocMaxAo) return QMCKL_INVALID_ARG_3_DEVICE;
  if (!coefficient) return QMCKL_INVALID_ARG_4_DEVICE;
  if (mo_num < 1 || mo_num > kNoAllocMaxMo) return QMCKL_INVALID_ARG_5_DEVICE;
  if (vgl_mask != 0 && vgl_mask != 1) return QMCKL_INVALID_ARG_6_DEVICE;
  if (!out) return QMCKL_INVALID_ARG_7_DEVICE;
  if (rows == 0) return QMCKL_SUCCESS_DEVICE;
  cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return QMCKL_FAILURE_DEVICE;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return QMCKL_FAILURE_DEVICE;
      g_noalloc_ptr[dev] = p;
    }
    scratch = g_noalloc_ptr[dev];
  }

  const int64_t kp = round_up(ao_num, kBK);
  const int64_t M = mo_num;
  __nv_bfloat16* bplanes = static_cast<__nv_bfloat16*>(scratch);
  __nv_bfloat16* aplanes = bplanes + 3 * M * kp;
  int* err = reinterpret_cast<int*>(static_cast<unsigned char*>(scratch) + kNoAllocBytes - 256);
  if (cudaMemsetAsync(err, 0, sizeof(int), stream) != cudaSuccess) return QMCKL_FAILURE_DEVICE;

  SplitJob* djob = reinterpret_cast<SplitJob*>(static_cast<unsigned char*>(scratch) + kNoAllocBytes - 2048);

  // Every launch's own status is checked where it is issued (cudaLaunchKernel returns it), so an
  // error pending from the caller's earlier work is neither reported as this call's nor cleared.
  auto split = [&](const double* src, int64_t n, int64_t ld, bool mask, __nv_bfloat16* dst) {
    int64_t blocks = (n * kp + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    int64_t k = ao_num;
    int m5 = mask ? 1 : 0;
    void* args[] = {(void*)&src, (void*)&n, (void*)&k, (void*)&ld, (void*)&kp, (void*)&m5, (void*)&dst};
    return cudaLaunchKernel((const void*)split_planes_kernel, dim3((unsigned)blocks), dim3(256), args, 0, stream);
  };
  if (split(coefficient, M, ao_num, false, bplanes) != cudaSuccess) return QMCKL_FAILURE_DEVICE;

  for (int64_t r0 = 0; r0 < rows; r0 += kNoAllocChunkRows) {
    const int64_t n = rows - r0 < kNoAllocChunkRows ? rows - r0 : kNoAllocChunkRows;
    if (split(ao + r0 * ao_num, n, ao_num, vgl_mask != 0, aplanes) != cudaSuccess) return QMCKL_FAILURE_DEVICE;
    SplitJob job;
    const int tiles = make_job(job, aplanes, n, bplanes, M, kp, out + r0 * M, 0);
    if (tiles < 0) return QMCKL_FAILURE_DEVICE;
    // the descriptor lives in the array too; the copy is ordered after the previous chunk's kernel
    if (cudaMemcpyAsync(djob, &job, sizeof job, cudaMemcpyHostToDevice, stream) != cudaSuccess)
      return QMCKL_FAILURE_DEVICE;
    if (launch_split_jobs(stream, djob, 1, tiles, err) != cudaSuccess) return QMCKL_FAILURE_DEVICE;
  }
  int h = 0;
  if (cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return QMCKL_FAILURE_DEVICE;
  return h ? QMCKL_FAILURE_DEVICE : QMCKL_SUCCESS_DEVICE;
}
