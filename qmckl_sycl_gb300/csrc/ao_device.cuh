// Device helpers shared by the fused AO kernels (ao_kernels.cu) and the adjoint kernels
// (vjp.cu): the per-warp staging buffer, bit-pattern helpers and the exponential, so that
// the adjoint recomputes every radial with exactly the forward kernel's arithmetic.
#pragma once

#include <cstdint>

namespace qg {
namespace dev {

constexpr int kStage = 8;          // AOs staged per warp between flushes
constexpr int kPad = 33;           // 32 points + 1 (bank-conflict padding), in doubles
constexpr unsigned kFull = 0xffffffffu;

template <int NC>
struct Stage {
  double v[NC][kStage][kPad];
  int64_t pidx[32];  // point index of each lane (-1: no point)
};

// The bit pattern of x through an opaque move: the compiler would otherwise turn tests such as
// (bits << 1) == 0 or bits == bits(1.0) back into FP64 compares, which run on the FP64 pipe
// (2.4 per AO in the split-BF16 planes kernel, 16 % of its FP64 instructions).
__device__ __forceinline__ uint64_t bits_of(double x) {
  uint64_t r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ bool is_one(double f) { return bits_of(f) == 0x3FF0000000000000ull; }

// ---------------------------------------------------------------- exponential
// e^(-x) for 0 <= x <= 27.7 (the screened range: fl(a r2) <= 27.631...), Tang's method:
// x = (n/32) ln 2 + r with |r| <= ln2/64, e^-x = 2^(n>>5) * 2^((n&31)/32) * e^r.
constexpr double kInvL = 46.166241308446828;               // 32 / ln 2 (only rounds n)
constexpr double kShifter = 6755399441055744.0;            // 1.5 * 2^52: rounds to an integer
constexpr double kL1 = 0.6931471805599453094 / 32.0;       // double nearest ln 2, / 32 (exact)
constexpr double kL2 = 2.3190468138462996e-17 / 32.0;      // ln 2 - that double, / 32

__device__ __forceinline__ double exp_neg(double x, const double* __restrict__ thi, const double* __restrict__ tlo) {
  const double y = -x;
  const double t = fma(y, kInvL, kShifter);
  const int n = __double2loint(t);
  const double nd = t - kShifter;
  double r = fma(-nd, kL1, y);
  r = fma(-nd, kL2, r);
  double p = fma(r, 1.0 / 720.0, 1.0 / 120.0);
  p = fma(p, r, 1.0 / 24.0);
  p = fma(p, r, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = p * r;  // e^r - 1
  const int j = n & 31, m = n >> 5;
  const double th = thi[j];
  const double res = fma(th, p, tlo[j]) + th;
  return __longlong_as_double(__double_as_longlong(res) + ((long long)m << 52));
}


// Loads the exponential's table (2^(j/32) as hi + lo) into shared memory.
__device__ __forceinline__ void load_exp_table(const double* __restrict__ hi, const double* __restrict__ lo,
                                               double* thi, double* tlo) {
  for (int i = threadIdx.x; i < 32; i += blockDim.x) {
    thi[i] = hi[i];
    tlo[i] = lo[i];
  }
}

}  // namespace dev
}  // namespace qg
