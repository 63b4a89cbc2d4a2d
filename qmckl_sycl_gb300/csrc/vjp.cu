// Adjoint form: vector-Jacobian products of the AO / MO vgl for sm_103a (no counterpart in the
// reference, which has no derivatives with respect to its parameters).
//
// For L = sum_{p,l,m} W[p][l][m] mo_vgl[p][l][m]:
//   dL/dC            = W^T (5P x M)^T . ao_vgl_masked (5P x A)   split-K DMMA GEMM, fixed-order sum
//   Gbar (5P x A)    = W . C                                     DMMA GEMM (adjoint of the AO vgl)
//   dL/dexponent,
//   dL/dcoord        = adjoint AO kernel below, from Gbar
// The mask is the MO kernel's zero-value skip (src/qmckl_mo_sycl.cpp:40 of qmckl_sycl): an AO
// whose value is exactly zero at a point contributes nothing there, so no gradient flows
// through any of its components. Screening decisions are constants.
//
// The adjoint AO kernel recomputes the shell radials instead of reading stored ones: one lane
// per point, warp tasks of 32 points x one nucleus chunk as in the forward kernel, the same
// screening bit tests and the same exponential (ao_device.cuh), so the recomputed AO values,
// and hence the mask, are the forward kernel's bit for bit. Per shell it forms the radial sums
//   R = sum v, R1 = sum -a v, R2 = sum a^2 v, R3 = sum -a^3 v      (v = c e^{-a r^2})
// (R1..R3 are the derivatives of R with respect to r^2), from which every AO component and its
// first derivatives in x, y, z follow:
//   ao_0 = f P R,  ao_d = f (P_d R + 2 x_d R1 P),
//   ao_4 = f (lap(P) R + P (6 R1 + 4 r^2 R2) + 4 l R1 P)          (Euler: x . grad P = l P)
// Exponent gradient: the adjoints of (R, R1, R2) per shell, times dR/da = -r^2 v,
// dR1/da = v (a r^2 - 1), dR2/da = a v (2 - a r^2), reduced over the warp's points in a fixed
// order and written per (point group, primitive); a second kernel sums the groups in order.
// Coordinate gradient: per point, per component, the adjoint-weighted x/y/z derivatives of the
// five outputs (third derivatives of the Gaussian for the Laplacian's gradient), summed over
// the point's nucleus chunks in a fixed order. Every result is deterministic.
#include <cstdint>

#include "ao_device.cuh"
#include "internal.hpp"

namespace qg {
namespace {

using namespace dev;

constexpr int kVjpWarps = 4;

struct VjpArgs {
  const NucleusEntry* nuclei;
  const ShellEntry* shells;
  const PrimEntry* prims;
  const double* aof;
  const NucleusChunk* chunks;
  const ExpTable* exp_table;
  const double* coord;     // [3][P]
  const int32_t* perm;     // processing order of the points, or null
  const double* gbar;      // [P][5][A]: adjoint of ao_vgl
  double* alpha_part;      // [groups][prim_num] (packed primitives), or null
  double* coord_part;      // [chunk_num][P][3], or null
  int64_t point_num;
  int64_t ao_num;
  int64_t task_num;
  int chunk_num;
  int prim_num;
  int mask;                // apply the MO kernel's zero-value skip
};

// The adjoint rows of the warp's 32 points for a window of kStage consecutive AOs, loaded
// through shared memory so that global reads are row segments.
struct Reader {
  Stage<5>* st;
  const double* g;
  int64_t A;
  int nvalid;
  int lane;
  int64_t base;
  int64_t end;

  __device__ __forceinline__ void load(int64_t i) {
    __syncwarp();
    base = i;
    end = i + kStage < A ? i + kStage : A;
    const int n = (int)(end - base);
    const int total = nvalid * 5 * kStage;
    for (int t = lane; t < total; t += 32) {
      const int j = t & (kStage - 1);
      const int rest = t / kStage;
      const int c = rest % 5;
      const int q = rest / 5;
      if (j < n) st->v[c][j][q] = __ldg(g + (5 * st->pidx[q] + c) * A + base + j);
    }
    __syncwarp();
  }
  __device__ __forceinline__ void get(int64_t i, double (&out)[5]) {
    if (i >= end) load(i);
#pragma unroll
    for (int c = 0; c < 5; ++c) out[c] = lane < nvalid ? st->v[c][i - base][lane] : 0.0;
  }
};

// Per-lane radial quantities of the current shell.
struct Rad {
  double x, y, z, r2;
  double R, R1, R2, R3;
  int l;
};

// falling(e, d) * t^(e - d): the d-th derivative of t^e, from the power table T.
template <int E, int D>
__device__ __forceinline__ double pw(const double (&T)[4]) {
  if constexpr (D > E) {
    return 0.0;
  } else {
    double f = 1.0;
#pragma unroll
    for (int i = 0; i < D; ++i) f *= (double)(E - i);
    return f * T[E - D];
  }
}

// Accumulates one Cartesian component's contributions (adjoint g[5] of its five outputs,
// AO factor f) to the shell's radial adjoints and to the point's coordinate gradient.
__device__ __forceinline__ void vjp_accumulate(const Rad& q, double f, const double (&g)[5], double P,
                                               const double (&Pj)[3], const double (&Pjd)[3][3],
                                               const double (&dlapP)[3], double& Rb, double& R1b, double& R2b,
                                               double (&de)[3], bool want_alpha, bool want_coord) {
  const double lapP = Pjd[0][0] + Pjd[1][1] + Pjd[2][2];
  const double xv[3] = {q.x, q.y, q.z};
  const double S1 = g[1] * q.x + g[2] * q.y + g[3] * q.z;
  const double S2 = g[1] * Pj[0] + g[2] * Pj[1] + g[3] * Pj[2];
  if (want_alpha) {
    Rb += f * (g[0] * P + S2 + g[4] * lapP);
    R1b += f * (2.0 * P * S1 + g[4] * (6.0 + 4.0 * q.l) * P);
    R2b += f * (g[4] * 4.0 * q.r2 * P);
  }
  if (want_coord) {
    const double K1 = (4.0 * q.l + 6.0) * q.R1 + 4.0 * q.r2 * q.R2;
    const double K2 = (8.0 * q.l + 20.0) * q.R2 + 8.0 * q.r2 * q.R3;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double HPj = g[1] * Pjd[j][0] + g[2] * Pjd[j][1] + g[3] * Pjd[j][2];
      const double xj = xv[j];
      double C = g[0] * (Pj[j] * q.R + 2.0 * xj * q.R1 * P);
      C += q.R * HPj + 2.0 * q.R1 * (Pj[j] * S1 + xj * S2 + P * g[1 + j]) + 4.0 * xj * q.R2 * P * S1;
      C += g[4] * (dlapP[j] * q.R + 2.0 * xj * q.R1 * lapP + Pj[j] * K1 + xj * P * K2);
      de[j] += f * C;
    }
  }
}

// Reads the component's adjoint and applies the zero-value mask: ao_0 is recomputed with the
// forward kernel's exact operations (P = X[a] * (Y[b] * Z[c]), times R, times f unless f == 1).
__device__ __forceinline__ bool load_adjoint(Reader& rd, int64_t ao, double P, double R, double f, bool scr,
                                             int mask, double (&g)[5]) {
  rd.get(ao, g);
  double a0 = P * R;
  if (!is_one(f)) a0 *= f;
  if (scr || (mask && a0 == 0.0)) {
#pragma unroll
    for (int c = 0; c < 5; ++c) g[c] = 0.0;
    return false;
  }
  return true;
}

template <int a, int b, int c>
__device__ __forceinline__ void vjp_cart(Reader& rd, const double (&X)[4], const double (&Y)[4], const double (&Z)[4],
                                         const Rad& q, double f, int64_t ao, bool scr, int mask, double& Rb,
                                         double& R1b, double& R2b, double (&de)[3], bool want_alpha,
                                         bool want_coord) {
  const double yz = Y[b] * Z[c];
  const double P = X[a] * yz;
  double g[5];
  if (!load_adjoint(rd, ao, P, q.R, f, scr, mask, g)) return;
  const double Pj[3] = {pw<a, 1>(X) * yz, X[a] * pw<b, 1>(Y) * Z[c], X[a] * Y[b] * pw<c, 1>(Z)};
  const double Pjd[3][3] = {
      {pw<a, 2>(X) * yz, pw<a, 1>(X) * pw<b, 1>(Y) * Z[c], pw<a, 1>(X) * Y[b] * pw<c, 1>(Z)},
      {pw<a, 1>(X) * pw<b, 1>(Y) * Z[c], X[a] * pw<b, 2>(Y) * Z[c], X[a] * pw<b, 1>(Y) * pw<c, 1>(Z)},
      {pw<a, 1>(X) * Y[b] * pw<c, 1>(Z), X[a] * pw<b, 1>(Y) * pw<c, 1>(Z), X[a] * Y[b] * pw<c, 2>(Z)}};
  const double dlapP[3] = {
      pw<a, 3>(X) * yz + pw<a, 1>(X) * pw<b, 2>(Y) * Z[c] + pw<a, 1>(X) * Y[b] * pw<c, 2>(Z),
      pw<a, 2>(X) * pw<b, 1>(Y) * Z[c] + X[a] * pw<b, 3>(Y) * Z[c] + X[a] * pw<b, 1>(Y) * pw<c, 2>(Z),
      pw<a, 2>(X) * Y[b] * pw<c, 1>(Z) + X[a] * pw<b, 2>(Y) * pw<c, 1>(Z) + X[a] * Y[b] * pw<c, 3>(Z)};
  vjp_accumulate(q, f, g, P, Pj, Pjd, dlapP, Rb, R1b, R2b, de, want_alpha, want_coord);
}

// The shell's components in the reference's order (a descending, then b descending).
template <int L>
__device__ __forceinline__ void vjp_shell_fixed(Reader& rd, const double (&X)[4], const double (&Y)[4],
                                                const double (&Z)[4], const Rad& q, const double* __restrict__ aof,
                                                int64_t ao0, bool scr, int mask, double& Rb, double& R1b,
                                                double& R2b, double (&de)[3], bool wa, bool wc) {
#define QG_VJP(A_, B_, C_, K_) \
  vjp_cart<A_, B_, C_>(rd, X, Y, Z, q, __ldg(aof + ao0 + K_), ao0 + K_, scr, mask, Rb, R1b, R2b, de, wa, wc)
  if constexpr (L == 0) {
    QG_VJP(0, 0, 0, 0);
  } else if constexpr (L == 1) {
    QG_VJP(1, 0, 0, 0);
    QG_VJP(0, 1, 0, 1);
    QG_VJP(0, 0, 1, 2);
  } else if constexpr (L == 2) {
    QG_VJP(2, 0, 0, 0);
    QG_VJP(1, 1, 0, 1);
    QG_VJP(1, 0, 1, 2);
    QG_VJP(0, 2, 0, 3);
    QG_VJP(0, 1, 1, 4);
    QG_VJP(0, 0, 2, 5);
  } else {
    QG_VJP(3, 0, 0, 0);
    QG_VJP(2, 1, 0, 1);
    QG_VJP(2, 0, 1, 2);
    QG_VJP(1, 2, 0, 3);
    QG_VJP(1, 1, 1, 4);
    QG_VJP(1, 0, 2, 5);
    QG_VJP(0, 3, 0, 6);
    QG_VJP(0, 2, 1, 7);
    QG_VJP(0, 1, 2, 8);
    QG_VJP(0, 0, 3, 9);
  }
#undef QG_VJP
}

__device__ __forceinline__ double pwr(int e, int d, const double* T) {
  if (d > e) return 0.0;
  double f = 1.0;
  for (int i = 0; i < d; ++i) f *= (double)(e - i);
  return f * T[e - d];
}

// l >= 4: the same formulas with run-time exponents (powers in local memory).
__device__ __noinline__ void vjp_shell_generic(Reader& rd, const Rad& q, const double* __restrict__ aof, int64_t ao0,
                                               bool scr, int mask, double& Rb, double& R1b, double& R2b,
                                               double (&de)[3], bool wa, bool wc) {
  double X[kMaxL + 1], Y[kMaxL + 1], Z[kMaxL + 1];
  X[0] = Y[0] = Z[0] = 1.0;
  for (int i = 1; i <= q.l; ++i) {
    X[i] = X[i - 1] * q.x;
    Y[i] = Y[i - 1] * q.y;
    Z[i] = Z[i - 1] * q.z;
  }
  int k = 0;
  for (int a = q.l; a >= 0; --a)
    for (int b = q.l - a; b >= 0; --b, ++k) {
      const int c = q.l - a - b;
      const double yz = Y[b] * Z[c];
      const double P = X[a] * yz;
      const double f = __ldg(aof + ao0 + k);
      double g[5];
      if (!load_adjoint(rd, ao0 + k, P, q.R, f, scr, mask, g)) continue;
      const double Pj[3] = {pwr(a, 1, X) * yz, X[a] * pwr(b, 1, Y) * Z[c], X[a] * Y[b] * pwr(c, 1, Z)};
      const double Pjd[3][3] = {
          {pwr(a, 2, X) * yz, pwr(a, 1, X) * pwr(b, 1, Y) * Z[c], pwr(a, 1, X) * Y[b] * pwr(c, 1, Z)},
          {pwr(a, 1, X) * pwr(b, 1, Y) * Z[c], X[a] * pwr(b, 2, Y) * Z[c], X[a] * pwr(b, 1, Y) * pwr(c, 1, Z)},
          {pwr(a, 1, X) * Y[b] * pwr(c, 1, Z), X[a] * pwr(b, 1, Y) * pwr(c, 1, Z), X[a] * Y[b] * pwr(c, 2, Z)}};
      const double dlapP[3] = {
          pwr(a, 3, X) * yz + pwr(a, 1, X) * pwr(b, 2, Y) * Z[c] + pwr(a, 1, X) * Y[b] * pwr(c, 2, Z),
          pwr(a, 2, X) * pwr(b, 1, Y) * Z[c] + X[a] * pwr(b, 3, Y) * Z[c] + X[a] * pwr(b, 1, Y) * pwr(c, 2, Z),
          pwr(a, 2, X) * Y[b] * pwr(c, 1, Z) + X[a] * pwr(b, 2, Y) * pwr(c, 1, Z) + X[a] * Y[b] * pwr(c, 3, Z)};
      vjp_accumulate(q, f, g, P, Pj, Pjd, dlapP, Rb, R1b, R2b, de, wa, wc);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__global__ void __launch_bounds__(kVjpWarps * 32) vjp_ao_kernel(const VjpArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* thi = reinterpret_cast<double*>(smem_raw);
  double* tlo = thi + 32;
  load_exp_table(a.exp_table->hi, a.exp_table->lo, thi, tlo);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t task = (int64_t)blockIdx.x * kVjpWarps + warp;
  if (task >= a.task_num) return;  // warp-uniform
  const int64_t group = task / a.chunk_num;
  const int ch = (int)(task - group * a.chunk_num);
  const int64_t p0 = group * 32;
  const int64_t P = a.point_num;
  const int nvalid = P - p0 < 32 ? (int)(P - p0) : 32;
  const int64_t slot = p0 + (lane < nvalid ? lane : nvalid - 1);
  const int64_t p = a.perm ? (int64_t)a.perm[slot] : slot;
  const double ex = a.coord[p], ey = a.coord[P + p], ez = a.coord[2 * P + p];
  const bool wa = a.alpha_part != nullptr, wc = a.coord_part != nullptr;

  Stage<5>* st = reinterpret_cast<Stage<5>*>(smem_raw + 512) + warp;
  st->pidx[lane] = p;
  Reader rd{st, a.gbar, a.ao_num, nvalid, lane, 0, 0};
  double de[3] = {0.0, 0.0, 0.0};
  double* apart = wa ? a.alpha_part + group * (int64_t)a.prim_num : nullptr;
  const int64_t apart_extent = (P + 31) / 32 * (int64_t)a.prim_num;  // bounds-checked build
  const NucleusChunk cj = a.chunks[ch];

  for (int n = cj.nucl_begin; n < cj.nucl_end; ++n) {
    const NucleusEntry& N = a.nuclei[n];
    const double x = ex - N.x, y = ey - N.y, z = ez - N.z;
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    const uint64_t r2b = bits_of(r2);
    const bool scr = r2b > N.screen_bits;
    if (__all_sync(kFull, scr)) {
      if (wa && N.shell_end > N.shell_begin) {
        const int k0 = a.shells[N.shell_begin].prim_begin, k1 = a.shells[N.shell_end - 1].prim_end;
        for (int k = k0 + lane; k < k1; k += 32)
          if (QG_STORE_OK(kSiteVjp, group * (int64_t)a.prim_num + k, apart_extent)) apart[k] = 0.0;
      }
      continue;
    }
    double X[4], Y[4], Z[4];
    X[0] = Y[0] = Z[0] = 1.0;
    X[1] = x;
    Y[1] = y;
    Z[1] = z;
    X[2] = X[1] * x;
    Y[2] = Y[1] * y;
    Z[2] = Z[1] * z;
    X[3] = X[2] * x;
    Y[3] = Y[2] * y;
    Z[3] = Z[2] * z;
    for (int si = N.shell_begin; si < N.shell_end; ++si) {
      const ShellEntry S = a.shells[si];
      Rad q;
      q.x = x;
      q.y = y;
      q.z = z;
      q.r2 = r2;
      q.l = S.l;
      double R = 0.0, R1 = 0.0, R2 = 0.0, R3 = 0.0;
      for (int pi = S.prim_begin; pi < S.prim_end; ++pi) {
        const bool act = !scr && (r2b < __ldg(&a.prims[pi].thr_bits));
        if (__any_sync(kFull, act)) {
          const double expo = __ldg(&a.prims[pi].expo);
          const double ar2 = expo * r2;
          const double e = exp_neg(ar2, thi, tlo);
          double v = __ldg(&a.prims[pi].coef) * e;
          v = act ? v : 0.0;
          R += v;  // the forward kernel's sum, in its order
          R1 = fma(-expo, v, R1);
          const double a2v = expo * expo * v;
          R2 += a2v;
          R3 = fma(-expo, a2v, R3);
        }
      }
      q.R = R;
      q.R1 = R1;
      q.R2 = R2;
      q.R3 = R3;
      double Rb = 0.0, R1b = 0.0, R2b = 0.0;
      switch (S.l) {
        case 0: vjp_shell_fixed<0>(rd, X, Y, Z, q, a.aof, S.ao_begin, scr, a.mask, Rb, R1b, R2b, de, wa, wc); break;
        case 1: vjp_shell_fixed<1>(rd, X, Y, Z, q, a.aof, S.ao_begin, scr, a.mask, Rb, R1b, R2b, de, wa, wc); break;
        case 2: vjp_shell_fixed<2>(rd, X, Y, Z, q, a.aof, S.ao_begin, scr, a.mask, Rb, R1b, R2b, de, wa, wc); break;
        case 3: vjp_shell_fixed<3>(rd, X, Y, Z, q, a.aof, S.ao_begin, scr, a.mask, Rb, R1b, R2b, de, wa, wc); break;
        default: vjp_shell_generic(rd, q, a.aof, S.ao_begin, scr, a.mask, Rb, R1b, R2b, de, wa, wc); break;
      }
      if (wa) {
        // exponent gradient of each primitive: radials recomputed, reduced over the warp's points
        for (int pi = S.prim_begin; pi < S.prim_end; ++pi) {
          const bool act = !scr && (r2b < __ldg(&a.prims[pi].thr_bits)) && lane < nvalid;
          double val = 0.0;
          if (__any_sync(kFull, act)) {
            const double expo = __ldg(&a.prims[pi].expo);
            const double ar2 = expo * r2;
            const double v = __ldg(&a.prims[pi].coef) * exp_neg(ar2, thi, tlo);
            const double t = -r2 * v * Rb + v * (ar2 - 1.0) * R1b + expo * v * (2.0 - ar2) * R2b;
            val = act ? t : 0.0;
          }
          val = warp_sum(val);
          if (lane == 0 && QG_STORE_OK(kSiteVjp, group * (int64_t)a.prim_num + pi, apart_extent)) apart[pi] = val;
        }
      }
    }
  }
  if (wc && lane < nvalid) {
    double* o = a.coord_part + ((int64_t)ch * P + p) * 3;
    if (!QG_STORE_OK(kSiteVjp, ((int64_t)ch * P + p) * 3 + 2, (int64_t)a.chunk_num * P * 3)) return;
    o[0] = de[0];
    o[1] = de[1];
    o[2] = de[2];
  }
}

// d_exponent[prim_orig[k]] (+)= sum over point groups (in order) of part[g][k].
__global__ void reduce_alpha_kernel(const double* __restrict__ part, int64_t groups, int K,
                                    const int32_t* __restrict__ prim_orig, int unique, double* __restrict__ out,
                                    int64_t out_num) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  double s = 0.0;
  for (int64_t g = 0; g < groups; ++g) s += part[g * K + k];
  if (!QG_STORE_OK(kSiteVjp, prim_orig[k], out_num)) return;
  if (unique) out[prim_orig[k]] = s;
  else atomicAdd(out + prim_orig[k], s);
}

// d_coord[p][j] = sum over nucleus chunks (in order) of part[ch][p][j].
__global__ void reduce_coord_kernel(const double* __restrict__ part, int chunks, int64_t n, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int c = 0; c < chunks; ++c) s += part[(int64_t)c * n + i];
  if (QG_STORE_OK(kSiteVjp, i, n)) out[i] = s;
}

// aoM = ao_vgl with the zero-value skip applied: rows 5p+1..5p+4 zero where row 5p is zero.
__global__ void mask_ao_kernel(const double* __restrict__ ao, int64_t P, int64_t A, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 5 * P * A) return;
  const int64_t k = i % A;
  const int64_t row = i / A;
  const int64_t p = row / 5;
  if (QG_STORE_OK(kSiteVjp, i, 5 * P * A)) out[i] = ao[p * 5 * A + k] == 0.0 ? 0.0 : ao[i];
}

int pick_vjp_level(const AoTables& t, int64_t groups) {
  const int64_t target = (int64_t)t.sm_count * 16;
  int best = 0;
  for (int lv = 0; lv < (int)t.level_offsets.size(); ++lv) {
    best = lv;
    if (groups * (int64_t)t.level_sizes[lv] >= target) break;
  }
  return best;
}

struct Scratch {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  }
};

// Grow-only scratch of the adjoint calls, owned by the context.
void* vjp_scratch(Ctx* ctx, size_t bytes) {
  void* p = ctx->vjp_buf;
  if (!ensure_raw(ctx, &p, &ctx->vjp_cap, bytes)) {
    ctx->vjp_buf = p;
    return nullptr;
  }
  ctx->vjp_buf = p;
  return p;
}

// Exponent and coordinate gradients from the AO adjoint gbar (device [P][5][A]). Outputs are
// device-accessible pointers (or null).
qmckl_exit_code_device ao_adjoint(Ctx* ctx, qmckl_context_device c, const char* fn, const double* gbar, int mask,
                                  double* d_expo_user, double* d_coord_pn, unsigned char* scratch, size_t off_alpha,
                                  size_t off_coord) {
  AoTables& t = ctx->ao_basis.tables;
  const int64_t P = ctx->point.num;
  const int64_t groups = (P + 31) / 32;
  const int lv = pick_vjp_level(t, groups);
  VjpArgs a;
  a.nuclei = t.nuclei;
  a.shells = t.shells;
  a.prims = t.prims;
  a.aof = t.ao_factor;
  a.chunk_num = t.level_sizes[lv];
  a.chunks = t.chunks + t.level_offsets[lv];
  a.exp_table = t.exp_table;
  a.coord = ctx->point.coord;
  a.perm = point_order(ctx);
  a.gbar = gbar;
  a.alpha_part = d_expo_user ? reinterpret_cast<double*>(scratch + off_alpha) : nullptr;
  a.coord_part = d_coord_pn ? reinterpret_cast<double*>(scratch + off_coord) : nullptr;
  a.point_num = P;
  a.ao_num = t.ao_num;
  a.task_num = groups * a.chunk_num;
  a.prim_num = t.prim_num;
  a.mask = mask;
  const size_t smem = 512 + sizeof(Stage<5>) * kVjpWarps;
  cudaFuncSetAttribute(vjp_ao_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    LaunchScope scope(ctx, "vjp_ao_adjoint");
    vjp_ao_kernel<<<(unsigned)((a.task_num + kVjpWarps - 1) / kVjpWarps), kVjpWarps * 32, smem, ctx->stream>>>(a);
  }
  if (d_expo_user) {
    cudaMemsetAsync(d_expo_user, 0, sizeof(double) * ctx->ao_basis.prim_num, ctx->stream);
    if (t.prim_num > 0) {
      LaunchScope scope(ctx, "vjp_reduce_exponent");
      reduce_alpha_kernel<<<(t.prim_num + 127) / 128, 128, 0, ctx->stream>>>(
          a.alpha_part, groups, t.prim_num, t.prim_orig, t.prims_unique ? 1 : 0, d_expo_user,
          ctx->ao_basis.prim_num);
    }
  }
  if (d_coord_pn) {
    LaunchScope scope(ctx, "vjp_reduce_coord");
    reduce_coord_kernel<<<(unsigned)((3 * P + 255) / 256), 256, 0, ctx->stream>>>(a.coord_part, a.chunk_num, 3 * P,
                                                                                  d_coord_pn);
  }
  if (cudaGetLastError() != cudaSuccess) return fail(c, QMCKL_FAILURE_DEVICE, fn, "adjoint kernel launch failed");
  return QMCKL_SUCCESS_DEVICE;
}

size_t alpha_part_bytes(const Ctx* ctx) {
  return sizeof(double) * (size_t)((ctx->point.num + 31) / 32) * (size_t)std::max<int64_t>(ctx->ao_basis.prim_num, 1);
}
size_t coord_part_bytes(const Ctx* ctx) {
  const AoTables& t = ctx->ao_basis.tables;
  int maxc = 1;
  for (int s : t.level_sizes) maxc = std::max(maxc, s);
  return sizeof(double) * 3 * (size_t)ctx->point.num * (size_t)maxc;
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" {

qmckl_exit_code_device qmckl_vjp_ao_vgl_device(qmckl_context_device context, const double* ao_vgl_bar,
                                               int64_t ao_vgl_bar_size, double* d_exponent, int64_t d_exponent_size,
                                               double* d_coord, int64_t d_coord_size) {
  QG_NVTX_RANGE("qmckl_vjp_ao_vgl_device");
  const char* fn = "qmckl_vjp_ao_vgl_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (!ctx->ao_basis.provided) return fail(context, QMCKL_NOT_PROVIDED_DEVICE, fn, "AO basis not provided");
  const int64_t P = ctx->point.num, A = ctx->ao_basis.ao_num, K = ctx->ao_basis.prim_num;
  if (!ao_vgl_bar) return fail(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (ao_vgl_bar_size < 5 * P * A) return fail(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "ao_vgl_bar too small");
  if (d_exponent && d_exponent_size < K) return fail(context, QMCKL_INVALID_ARG_5_DEVICE, fn, "d_exponent too small");
  if (d_coord && d_coord_size < 3 * P) return fail(context, QMCKL_INVALID_ARG_7_DEVICE, fn, "d_coord too small");
  if (!ensure_device(ctx)) return fail(context, QMCKL_FAILURE_DEVICE, fn, "no usable CUDA device");
  if (!d_exponent && !d_coord) return QMCKL_SUCCESS_DEVICE;
  if (P <= 0) {  // no points: the exponent gradient is zero, the coordinate gradient empty
    if (d_exponent && gpu_accessible(d_exponent)) cudaMemsetAsync(d_exponent, 0, sizeof(double) * K, ctx->stream);
    else if (d_exponent) memset(d_exponent, 0, sizeof(double) * K);
    return finish(ctx, context, fn);
  }
  qmckl_exit_code_device rc = ensure_tables(ctx, context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  Scratch s;
  const size_t o_in = gpu_accessible(ao_vgl_bar) ? 0 : s.take(sizeof(double) * 5 * P * A);
  const size_t o_alpha = s.take(d_exponent ? alpha_part_bytes(ctx) : 0);
  const size_t o_coord = s.take(d_coord ? coord_part_bytes(ctx) : 0);
  const bool e_dev = !d_exponent || gpu_accessible(d_exponent);
  const bool c_dev = !d_coord || gpu_accessible(d_coord);
  const size_t o_e = e_dev ? 0 : s.take(sizeof(double) * K);
  const size_t o_c = c_dev ? 0 : s.take(sizeof(double) * 3 * P);
  unsigned char* buf = static_cast<unsigned char*>(vjp_scratch(ctx, s.off + 256));
  if (!buf) return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "adjoint scratch");
  const double* gbar = ao_vgl_bar;
  if (!gpu_accessible(ao_vgl_bar)) {
    rc = copy(ctx, context, buf + o_in, ao_vgl_bar, sizeof(double) * 5 * P * A, fn);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    gbar = reinterpret_cast<const double*>(buf + o_in);
  }
  double* de = d_exponent ? (e_dev ? d_exponent : reinterpret_cast<double*>(buf + o_e)) : nullptr;
  double* dc = d_coord ? (c_dev ? d_coord : reinterpret_cast<double*>(buf + o_c)) : nullptr;
  rc = ao_adjoint(ctx, context, fn, gbar, 0, de, dc, buf, o_alpha, o_coord);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (d_exponent && !e_dev) rc = copy(ctx, context, d_exponent, de, sizeof(double) * K, fn, true);
  if (rc == QMCKL_SUCCESS_DEVICE && d_coord && !c_dev) rc = copy(ctx, context, d_coord, dc, sizeof(double) * 3 * P, fn, true);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  return finish(ctx, context, fn);
}

qmckl_exit_code_device qmckl_vjp_mo_vgl_device(qmckl_context_device context, const double* w, int64_t w_size,
                                               double* d_coefficient, int64_t d_coefficient_size, double* d_exponent,
                                               int64_t d_exponent_size, double* d_coord, int64_t d_coord_size) {
  QG_NVTX_RANGE("qmckl_vjp_mo_vgl_device");
  const char* fn = "qmckl_vjp_mo_vgl_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  Ctx* ctx = ctx_of(context);
  if (!ctx->ao_basis.provided) return fail(context, QMCKL_NOT_PROVIDED_DEVICE, fn, "AO basis not provided");
  if (!ctx->mo_basis.provided) return fail(context, QMCKL_NOT_PROVIDED_DEVICE, fn, "MO basis not provided");
  const int64_t P = ctx->point.num, A = ctx->ao_basis.ao_num, K = ctx->ao_basis.prim_num, M = ctx->mo_basis.mo_num;
  if (!w) return fail(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (w_size < 5 * P * M) return fail(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "w too small");
  if (d_coefficient && d_coefficient_size < M * A)
    return fail(context, QMCKL_INVALID_ARG_5_DEVICE, fn, "d_coefficient too small");
  if (d_exponent && d_exponent_size < K) return fail(context, QMCKL_INVALID_ARG_7_DEVICE, fn, "d_exponent too small");
  if (d_coord && d_coord_size < 3 * P) return fail(context, QMCKL_INVALID_ARG_9_DEVICE, fn, "d_coord too small");
  if (!ensure_device(ctx)) return fail(context, QMCKL_FAILURE_DEVICE, fn, "no usable CUDA device");
  if (!d_coefficient && !d_exponent && !d_coord) return QMCKL_SUCCESS_DEVICE;
  qmckl_exit_code_device rc = ensure_tables(ctx, context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (d_coefficient) {
    rc = qmckl_provide_ao_basis_ao_vgl_device(context);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  }
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t nparts = dgemm_splitk_parts(M, 5 * P, A, sms);

  Scratch s;
  const bool w_dev = gpu_accessible(w);
  const size_t o_w = w_dev ? 0 : s.take(sizeof(double) * 5 * P * M);
  const bool need_ao = d_exponent || d_coord;
  const size_t o_g = s.take(need_ao ? sizeof(double) * 5 * P * A : 0);
  const size_t o_alpha = s.take(d_exponent ? alpha_part_bytes(ctx) : 0);
  const size_t o_coord = s.take(d_coord ? coord_part_bytes(ctx) : 0);
  const size_t o_wt = s.take(d_coefficient ? sizeof(double) * 5 * P * M : 0);
  const size_t o_aom = s.take(d_coefficient ? sizeof(double) * 5 * P * A : 0);
  const size_t o_parts = s.take(d_coefficient ? sizeof(double) * (size_t)nparts * M * A : 0);
  const bool cf_dev = !d_coefficient || gpu_accessible(d_coefficient);
  const bool e_dev = !d_exponent || gpu_accessible(d_exponent);
  const bool c_dev = !d_coord || gpu_accessible(d_coord);
  const size_t o_cf = cf_dev ? 0 : s.take(sizeof(double) * M * A);
  const size_t o_e = e_dev ? 0 : s.take(sizeof(double) * K);
  const size_t o_c = c_dev ? 0 : s.take(sizeof(double) * 3 * P);
  unsigned char* buf = static_cast<unsigned char*>(vjp_scratch(ctx, s.off + 256));
  if (!buf) return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "adjoint scratch");
  const double* wd = w;
  if (!w_dev) {
    rc = copy(ctx, context, buf + o_w, w, sizeof(double) * 5 * P * M, fn);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    wd = reinterpret_cast<const double*>(buf + o_w);
  }
  if (P > 0 && d_coefficient) {
    double* wt = reinterpret_cast<double*>(buf + o_wt);
    double* aom = reinterpret_cast<double*>(buf + o_aom);
    double* out = cf_dev ? d_coefficient : reinterpret_cast<double*>(buf + o_cf);
    launch_transpose(ctx, wd, 5 * P, M, wt);
    {
      LaunchScope scope(ctx, "vjp_mask_ao");
      mask_ao_kernel<<<(unsigned)((5 * P * A + 255) / 256), 256, 0, ctx->stream>>>(ctx->ao_basis.ao_vgl, P, A, aom);
    }
    launch_dgemm_splitk(ctx, wt, aom, reinterpret_cast<double*>(buf + o_parts), nparts, out, M, 5 * P, A,
                        "vjp_coefficient_dgemm");
    if (!cf_dev) {
      rc = copy(ctx, context, d_coefficient, out, sizeof(double) * M * A, fn, true);
      if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    }
  } else if (d_coefficient) {
    if (cf_dev) cudaMemsetAsync(d_coefficient, 0, sizeof(double) * M * A, ctx->stream);
    else memset(d_coefficient, 0, sizeof(double) * M * A);
  }
  if (P > 0 && need_ao) {
    double* gbar = reinterpret_cast<double*>(buf + o_g);
    launch_dgemm_rm(ctx, wd, ctx->mo_basis.coefficient, gbar, 5 * P, M, A, "vjp_ao_adjoint_dgemm");
    double* de = d_exponent ? (e_dev ? d_exponent : reinterpret_cast<double*>(buf + o_e)) : nullptr;
    double* dc = d_coord ? (c_dev ? d_coord : reinterpret_cast<double*>(buf + o_c)) : nullptr;
    rc = ao_adjoint(ctx, context, fn, gbar, 1, de, dc, buf, o_alpha, o_coord);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    if (d_exponent && !e_dev) rc = copy(ctx, context, d_exponent, de, sizeof(double) * K, fn, true);
    if (rc == QMCKL_SUCCESS_DEVICE && d_coord && !c_dev)
      rc = copy(ctx, context, d_coord, dc, sizeof(double) * 3 * P, fn, true);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  } else if (d_exponent) {
    if (e_dev) cudaMemsetAsync(d_exponent, 0, sizeof(double) * K, ctx->stream);
    else memset(d_exponent, 0, sizeof(double) * K);
  }
  return finish(ctx, context, fn);
}

}  // extern "C"
