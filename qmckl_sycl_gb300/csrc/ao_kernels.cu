// Fused AO kernels for sm_103a: electron-nucleus displacement, exponent-cutoff screening,
// Gaussian shell radials, Cartesian polynomial and AO assembly in one pass, writing
// ao_vgl[point][5][ao] (or ao_value[point][ao]) without any intermediate global array.
//
// Reference computation (qmckl_sycl): shell radials src/qmckl_ao_sycl.cpp:40-95, the
// polynomial kernel :195-334 and the assembly kernel :337-422 (value-only :438-740),
// which round-trip shell_vgl, pows and poly_vgl through global memory.
//
// Design for GB300. FP64 issues at ~1/66 of the FP32 rate on this part (measured
// 1.05 TFLOP/s DFMA and DMMA against 69 TFLOP/s FFMA), so this kernel is bound by its
// FP64 instruction count, not by HBM. Hence:
//  * one lane per point: every lane of a warp walks the same nucleus/shell/primitive/AO
//    sequence, so table loads are warp-uniform broadcasts and every FP64 instruction
//    runs with all 32 lanes busy;
//  * screening costs no FP64 instruction: the reference's tests `r2 > cutoff*range`
//    and `expo*r2 > cutoff` are replaced by unsigned compares of bit patterns against
//    thresholds precomputed on the host (for non-negative doubles the bit order is the
//    numeric order, and fl(expo*r2) is monotone in r2), which gives the reference's
//    decisions exactly; an exponential is only evaluated when some lane needs it;
//  * r2 is formed with the reference's rounding ((x*x + y*y) + z*z, no fused
//    multiply-add), so the screening inputs are the reference's bits;
//  * the radial derivatives are accumulated as g = sum(-2 a v) and h = sum(-2 a v a r2)
//    (two accumulators instead of four) and the Laplacian assembly uses Euler's identity
//    x.dP/dx + y.dP/dy + z.dP/dz = l P for the degree-l monomial P, so that
//    2 grad(P).grad(R) = 2 l g P; both are exact identities, differing from the
//    reference's evaluation order only by rounding;
//  * Cartesian components are specialised at compile time for l <= 3 (products with
//    0 and 1 fold away); higher l takes a generic path;
//  * results are staged per warp in shared memory and stored as contiguous row
//    segments of ao_vgl, so global stores are coalesced whatever the point order.
#include <cstdint>

#include "internal.hpp"

namespace qg {
namespace {

constexpr int kWarps = 4;          // warps per CTA (each runs its own task)
constexpr int kStage = 8;          // AOs staged per warp between flushes
constexpr int kPad = 33;           // 32 points + 1 (bank-conflict padding), in doubles
constexpr unsigned kFull = 0xffffffffu;

template <int NC>
struct Stage {
  double v[NC][kStage][kPad];
};

__device__ __forceinline__ uint64_t bits_of(double x) { return static_cast<uint64_t>(__double_as_longlong(x)); }
__device__ __forceinline__ bool is_one(double f) { return bits_of(f) == 0x3FF0000000000000ull; }

// Collects one warp's AO values (lane = point) and writes them as row segments.
template <int NC>
struct Writer {
  Stage<NC>* st;
  double* out;       // ao_vgl or ao_value
  int64_t p0;        // first point of the warp
  int64_t ao_num;
  int nvalid;        // points of the warp that exist
  int lane;
  int base;          // AO index of stage slot 0
  int fill;          // staged AOs

  __device__ __forceinline__ void flush() {
    __syncwarp();
    const int total = nvalid * NC * kStage;
    for (int i = lane; i < total; i += 32) {
      const int j = i & (kStage - 1);
      const int rest = i / kStage;
      const int c = rest % NC;
      const int q = rest / NC;
      if (j < fill) out[(p0 + q) * (NC * ao_num) + c * ao_num + base + j] = st->v[c][j][q];
    }
    __syncwarp();
    base += fill;
    fill = 0;
  }
  __device__ __forceinline__ void emit(const double (&v)[NC]) {
    if (fill == kStage) flush();
#pragma unroll
    for (int c = 0; c < NC; ++c) st->v[c][fill][lane] = v[c];
    fill += 1;
  }
  __device__ __forceinline__ void emit_zeros(int count) {
    double z[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) z[c] = 0.0;
    for (int i = 0; i < count; ++i) emit(z);
  }
};

// Shell quantities shared by the shell's Cartesian components.
struct ShellVals {
  double R;    // radial value t0
  double t1, t2, t3;  // radial gradient = g * (x, y, z)
  double Rt;   // t4 + 2 l g, the radial part of the Laplacian after Euler's identity
};

// One Cartesian component x^a y^b z^c (a, b, c compile-time), assembled like the
// reference's src/qmckl_ao_sycl.cpp:371-420 and multiplied by the AO factor.
template <int NC, int a, int b, int c>
__device__ __forceinline__ void cart(Writer<NC>& w, const double (&X)[4], const double (&Y)[4], const double (&Z)[4],
                                     const ShellVals& s, double f, bool zero) {
  const double yz = Y[b] * Z[c];
  const double P = X[a] * yz;
  double v[NC];
  if constexpr (NC == 1) {
    v[0] = P * s.R;
  } else {
    const double xz = X[a] * Z[c];
    const double xy = X[a] * Y[b];
    double gx = P * s.t1, gy = P * s.t2, gz = P * s.t3;
    if constexpr (a > 0) gx = fma((double)a * X[a - 1], yz * s.R, gx);
    if constexpr (b > 0) gy = fma((double)b * Y[b - 1], xz * s.R, gy);
    if constexpr (c > 0) gz = fma((double)c * Z[c - 1], xy * s.R, gz);
    double lap = P * s.Rt;
    if constexpr (a > 1) lap = fma((double)(a * (a - 1)) * X[a - 2], yz * s.R, lap);
    if constexpr (b > 1) lap = fma((double)(b * (b - 1)) * Y[b - 2], xz * s.R, lap);
    if constexpr (c > 1) lap = fma((double)(c * (c - 1)) * Z[c - 2], xy * s.R, lap);
    v[0] = P * s.R;
    v[1] = gx;
    v[2] = gy;
    v[3] = gz;
    v[4] = lap;
  }
  if (!is_one(f)) {
#pragma unroll
    for (int k = 0; k < NC; ++k) v[k] *= f;
  }
  if (zero) {
#pragma unroll
    for (int k = 0; k < NC; ++k) v[k] = 0.0;
  }
  w.emit(v);
}

// Components of one shell in the reference's order: a descending, then b descending
// (src/qmckl_ao_sycl.cpp:297-305).
template <int NC, int L>
__device__ __forceinline__ void shell_fixed(Writer<NC>& w, const double (&X)[4], const double (&Y)[4],
                                            const double (&Z)[4], const ShellVals& s, const double* __restrict__ aof,
                                            int ao0, bool zero) {
  if constexpr (L == 0) {
    cart<NC, 0, 0, 0>(w, X, Y, Z, s, __ldg(aof + ao0), zero);
  } else if constexpr (L == 1) {
    cart<NC, 1, 0, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 0), zero);
    cart<NC, 0, 1, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 1), zero);
    cart<NC, 0, 0, 1>(w, X, Y, Z, s, __ldg(aof + ao0 + 2), zero);
  } else if constexpr (L == 2) {
    cart<NC, 2, 0, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 0), zero);
    cart<NC, 1, 1, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 1), zero);
    cart<NC, 1, 0, 1>(w, X, Y, Z, s, __ldg(aof + ao0 + 2), zero);
    cart<NC, 0, 2, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 3), zero);
    cart<NC, 0, 1, 1>(w, X, Y, Z, s, __ldg(aof + ao0 + 4), zero);
    cart<NC, 0, 0, 2>(w, X, Y, Z, s, __ldg(aof + ao0 + 5), zero);
  } else {
    cart<NC, 3, 0, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 0), zero);
    cart<NC, 2, 1, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 1), zero);
    cart<NC, 2, 0, 1>(w, X, Y, Z, s, __ldg(aof + ao0 + 2), zero);
    cart<NC, 1, 2, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 3), zero);
    cart<NC, 1, 1, 1>(w, X, Y, Z, s, __ldg(aof + ao0 + 4), zero);
    cart<NC, 1, 0, 2>(w, X, Y, Z, s, __ldg(aof + ao0 + 5), zero);
    cart<NC, 0, 3, 0>(w, X, Y, Z, s, __ldg(aof + ao0 + 6), zero);
    cart<NC, 0, 2, 1>(w, X, Y, Z, s, __ldg(aof + ao0 + 7), zero);
    cart<NC, 0, 1, 2>(w, X, Y, Z, s, __ldg(aof + ao0 + 8), zero);
    cart<NC, 0, 0, 3>(w, X, Y, Z, s, __ldg(aof + ao0 + 9), zero);
  }
}

// Generic path for l >= 4 (rare): powers in local memory, same formulas.
template <int NC>
__device__ __noinline__ void shell_generic(Writer<NC>& w, double x, double y, double z, int L, const ShellVals& s,
                                           const double* __restrict__ aof, int ao0, bool zero) {
  double X[kMaxL + 1], Y[kMaxL + 1], Z[kMaxL + 1];
  X[0] = Y[0] = Z[0] = 1.0;
  for (int i = 1; i <= L; ++i) {
    X[i] = X[i - 1] * x;
    Y[i] = Y[i - 1] * y;
    Z[i] = Z[i - 1] * z;
  }
  int k = 0;
  for (int a = L; a >= 0; --a)
    for (int b = L - a; b >= 0; --b) {
      const int c = L - a - b;
      const double yz = Y[b] * Z[c], xz = X[a] * Z[c], xy = X[a] * Y[b];
      const double P = X[a] * yz;
      double v[NC];
      v[0] = P * s.R;
      if constexpr (NC == 5) {
        double gx = P * s.t1, gy = P * s.t2, gz = P * s.t3, lap = P * s.Rt;
        if (a > 0) gx = fma((double)a * X[a - 1], yz * s.R, gx);
        if (b > 0) gy = fma((double)b * Y[b - 1], xz * s.R, gy);
        if (c > 0) gz = fma((double)c * Z[c - 1], xy * s.R, gz);
        if (a > 1) lap = fma((double)(a * (a - 1)) * X[a - 2], yz * s.R, lap);
        if (b > 1) lap = fma((double)(b * (b - 1)) * Y[b - 2], xz * s.R, lap);
        if (c > 1) lap = fma((double)(c * (c - 1)) * Z[c - 2], xy * s.R, lap);
        v[1] = gx;
        v[2] = gy;
        v[3] = gz;
        v[4] = lap;
      }
      const double f = __ldg(aof + ao0 + k);
      if (!is_one(f))
        for (int q = 0; q < NC; ++q) v[q] *= f;
      if (zero)
        for (int q = 0; q < NC; ++q) v[q] = 0.0;
      w.emit(v);
      ++k;
    }
}

// One warp task: 32 points (lane = point) x one chunk of consecutive nuclei.
template <int NC>
__global__ void __launch_bounds__(kWarps * 32) ao_fused_kernel(const NucleusEntry* __restrict__ nuclei,
                                                               const ShellEntry* __restrict__ shells,
                                                               const PrimEntry* __restrict__ prims,
                                                               const double* __restrict__ aof,
                                                               const NucleusChunk* __restrict__ chunks, int chunk_num,
                                                               const double* __restrict__ coord, int64_t point_num,
                                                               int64_t ao_num, int64_t task_num,
                                                               double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t task = (int64_t)blockIdx.x * kWarps + warp;
  if (task >= task_num) return;  // warp-uniform
  const int64_t group = task / chunk_num;
  const int ch = (int)(task - group * chunk_num);
  const int64_t p0 = group * 32;
  const int64_t remaining = point_num - p0;
  const int nvalid = remaining < 32 ? (int)remaining : 32;
  const int64_t p = p0 + (lane < nvalid ? lane : nvalid - 1);
  const double ex = coord[p], ey = coord[point_num + p], ez = coord[2 * point_num + p];

  Writer<NC> w;
  w.st = reinterpret_cast<Stage<NC>*>(smem_raw) + warp;
  w.out = out;
  w.p0 = p0;
  w.ao_num = ao_num;
  w.nvalid = nvalid;
  w.lane = lane;
  const NucleusChunk cj = chunks[ch];
  w.base = cj.ao_begin;
  w.fill = 0;

  for (int n = cj.nucl_begin; n < cj.nucl_end; ++n) {
    const NucleusEntry& N = nuclei[n];
    const double x = ex - N.x, y = ey - N.y, z = ez - N.z;
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    const uint64_t r2b = bits_of(r2);
    const bool scr = r2b > N.screen_bits;
    if (__all_sync(kFull, scr)) {
      w.emit_zeros(N.ao_end - N.ao_begin);
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
      const ShellEntry S = shells[si];
      double t0 = 0.0, g = 0.0, h = 0.0;
      for (int pi = S.prim_begin; pi < S.prim_end; ++pi) {
        const bool act = !scr && (r2b < __ldg(&prims[pi].thr_bits));
        if (__any_sync(kFull, act)) {
          const double expo = __ldg(&prims[pi].expo);
          const double ar2 = expo * r2;
          const double e = exp(-ar2);
          double v = __ldg(&prims[pi].coef) * e;
          v = act ? v : 0.0;
          t0 += v;
          if constexpr (NC == 5) {
            const double two_a = __ldg(&prims[pi].m2a) * v;
            g += two_a;
            h = fma(two_a, ar2, h);
          }
        }
      }
      ShellVals sv;
      sv.R = t0;
      if constexpr (NC == 5) {
        sv.t1 = g * x;
        sv.t2 = g * y;
        sv.t3 = g * z;
        const double t4 = fma(-2.0, h, 3.0 * g);
        sv.Rt = fma((double)(2 * S.l), g, t4);
      } else {
        sv.t1 = sv.t2 = sv.t3 = sv.Rt = 0.0;
      }
      switch (S.l) {
        case 0: shell_fixed<NC, 0>(w, X, Y, Z, sv, aof, S.ao_begin, scr); break;
        case 1: shell_fixed<NC, 1>(w, X, Y, Z, sv, aof, S.ao_begin, scr); break;
        case 2: shell_fixed<NC, 2>(w, X, Y, Z, sv, aof, S.ao_begin, scr); break;
        case 3: shell_fixed<NC, 3>(w, X, Y, Z, sv, aof, S.ao_begin, scr); break;
        default: shell_generic<NC>(w, x, y, z, S.l, sv, aof, S.ao_begin, scr); break;
      }
    }
  }
  w.flush();
}

// Shell radials on their own (qmckl_get_ao_basis_shell_vgl_device), one thread per
// (point, packed shell), the reference's formulas of src/qmckl_ao_sycl.cpp:47-95.
__global__ void shell_vgl_kernel(const NucleusEntry* __restrict__ nuclei, const ShellEntry* __restrict__ shells,
                                 const PrimEntry* __restrict__ prims, const int32_t* __restrict__ shell_orig,
                                 const int32_t* __restrict__ shell_nucl, const double* __restrict__ coord,
                                 int64_t point_num, int packed_shells, int64_t shell_num, double* __restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= point_num * packed_shells) return;
  const int64_t ip = idx / packed_shells;
  const int si = (int)(idx - ip * packed_shells);
  const NucleusEntry& N = nuclei[shell_nucl[si]];
  const double x = coord[ip] - N.x, y = coord[point_num + ip] - N.y, z = coord[2 * point_num + ip] - N.z;
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
  const int64_t os = shell_orig[si];
  double* o = out + ip * 5 * shell_num + os;
  if (bits_of(r2) > N.screen_bits) {
    o[0] = o[shell_num] = o[2 * shell_num] = o[3 * shell_num] = o[4 * shell_num] = 0.0;
    return;
  }
  const ShellEntry S = shells[si];
  double t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0;
  for (int pi = S.prim_begin; pi < S.prim_end; ++pi) {
    const PrimEntry Pr = prims[pi];
    if (bits_of(r2) >= Pr.thr_bits) continue;
    const double ar2 = __dmul_rn(Pr.expo, r2);
    const double v = __dmul_rn(Pr.coef, exp(-ar2));
    const double two_a = __dmul_rn(Pr.m2a, v);
    t0 = __dadd_rn(t0, v);
    t1 = __dadd_rn(t1, __dmul_rn(two_a, x));
    t2 = __dadd_rn(t2, __dmul_rn(two_a, y));
    t3 = __dadd_rn(t3, __dmul_rn(two_a, z));
    t4 = __dadd_rn(t4, __dmul_rn(two_a, __dsub_rn(3.0, __dmul_rn(2.0, ar2))));
  }
  o[0] = t0;
  o[shell_num] = t1;
  o[2 * shell_num] = t2;
  o[3 * shell_num] = t3;
  o[4 * shell_num] = t4;
}

// Picks the nucleus-chunk level whose task count best fills the GPU.
int pick_level(const AoTables& t, int64_t groups, int sms) {
  const int64_t target = (int64_t)sms * 16;  // ~16 warp tasks per SM
  int best = 0;
  for (int lv = 0; lv < (int)t.level_offsets.size(); ++lv) {
    best = lv;
    if (groups * (int64_t)t.level_sizes[lv] >= target) break;
  }
  return best;
}

template <int NC>
cudaError_t launch_fused(Ctx* ctx, const AoTables& t, const double* coord, int64_t point_num, double* out,
                         const char* name) {
  if (point_num <= 0 || t.ao_num <= 0) return cudaSuccess;
  const int64_t groups = (point_num + 31) / 32;
  const int lv = pick_level(t, groups, t.sm_count);
  const int chunk_num = t.level_sizes[lv];
  const NucleusChunk* chunks = t.chunks + t.level_offsets[lv];
  const int64_t tasks = groups * chunk_num;
  const int64_t blocks = (tasks + kWarps - 1) / kWarps;
  const size_t smem = sizeof(Stage<NC>) * kWarps;
  cudaFuncSetAttribute(ao_fused_kernel<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  LaunchScope scope(ctx, name);
  ao_fused_kernel<NC><<<(unsigned)blocks, kWarps * 32, smem, ctx->stream>>>(
      t.nuclei, t.shells, t.prims, t.ao_factor, chunks, chunk_num, coord, point_num, t.ao_num, tasks, out);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_ao_vgl(Ctx* ctx, const AoTables& t, const double* coord, int64_t point_num, double* ao_vgl) {
  return launch_fused<5>(ctx, t, coord, point_num, ao_vgl, "ao_vgl_fused");
}

cudaError_t launch_ao_value(Ctx* ctx, const AoTables& t, const double* coord, int64_t point_num, double* ao_value) {
  return launch_fused<1>(ctx, t, coord, point_num, ao_value, "ao_value_fused");
}

cudaError_t launch_shell_vgl(Ctx* ctx, const AoTables& t, const double* coord, int64_t point_num, int64_t shell_num,
                             double* shell_vgl) {
  if (point_num <= 0 || shell_num <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(shell_vgl, 0, sizeof(double) * 5 * shell_num * point_num, ctx->stream);
  if (e != cudaSuccess || t.shell_num == 0) return e;
  const int64_t n = point_num * t.shell_num;
  LaunchScope scope(ctx, "shell_vgl");
  shell_vgl_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(
      t.nuclei, t.shells, t.prims, t.shell_orig, t.shell_nucl, coord, point_num, t.shell_num, shell_num, shell_vgl);
  return cudaGetLastError();
}

}  // namespace qg
