// Fused AO kernels for sm_103a: electron-nucleus displacement, exponent-cutoff screening,
// Gaussian shell radials, Cartesian polynomial and AO assembly in one pass, writing
// ao_vgl[point][5][ao] (or ao_value[point][ao], or the BF16 planes of the split-BF16 MO
// contraction) without any intermediate global array.
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
//  * points are processed in an order that puts spatial neighbours in the same warp
//    (launch_point_order), because a primitive's exponential is evaluated when any lane
//    of the warp needs it: on the medium workload this cuts the exponentials per point
//    from 65 % to 36 % of the primitives (30 % is the per-lane share);
//  * screening costs no FP64 instruction: the reference's tests `r2 > cutoff*range`
//    and `expo*r2 > cutoff` are replaced by unsigned compares of bit patterns against
//    thresholds precomputed on the host (for non-negative doubles the bit order is the
//    numeric order, and fl(expo*r2) is monotone in r2), which gives the reference's
//    decisions exactly;
//  * r2 is formed with the reference's rounding ((x*x + y*y) + z*z, no fused
//    multiply-add), so the screening inputs are the reference's bits;
//  * the exponential is evaluated with Tang's table-driven method on the screened range
//    x in [-27.64, 0] (12 FP64 instructions: reduction by ln2/32, a degree-6 polynomial, a
//    32-entry table of 2^(j/32) in shared memory, exponent scaling by integer addition);
//  * the radial derivatives are accumulated as g = sum(-2 a v) and h = sum(-2 a v a r2)
//    (two accumulators instead of four) and the Laplacian assembly uses Euler's identity
//    x.dP/dx + y.dP/dy + z.dP/dz = l P for the degree-l monomial P, so that
//    2 grad(P).grad(R) = 2 l g P; both are exact identities, differing from the
//    reference's evaluation order only by rounding;
//  * Cartesian components are specialised at compile time for l <= 3 (products with
//    0 and 1 fold away); higher l takes a generic path;
//  * results are staged per warp in shared memory and stored as contiguous row
//    segments, so global stores are coalesced whatever the point order.
// The split-BF16 form's planes carry 24 significant bits, so its kernel keeps the FP64 pipe for
// r2 alone (the screening inputs): primitives, radial sums and the radial Laplacian factor run in
// FP32 pair arithmetic (~44 bits), the per-AO assembly in FP32.
#include <cuda_bf16.h>

#include <cstddef>
#include <cstdint>

#include "internal.hpp"
#include "ao_device.cuh"

namespace qg {
namespace {

constexpr int kWarps = 4;          // warps per CTA (each runs its own task)
#ifndef QMCKL_AO_TASKS_PER_WARP
#define QMCKL_AO_TASKS_PER_WARP 2
#endif
#ifndef QMCKL_AO_PLANES_TASKS_PER_WARP
#define QMCKL_AO_PLANES_TASKS_PER_WARP 1
#endif
// Tasks per resident warp the nucleus-chunk level is chosen for (finer chunks give more tasks):
// 2 for the FP64 outputs; 1 for the split-BF16 planes, whose FP32 radials make a task about half
// as long (planes on the medium workload 0.446 ms against 0.455 ms with 2 and 0.497 ms with 4).
constexpr int kTasksPerWarp = QMCKL_AO_TASKS_PER_WARP;
constexpr int kPlanesTasksPerWarp = QMCKL_AO_PLANES_TASKS_PER_WARP;
#ifndef QMCKL_AO_TAIL_SEGMENTS
#define QMCKL_AO_TAIL_SEGMENTS 8
#endif
// Segments of a launch's schedule (1: every task at the chosen level; more: the last point
// groups at finer levels, down to pieces of nuclei).
constexpr int kTailSegments = QMCKL_AO_TAIL_SEGMENTS;
#ifndef QMCKL_AO_BATCH_PLANES_SKIP_DEAD
#define QMCKL_AO_BATCH_PLANES_SKIP_DEAD 0
#endif
// Whether the batch kernel's planes skip the assembly of shells that are zero on every lane.
constexpr bool kBatchPlanesSkipDead = QMCKL_AO_BATCH_PLANES_SKIP_DEAD != 0;
using namespace dev;

enum class Out { Vgl, Value, Planes };
template <Out O>
__host__ __device__ constexpr int ncomp() {
  return O == Out::Value ? 1 : 5;
}
// Resident CTAs per SM the register allocation must allow. The planes output stages nothing in
// shared memory, so registers alone bound its occupancy: 7 CTAs (28 warps, 72 registers) per SM
// measured 0.559 ms against 0.586 / 0.575 ms with 6 / 8 on the medium workload (the FP32 pair
// radials; with the earlier FP64 radials 6 CTAs measured 2.13 ms against 2.76 ms with the
// compiler's unconstrained 4). The staged ao_vgl output fits 5 CTAs in shared memory, ao_value 8
// or more.
#ifndef QMCKL_AO_PLANES_CTAS
#define QMCKL_AO_PLANES_CTAS 7
#endif
template <Out O>
__host__ __device__ constexpr int min_ctas() {
  return O == Out::Planes ? QMCKL_AO_PLANES_CTAS : (O == Out::Vgl ? 5 : 8);
}

// Dynamic shared memory: the exponential's tables (2 x 32 doubles, plus the split-BF16 form's
// 2048-entry table of FP32 pairs), then the per-warp staging buffers.
template <Out O>
__host__ __device__ constexpr size_t stage_offset() {
  return O == Out::Planes ? 512 + 8 * kFine : 512;
}

// ---------------------------------------------------------------- output staging
// Splits an FP64 value into three BF16 terms (hi + mid + lo carries 24 significant bits) with
// integer and FP32 instructions only: FP64 -> FP32 by round-to-nearest-even on the bit pattern
// (values below the FP32 normal range become zero, which is below the form's error budget).
__device__ __forceinline__ float f64_to_f32(double a) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FF) - 896;
  if (e <= 0) return __uint_as_float(sign);
  const unsigned long long frac = b & 0xFFFFFFFFFFFFFull;
  const unsigned int mm = (unsigned int)(frac >> 29);
  const unsigned long long rem = frac & 0x1FFFFFFFull;
  unsigned int bits = ((unsigned int)(e < 255 ? e : 255) << 23) | (e < 255 ? mm : 0u);
  if (e < 255 && (rem > 0x10000000ull || (rem == 0x10000000ull && (mm & 1u)))) bits += 1u;
  return __uint_as_float(sign | bits);
}

// An FP32 value as three BF16 terms (exact: 24 significant bits).
__device__ __forceinline__ void split_bf16x3f(float f, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
  h = __float2bfloat16_rn(f);
  const float r1 = f - __bfloat162float(h);
  m = __float2bfloat16_rn(r1);
  l = __float2bfloat16_rn(r1 - __bfloat162float(m));
}

__device__ __forceinline__ void split_bf16x3(double a, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
  split_bf16x3f(f64_to_f32(a), h, m, l);
}

// c ? v : +0.0 on the bit pattern (an integer AND instead of a select of doubles).
__device__ __forceinline__ double keep_if(bool c, double v) {
  return __longlong_as_double(__double_as_longlong(v) & -(long long)c);
}

// 2l of the radial Laplacian term as doubles, by l (no integer-to-FP64 conversion per shell).
__constant__ double kTwoL[kMaxL + 1] = {0, 2, 4, 6, 8, 10, 12, 14, 16, 18, 20, 22, 24, 26, 28, 30, 32, 34, 36, 38};

// ---------------------------------------------------------------- FP32 pair arithmetic
// The split-BF16 form's radials run on the FP32 pipe (64 times the FP64 rate on this part) as
// pairs hi + lo of floats carrying about 44 significant bits: products of the high parts made
// exact with fmaf (the low part of a*b is fmaf(a, b, -a*b)), sums made exact with Knuth's
// two-sum. The _rn intrinsics are never contracted into fused multiply-adds, which would break
// these identities.
struct F2 {
  float h, l;
};

// (xh + xl) * (yh + yl) to ~2^-47 relative: xh*yh exactly, the cross terms rounded, xl*yl dropped.
__device__ __forceinline__ F2 mul_pair(float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float e = fmaf(xh, yh, -p);
  return {p, fmaf(xh, yl, fmaf(xl, yh, e))};
}

// s += b: the high parts' sum exactly (two-sum), its error and the low parts into s.l.
__device__ __forceinline__ void add_pair(F2& s, F2 b) {
  const float t = __fadd_rn(s.h, b.h);
  const float bb = __fsub_rn(t, s.h);
  const float err = __fadd_rn(__fsub_rn(s.h, __fsub_rn(t, bb)), __fsub_rn(b.h, bb));
  s.l = __fadd_rn(s.l, __fadd_rn(err, b.l));
  s.h = t;
}

// An FP32 value as a double, with integer instructions (normal values and zeros; values below
// the float normal range become zero, infinities and NaN stay).
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long mant = (unsigned long long)(u & 0x7FFFFFu) << 29;
  const unsigned long long ex = e == 0 ? 0ull : (e == 255 ? 0x7FFull : (unsigned long long)(e + 896)) << 52;
  return __longlong_as_double((long long)(sign | ex | (e == 0 ? 0ull : mant)));
}

constexpr float kInvLFinef = (float)(kFine / 0.6931471805599453094);  // kFine / ln 2 (picks the index)
constexpr double kLFine = 0.6931471805599453094 / kFine;              // ln 2 / kFine (the double)
constexpr float kLh = (float)kLFine;                                   // as an FP32 pair
constexpr float kLm = (float)(kLFine - (double)kLh);

// A PrimFold loaded as two 16-byte vectors instead of one load per field.
struct FoldRec {
  uint64_t thr;
  float nah, nal, dh;
  uint32_t jeb;
  float ch, cl;
};
static_assert(offsetof(PrimFold, nah) == 8 && offsetof(PrimFold, dh) == 16 && offsetof(PrimFold, jeb) == 20 &&
                  offsetof(PrimFold, c) == 24,
              "FoldRec reads PrimFold's fields in this order");
__device__ __forceinline__ FoldRec load_fold(const PrimFold* __restrict__ F) {
  const uint4 q0 = __ldg(reinterpret_cast<const uint4*>(F));
  const uint4 q1 = __ldg(reinterpret_cast<const uint4*>(F) + 1);
  FoldRec r;
  r.thr = (uint64_t)q0.x | ((uint64_t)q0.y << 32);
  r.nah = __uint_as_float(q0.z);
  r.nal = __uint_as_float(q0.w);
  r.dh = __uint_as_float(q1.x);
  r.jeb = q1.y;
  r.ch = __uint_as_float(q1.z);
  r.cl = __uint_as_float(q1.w);
  return r;
}

// One primitive of the split-BF16 form, v = coef * e^(-expo r2), as an FP32 pair, for
// r2 = r2h + r2l (an FP32 pair). With L = ln 2 / 1024, y = -expo r2 + ln(mant) and n = n1 + jm:
//   e^y = 2^(n >> 10) * 2^((n & 1023)/1024) * e^r,  r = (p - n1 L) + (dh + low parts),
// where p = fl(-expo r2h) and n1 = round(p / L). t1 = p - n1 Lh is exact (|t1| < 2^-11 and both
// terms are multiples of 2^-34, or of 2^-35 when |p| < 2^-11), e^r - 1 - t1 = rl + r^2 (1/2 + r/6)
// (truncation below 1e-14 for |r| <= 7e-4), the table gives 2^(j/1024) as a pair, and
// sign * 2^k * 2^(n >> 10) is one float multiply (exact). Relative error within 1e-10 of the
// exact value over the active range y in [-27.7, ln 2) (long-double comparison on the test
// bases; the rounding of rl, |rl| <= L / 2, dominates); only FP32 and integer instructions. Lanes
// outside the active range compute garbage that the caller discards.
__device__ __forceinline__ F2 prim_pair(const FoldRec& F, float r2h, float r2l, const float2* __restrict__ fine) {
  const float nah = F.nah, nal = F.nal;
  const float ph = __fmul_rn(nah, r2h);
  const float pe = fmaf(nah, r2h, -ph);
  const float pl = fmaf(nah, r2l, fmaf(nal, r2h, pe));
  const float tf = fmaf(ph, kInvLFinef, 12582912.0f);  // 1.5 * 2^23: rounds to an integer
  const int n1 = __float_as_int(tf) - 0x4B400000;
  const float nf = __fsub_rn(tf, 12582912.0f);
  const float t1 = fmaf(nf, -kLh, ph);
  const float rl = fmaf(nf, -kLm, __fadd_rn(pl, F.dh));
  const float rr = __fadd_rn(t1, rl);
  const float pp = fmaf(__fmul_rn(rr, rr), fmaf(rr, 1.0f / 6.0f, 0.5f), rl);
  const int n = n1 + (int)(F.jeb & kFoldJmMask);
  const float2 T = fine[n & (kFine - 1)];
  const float ah = __fmul_rn(T.x, t1);
  const float al = fmaf(T.x, t1, -ah);
  const float s = __fadd_rn(T.x, ah);  // T.x >= 1 > |ah|: s + e = T.x + ah exactly
  const float e = __fsub_rn(ah, __fsub_rn(s, T.x));
  const float vl = __fadd_rn(__fadd_rn(e, al), fmaf(T.x, pp, fmaf(T.y, t1, T.y)));
  const float sc = __uint_as_float((F.jeb & ~kFoldJmMask) + ((unsigned)(n >> kFineBits) << 23));
  return {__fmul_rn(s, sc), __fmul_rn(vl, sc)};
}

// A primitive's contribution to the radial sums of the split-BF16 form: R += v, G += -expo v,
// H += expo^2 v (so that sum(-2 a v) = 2 G and sum(-2 a^2 v) = -2 H).
__device__ __forceinline__ void acc_prim(F2& R, F2& G, F2& H, F2 v, float nah, float nal) {
  add_pair(R, v);
  const F2 m = mul_pair(nah, nal, v.h, v.l);
  add_pair(G, m);
  add_pair(H, mul_pair(nah, nal, m.h, m.l));
}

// Collects one warp's AO values (lane = point) for ao_vgl / ao_value and writes them as row
// segments (lanes hold scattered points, so rows are staged in shared memory). Windows of
// kStage AOs are aligned to multiples of kStage (the first window of a task may be shorter):
// when the row length is a multiple of 4, a full window of ao_vgl then covers whole 32-byte
// sectors, which saves the memory system a read-modify-write per row (17 % of the FP64 AO
// kernel's time on the medium workload).
template <Out O>
struct Writer {
  static constexpr int NC = ncomp<O>();
  Stage<NC>* st;
  double* out;               // ao_vgl / ao_value
  int64_t row_len;           // ao_num
  int nvalid;                // points of the warp that exist
  int lane;
  int base;                  // AO index of stage slot 0
  int fill;                  // staged AOs
  int cap;                   // capacity of the current window
  int64_t extent;            // elements of out (bounds-checked build)

  __device__ __forceinline__ void init(const FusedArgs& a, Stage<NC>* stage, int64_t p0, int ln, int nv, int64_t p,
                                       int ao_begin) {
    st = stage;
    out = a.out;
    row_len = a.row_len;
    extent = a.point_num * NC * a.row_len;
    st->pidx[ln] = p;
    nvalid = nv;
    lane = ln;
    base = ao_begin;
    fill = 0;
    cap = kStage - (ao_begin & (kStage - 1));
  }
  __device__ __forceinline__ void flush() {
    __syncwarp();
    const int total = nvalid * NC * kStage;
    for (int i = lane; i < total; i += 32) {
      const int j = i & (kStage - 1);
      const int rest = i / kStage;
      const int c = rest % NC;
      const int q = rest / NC;
      if (j >= fill) continue;
      const int64_t pt = st->pidx[q];
      const double val = st->v[c][j][q];
      const int64_t at = pt * (NC * row_len) + c * row_len + base + j;
      if (QG_STORE_OK(kSiteAoOut, at, extent)) out[at] = val;
    }
    __syncwarp();
    base += fill;
    fill = 0;
    cap = kStage;
  }
  __device__ __forceinline__ void emit(const double (&v)[NC]) {
    if (fill == cap) flush();
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

// The split-BF16 form's AO operand, written straight from registers. Each plane is an M-major
// matrix [kp][5 pp] whose operand row (5 g + c) 64 + j is component c of the point at processing
// slot 64 g + j (64-point blocks, pp a multiple of 64): plane p, AO k of that point and component
// at planes[(p kp + k) 5 pp + (5 g + c) 64 + j]. A lane's five components of one AO then lie at
// fixed offsets (64 elements apart) from one address per plane, instead of pp apart (one address
// computation per store), and the 32 lanes of a warp (32 consecutive slots, half a block) fill 64
// contiguous bytes per store (two whole sectors); nothing is staged in shared memory. Slots past
// the last point (padding rows) are not written; the contraction discards their rows.
template <>
struct Writer<Out::Planes> {
  static constexpr int NC = 5;
  static constexpr int kBlock = 64;  // points per block (and elements between components)
  __nv_bfloat16* o;          // this lane's element of plane 0, component 0, AO row 0
  int64_t row_len;           // elements between consecutive AOs: 5 pp
  int64_t plane_stride;      // elements between the planes: kp 5 pp
  int base;                  // AO index of the next emit
  int fill;
  bool valid;                // the lane holds a point
  int64_t slot;              // offset of o in the planes (bounds-checked build)

  __device__ __forceinline__ void init(const FusedArgs& a, Stage<5>*, int64_t p0, int ln, int nv, int64_t,
                                       int ao_begin) {
    // p0 is a multiple of 32: block p0 / 64, half (p0 / 32) % 2
    slot = (p0 / kBlock) * (5 * kBlock) + (p0 & (kBlock - 1)) + ln;
    o = static_cast<__nv_bfloat16*>(a.planes) + slot;
    row_len = 5 * a.plane_pp;
    plane_stride = a.row_len * 5 * a.plane_pp;
    base = ao_begin;
    fill = 0;
    valid = ln < nv;
  }
  __device__ __forceinline__ void flush() {
    base += fill;
    fill = 0;
  }
  // Bounds-checked build: the first and last element this emit writes (plane 0 component 0,
  // plane 2 component 4) lie inside the three planes.
  __device__ __forceinline__ bool row_ok() const {
    const int64_t first = slot + (int64_t)(base + fill) * row_len;
    return QG_STORE_OK(kSiteAoPlanes, first, 3 * plane_stride) &&
           QG_STORE_OK(kSiteAoPlanes, first + 2 * plane_stride + 4 * kBlock, 3 * plane_stride);
  }
  __device__ __forceinline__ void emit(const double (&v)[NC]) {
    if (valid && row_ok()) {
      // the reference's MO kernel drops an AO whose value is exactly zero from every
      // component of the point (src/qmckl_mo_sycl.cpp:40); tested on the bit pattern (+-0),
      // which keeps the FP64 pipe free
      const bool drop = (bits_of(v[0]) << 1) == 0;
      __nv_bfloat16* r = o + (int64_t)(base + fill) * row_len;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        __nv_bfloat16 h, m, l;
        split_bf16x3(c > 0 && drop ? 0.0 : v[c], h, m, l);
        r[c * kBlock] = h;
        r[plane_stride + c * kBlock] = m;
        r[2 * plane_stride + c * kBlock] = l;
      }
    }
    fill += 1;
  }
  // value, gradient and Laplacian (assembled in FP32); drop: the AO's FP64 value is zero
  __device__ __forceinline__ void emit_mixed(float v0, float gx, float gy, float gz, float lapf, bool drop) {
    if (valid && row_ok()) {
      __nv_bfloat16* r = o + (int64_t)(base + fill) * row_len;
      const float vals[5] = {v0, drop ? 0.f : gx, drop ? 0.f : gy, drop ? 0.f : gz, drop ? 0.f : lapf};
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        __nv_bfloat16 h, m, l;
        split_bf16x3f(vals[c], h, m, l);
        r[c * kBlock] = h;
        r[plane_stride + c * kBlock] = m;
        r[2 * plane_stride + c * kBlock] = l;
      }
    }
    fill += 1;
  }
  __device__ __forceinline__ void emit_zeros(int count) {
    const double z[NC] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < count; ++i) emit(z);
  }
};

// Shell quantities shared by the shell's Cartesian components.
struct ShellVals {
  double R;    // radial value t0
  double t1, t2, t3;  // radial gradient = g * (x, y, z)
  double Rt;   // t4 + 2 l g, the radial part of the Laplacian after Euler's identity
  // split-BF16 form (FP32): the same quantities, 2 R and 6 R (shells with l = 2 and 3), and
  // whether the FP64 radial value is zero (the AO is then dropped from the derivative rows)
  float Rf, t1f, t2f, t3f, Rtf, R2f, R6f;
  bool rzero;
};

// Powers 0..3 of the displacement from the nucleus: FP64 for the FP64 outputs, FP32 for the
// split-BF16 form.
struct Pows {
  double X[4], Y[4], Z[4];
  float Xf[4], Yf[4], Zf[4];
};

// What the split-BF16 form needs to decide, per AO, whether the FP64 polynomial
// P = x^a (y^b z^c) is zero (the reference's zero-value test is on the FP64 value P R f): the
// displacements, whether each is +-0, and whether the warp needs the FP64 product itself (a
// lane with a NaN coordinate, or a displacement below 2^-340 in magnitude that could underflow
// the product; for l <= 3 no other product of nonzero displacements is zero).
struct PolyZero {
  double x, y, z;
  bool zx, zy, zz;
  bool exact;  // warp-uniform
};

template <int e>
__device__ __forceinline__ double dpow(double x) {
  if constexpr (e == 0) return 1.0;
  else if constexpr (e == 1) return x;
  else if constexpr (e == 2) return x * x;
  else return (x * x) * x;
}

template <int a, int b, int c>
__device__ __forceinline__ bool poly_zero(const PolyZero& pz) {
  if (pz.exact) return (bits_of(dpow<a>(pz.x) * (dpow<b>(pz.y) * dpow<c>(pz.z))) << 1) == 0;
  return (a > 0 && pz.zx) || (b > 0 && pz.zy) || (c > 0 && pz.zz);
}

// Powers up to L only, formed per shell: nothing of them stays live across the shell loop
// (registers), and a nucleus without d or f shells multiplies nothing.
template <Out O, int L>
__device__ __forceinline__ Pows make_pows(double x, double y, double z, float xf, float yf, float zf) {
  Pows pw;
  if constexpr (O == Out::Planes) {
    pw.Xf[0] = pw.Yf[0] = pw.Zf[0] = 1.f;
    if constexpr (L >= 1) {
      pw.Xf[1] = xf;
      pw.Yf[1] = yf;
      pw.Zf[1] = zf;
    }
    if constexpr (L >= 2) {
      pw.Xf[2] = xf * xf;
      pw.Yf[2] = yf * yf;
      pw.Zf[2] = zf * zf;
    }
    if constexpr (L >= 3) {
      pw.Xf[3] = pw.Xf[2] * xf;
      pw.Yf[3] = pw.Yf[2] * yf;
      pw.Zf[3] = pw.Zf[2] * zf;
    }
  } else {
    pw.X[0] = pw.Y[0] = pw.Z[0] = 1.0;
    if constexpr (L >= 1) {
      pw.X[1] = x;
      pw.Y[1] = y;
      pw.Z[1] = z;
    }
    if constexpr (L >= 2) {
      pw.X[2] = x * x;
      pw.Y[2] = y * y;
      pw.Z[2] = z * z;
    }
    if constexpr (L >= 3) {
      pw.X[3] = pw.X[2] * x;
      pw.Y[3] = pw.Y[2] * y;
      pw.Z[3] = pw.Z[2] * z;
    }
  }
  return pw;
}

// One Cartesian component x^a y^b z^c (a, b, c compile-time), assembled like the
// reference's src/qmckl_ao_sycl.cpp:371-420 and multiplied by the AO factor.
template <Out O, int a, int b, int c>
__device__ __forceinline__ void cart(Writer<O>& w, const Pows& pw, const ShellVals& s, double f, bool zero,
                                     const PolyZero& pz) {
  constexpr int NC = ncomp<O>();
  if constexpr (O == Out::Planes) {
    // Split-BF16 form: the planes carry 24 significant bits, so every component is assembled in
    // FP32 from the radial quantities rounded to FP32 (the Laplacian's radial part Rt is formed
    // in pair arithmetic before that rounding, so its cancellation costs no accuracy).
    const float(&Xf)[4] = pw.Xf;
    const float(&Yf)[4] = pw.Yf;
    const float(&Zf)[4] = pw.Zf;
    const float yzf = Yf[b] * Zf[c];
    const float Pf = Xf[a] * yzf;
    float gx = Pf * s.t1f, gy = Pf * s.t2f, gz = Pf * s.t3f;
    if constexpr (a > 0) gx = fmaf((float)a * Xf[a - 1], yzf * s.Rf, gx);
    if constexpr (b > 0) gy = fmaf((float)b * Yf[b - 1], (Xf[a] * Zf[c]) * s.Rf, gy);
    if constexpr (c > 0) gz = fmaf((float)c * Zf[c - 1], (Xf[a] * Yf[b]) * s.Rf, gz);
    float v0 = Pf * s.Rf;
    // l <= 3: at most one exponent e of a, b, c is 2 or more, so the polynomial's second
    // derivatives add one term e (e - 1) x^(e-2) m R, with m the other two coordinates' powers
    // (1, x, y or z) and x^(e-2) = 1 or the coordinate itself: lap = fma(P, Rt, (e (e - 1) R) m)
    static_assert(a + b + c <= 3, "the fixed-l path covers l <= 3");
    float lap;
    if constexpr (a > 1) {
      lap = fmaf(Pf, s.Rtf, (a == 2 ? s.R2f : s.R6f) * (Xf[a - 2] * yzf));
    } else if constexpr (b > 1) {
      lap = fmaf(Pf, s.Rtf, (b == 2 ? s.R2f : s.R6f) * (Yf[b - 2] * (Xf[a] * Zf[c])));
    } else if constexpr (c > 1) {
      lap = fmaf(Pf, s.Rtf, (c == 2 ? s.R2f : s.R6f) * (Zf[c - 2] * (Xf[a] * Yf[b])));
    } else {
      lap = Pf * s.Rtf;
    }
    if (!is_one(f)) {
      const float ff = f64_to_f32(f);
      v0 *= ff;
      gx *= ff;
      gy *= ff;
      gz *= ff;
      lap *= ff;
    }
    // the reference's MO kernel skips an AO whose FP64 value P R f is exactly zero
    // (src/qmckl_mo_sycl.cpp:40): decided on the FP64 factors' zero tests
    const bool drop = zero || s.rzero || (bits_of(f) << 1) == 0 || poly_zero<a, b, c>(pz);
    if (zero) v0 = 0.f;
    w.emit_mixed(v0, gx, gy, gz, lap, drop);
    return;
  }
  const double(&X)[4] = pw.X;
  const double(&Y)[4] = pw.Y;
  const double(&Z)[4] = pw.Z;
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

// The AO factor of AO i: 1 without a load when the shell's factors are all exactly 1 (unit is
// warp-uniform; the load is predicated, so no code is duplicated).
__device__ __forceinline__ double ao_factor_at(const double* __restrict__ aof, int i, bool unit) {
  double f = 1.0;
  if (!unit) f = __ldg(aof + i);
  return f;
}

// Components of one shell in the reference's order: a descending, then b descending
// (src/qmckl_ao_sycl.cpp:297-305).
template <Out O, int L>
__device__ __forceinline__ void shell_fixed(Writer<O>& w, const Pows& pw, const ShellVals& sv_in,
                                            const double* __restrict__ aof, int ao0, bool unit, bool zero,
                                            const PolyZero& pz) {
  ShellVals s = sv_in;
  if constexpr (O == Out::Planes && L >= 2) {
    s.R2f = s.Rf + s.Rf;  // exact
    if constexpr (L >= 3) s.R6f = 3.f * s.R2f;
  }
  if constexpr (L == 0) {
    cart<O, 0, 0, 0>(w, pw, s, ao_factor_at(aof, ao0, unit), zero, pz);
  } else if constexpr (L == 1) {
    cart<O, 1, 0, 0>(w, pw, s, ao_factor_at(aof, ao0 + 0, unit), zero, pz);
    cart<O, 0, 1, 0>(w, pw, s, ao_factor_at(aof, ao0 + 1, unit), zero, pz);
    cart<O, 0, 0, 1>(w, pw, s, ao_factor_at(aof, ao0 + 2, unit), zero, pz);
  } else if constexpr (L == 2) {
    cart<O, 2, 0, 0>(w, pw, s, ao_factor_at(aof, ao0 + 0, unit), zero, pz);
    cart<O, 1, 1, 0>(w, pw, s, ao_factor_at(aof, ao0 + 1, unit), zero, pz);
    cart<O, 1, 0, 1>(w, pw, s, ao_factor_at(aof, ao0 + 2, unit), zero, pz);
    cart<O, 0, 2, 0>(w, pw, s, ao_factor_at(aof, ao0 + 3, unit), zero, pz);
    cart<O, 0, 1, 1>(w, pw, s, ao_factor_at(aof, ao0 + 4, unit), zero, pz);
    cart<O, 0, 0, 2>(w, pw, s, ao_factor_at(aof, ao0 + 5, unit), zero, pz);
  } else {
    cart<O, 3, 0, 0>(w, pw, s, ao_factor_at(aof, ao0 + 0, unit), zero, pz);
    cart<O, 2, 1, 0>(w, pw, s, ao_factor_at(aof, ao0 + 1, unit), zero, pz);
    cart<O, 2, 0, 1>(w, pw, s, ao_factor_at(aof, ao0 + 2, unit), zero, pz);
    cart<O, 1, 2, 0>(w, pw, s, ao_factor_at(aof, ao0 + 3, unit), zero, pz);
    cart<O, 1, 1, 1>(w, pw, s, ao_factor_at(aof, ao0 + 4, unit), zero, pz);
    cart<O, 1, 0, 2>(w, pw, s, ao_factor_at(aof, ao0 + 5, unit), zero, pz);
    cart<O, 0, 3, 0>(w, pw, s, ao_factor_at(aof, ao0 + 6, unit), zero, pz);
    cart<O, 0, 2, 1>(w, pw, s, ao_factor_at(aof, ao0 + 7, unit), zero, pz);
    cart<O, 0, 1, 2>(w, pw, s, ao_factor_at(aof, ao0 + 8, unit), zero, pz);
    cart<O, 0, 0, 3>(w, pw, s, ao_factor_at(aof, ao0 + 9, unit), zero, pz);
  }
}

// Generic path for l >= 4 (rare): powers in local memory, same formulas. Inlined: a call would
// take the address of the caller's writer and keep the hot path's writer state in local memory.
template <Out O>
__device__ __forceinline__ void shell_generic(Writer<O>& w, double x, double y, double z, int L, const ShellVals& s,
                                              const double* __restrict__ aof, int ao0, bool zero) {
  constexpr int NC = ncomp<O>();
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


// A displacement that is nonzero and below 2^-340 in magnitude (biased exponent below 683): a
// product of such powers could underflow, so the zero test of the FP64 polynomial needs the
// product itself.
__device__ __forceinline__ bool tiny_disp(double x) {
  const uint64_t b = bits_of(x) << 1;
  return b != 0 && b < (683ull << 53);
}

// One warp task: 32 points (lane = point) x one chunk of consecutive nuclei. G: the basis has
// shells with l >= 4 (the generic path is compiled in only then, since its local arrays and
// extra live values cost the common kernel registers).
template <Out O, bool G, bool B, bool S, bool kSkipDead = true>
__device__ __forceinline__ void ao_task_at(const FusedArgs& a, int64_t group, const NucleusChunk* chunk,
                                           Stage<ncomp<O>()>* st, const double* __restrict__ thi,
                                           const double* __restrict__ tlo, const float2* __restrict__ fine,
                                           double* __restrict__ ebuf, int lane) {
  constexpr int NC = ncomp<O>();
  const int64_t p0 = group * 32;
  const int64_t remaining = a.point_num - p0;
  const int nvalid = remaining < 32 ? (int)remaining : 32;
  const int64_t slot = p0 + (lane < nvalid ? lane : nvalid - 1);
  const int64_t p = a.perm ? (int64_t)a.perm[slot] : slot;
  const double ex = a.coord[p], ey = a.coord[a.coord_ld + p], ez = a.coord[2 * a.coord_ld + p];

  const NucleusChunk cj = *chunk;
  Writer<O> w;
  w.init(a, st, p0, lane, nvalid, p, cj.ao_begin);

  for (int n = cj.nucl_begin; n < cj.nucl_end; ++n) {
    const NucleusEntry& N = a.nuclei[n];
    // the nucleus's shells, or with S the chunk's part of them (a piece). Compiled in only where
    // pieces are used: the clamped bounds cost the batch kernel 40 % (2.27 -> 3.18 ms on the
    // 64-molecule batch's planes)
    int s_begin = N.shell_begin, s_end = N.shell_end;
    if constexpr (S) {
      s_begin = max(s_begin, cj.shell_lo);
      s_end = min(s_end, cj.shell_hi);
    }
    const double x = ex - N.x, y = ey - N.y, z = ez - N.z;
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    const uint64_t r2b = bits_of(r2);
    // A NaN coordinate makes r2 NaN. The reference's screening tests (`r2 > cutoff * range`,
    // `expo * r2 > cutoff`) are false for NaN, so it screens nothing and every primitive gives
    // exp(NaN) = NaN (src/qmckl_ao_sycl.cpp:53,72-75): such a lane is never screened here, and
    // the radial sums of its shells with primitives become NaN below. Screened: screen_bits <
    // r2b <= bits(+inf), as one unsigned range compare (NaN patterns lie above +inf); written as
    // `r2b > screen_bits && !nan` the kernel measured 21 % slower (1.20 against 0.99 ms on the
    // medium workload's planes).
    const bool nanr = (r2b << 1) > 0xFFE0000000000000ull;
    const bool scr = r2b - N.screen_bits - 1ull < 0x7FF0000000000000ull - N.screen_bits;
    const bool nan_warp = __any_sync(kFull, nanr);  // warp-uniform: the NaN fix-up below costs a branch
    if (__all_sync(kFull, scr)) {
      if constexpr (S) {
        const int ao_lo = s_begin == N.shell_begin ? N.ao_begin : a.shells[s_begin].ao_begin;
        const int ao_hi = s_end == N.shell_end ? N.ao_end : a.shells[s_end].ao_begin;
        w.emit_zeros(ao_hi - ao_lo);
      } else {
        w.emit_zeros(N.ao_end - N.ao_begin);
      }
      continue;
    }
    if constexpr (O == Out::Planes) {
      // Split-BF16 form: radials in FP32 pair arithmetic (the FP64 pipe only forms r2 and its
      // split), assembly in FP32.
      const float xf = f64_to_f32(x), yf = f64_to_f32(y), zf = f64_to_f32(z);
      const float r2h = f64_to_f32(r2);
      const float r2l = f64_to_f32(r2 - f32_to_f64(r2h));  // r2h + r2l = r2 to ~2^-48
      PolyZero pz;
      pz.x = x;
      pz.y = y;
      pz.z = z;
      pz.zx = (bits_of(x) << 1) == 0;
      pz.zy = (bits_of(y) << 1) == 0;
      pz.zz = (bits_of(z) << 1) == 0;
      pz.exact = nan_warp || __any_sync(kFull, !scr && (tiny_disp(x) || tiny_disp(y) || tiny_disp(z)));
      const bool pairs = a.fold != nullptr;  // uniform: the basis is in the folded range
      // Shared exponentials (B): each distinct exponent of the nucleus once per lane, as a pair
      // in this lane's column of the warp's buffer; the shells' primitives multiply it by their
      // coefficient.
      bool shared_e = false;
      if constexpr (B) {
        if (a.ent && pairs) {
          shared_e = true;
          float2* eb = reinterpret_cast<float2*>(ebuf);
          for (int u = 0; u < N.ent_num; ++u) {
            const FoldRec E = load_fold(a.ent + N.ent_begin + u);
            const bool act = !scr && (r2b < E.thr);
            if (__any_sync(kFull, act)) {
              const F2 e = prim_pair(E, r2h, r2l, fine);
              eb[u * 32 + lane] = make_float2(act ? e.h : 0.f, act ? e.l : 0.f);
            }
          }
        }
      }
      for (int si = s_begin; si < s_end; ++si) {
        const ShellEntry sh = a.shells[si];
        F2 R{0.f, 0.f}, Gs{0.f, 0.f}, Hs{0.f, 0.f};  // sum v, sum -expo v, sum expo^2 v
        double t0 = 0.0, g = 0.0, h = 0.0;           // FP64 sums (basis outside the folded range)
        if (pairs) {
          if (shared_e) {
            const float2* eb = reinterpret_cast<const float2*>(ebuf);
            for (int pi = sh.prim_begin; pi < sh.prim_end; ++pi) {
              const FoldRec F = load_fold(a.fold + pi);
              const bool act = !scr && (r2b < F.thr);
              if (__any_sync(kFull, act)) {
                const float2 e = eb[__ldg(&a.prims[pi].ent) * 32 + lane];
                F2 v = mul_pair(F.ch, F.cl, e.x, e.y);
                if (!act) v = F2{0.f, 0.f};
                acc_prim(R, Gs, Hs, v, F.nah, F.nal);
              }
            }
          } else {
            for (int pi = sh.prim_begin; pi < sh.prim_end; ++pi) {
              const FoldRec F = load_fold(a.fold + pi);
              const bool act = !scr && (r2b < F.thr);
              if (__any_sync(kFull, act)) {
                F2 v = prim_pair(F, r2h, r2l, fine);
                if (!act) v = F2{0.f, 0.f};
                acc_prim(R, Gs, Hs, v, F.nah, F.nal);
              }
            }
          }
        } else {
          for (int pi = sh.prim_begin; pi < sh.prim_end; ++pi) {
            const bool act = !scr && (r2b < __ldg(&a.prims[pi].thr_bits));
            if (__any_sync(kFull, act)) {
              const double ar2 = __ldg(&a.prims[pi].expo) * r2;
              const double e = exp_neg(ar2, thi, tlo);
              const double v = keep_if(act, __ldg(&a.prims[pi].coef) * e);
              t0 += v;
              const double two_a = __ldg(&a.prims[pi].m2a) * v;
              g += two_a;
              h = fma(two_a, ar2, h);
            }
          }
        }
        if (nan_warp) {
          // every primitive of a NaN lane is NaN in the reference; the outputs follow by arithmetic
          // (the FP32 quantities become NaN, and so does the contraction)
          if (nanr && sh.prim_end > sh.prim_begin) {
            R.h = Gs.h = Hs.h = __uint_as_float(0x7FC00000u);
            t0 = g = h = __longlong_as_double(0x7FF8000000000000ll);
          }
        } else if (kSkipDead) {
          // no lane has a nonzero radial sum (every primitive screened for the warp's points: about
          // a third of the shells a warp evaluates on the medium workload, mostly tight core
          // shells): the shell's AOs are zero in every component, written without the assembly
          const bool nz = pairs ? ((__float_as_uint(R.h) | __float_as_uint(R.l) | __float_as_uint(Gs.h) |
                                    __float_as_uint(Gs.l) | __float_as_uint(Hs.h) | __float_as_uint(Hs.l)) << 1) != 0
                                : ((bits_of(t0) | bits_of(g) | bits_of(h)) << 1) != 0;
          if (!__any_sync(kFull, nz)) {
            w.emit_zeros((sh.l + 1) * (sh.l + 2) / 2);
            continue;
          }
        }
        ShellVals sv;
        float gf;
        F2 rt{0.f, 0.f};
        double Rt = 0.0;
        if (pairs) {
          // Rt = sum v (4 expo^2 r2 - 2 expo (3 + 2l)) = 2 ((3 + 2l) G + 2 r2 H), the
          // cancellation-prone part of the Laplacian, in pair arithmetic before one rounding
          sv.Rf = __fadd_rn(R.h, R.l);
          gf = 2.f * __fadd_rn(Gs.h, Gs.l);
          rt = mul_pair((float)(3 + 2 * sh.l), 0.f, Gs.h, Gs.l);
          const F2 rh = mul_pair(r2h, r2l, Hs.h, Hs.l);
          add_pair(rt, F2{2.f * rh.h, 2.f * rh.l});
          sv.Rtf = 2.f * __fadd_rn(rt.h, rt.l);
          sv.rzero = R.h == -R.l;  // the FP64 value R.h + R.l is zero
        } else {
          Rt = fma(kTwoL[sh.l], g, fma(-2.0, h, 3.0 * g));
          sv.Rf = f64_to_f32(t0);
          gf = f64_to_f32(g);
          sv.Rtf = f64_to_f32(Rt);
          sv.rzero = (bits_of(t0) << 1) == 0;
        }
        sv.t1f = gf * xf;
        sv.t2f = gf * yf;
        sv.t3f = gf * zf;
        switch (sh.l) {
          case 0: shell_fixed<O, 0>(w, make_pows<O, 0>(x, y, z, xf, yf, zf), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          case 1: shell_fixed<O, 1>(w, make_pows<O, 1>(x, y, z, xf, yf, zf), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          case 2: shell_fixed<O, 2>(w, make_pows<O, 2>(x, y, z, xf, yf, zf), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          case 3: shell_fixed<O, 3>(w, make_pows<O, 3>(x, y, z, xf, yf, zf), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          default:
            if constexpr (G) {  // the generic path assembles in FP64
              const double g64 = pairs ? 2.0 * (f32_to_f64(Gs.h) + f32_to_f64(Gs.l)) : g;
              sv.R = pairs ? f32_to_f64(R.h) + f32_to_f64(R.l) : t0;
              sv.Rt = pairs ? 2.0 * (f32_to_f64(rt.h) + f32_to_f64(rt.l)) : Rt;
              sv.t1 = g64 * x;
              sv.t2 = g64 * y;
              sv.t3 = g64 * z;
              shell_generic<O>(w, x, y, z, sh.l, sv, a.aof, sh.ao_begin, scr);
            }
            break;
        }
      }
      continue;
    } else {
      // Shared exponentials (B): each distinct exponent of the nucleus once per lane, kept in
      // this lane's column of the warp's buffer; the shells' primitives then read them
      // (coef * e^(-expo r2) with the same operations as the per-primitive loop: bit-identical
      // results).
      bool shared_e = false;
      if constexpr (B) {
        if (a.ent) {
          shared_e = true;
          for (int u = 0; u < N.ent_num; ++u) {
            const PrimFold* E = a.ent + N.ent_begin + u;
            const bool act = !scr && (r2b < __ldg(&E->thr_bits));
            if (__any_sync(kFull, act)) {
              const double e = exp_neg((-__ldg(&E->na)) * r2, thi, tlo);
              ebuf[u * 32 + lane] = keep_if(act, e);
            }
          }
        }
      }
      for (int si = s_begin; si < s_end; ++si) {
        const ShellEntry sh = a.shells[si];
        double t0 = 0.0, g = 0.0, h = 0.0;
        if (shared_e) {
          for (int pi = sh.prim_begin; pi < sh.prim_end; ++pi) {
            const PrimEntry* P = a.prims + pi;
            const bool act = !scr && (r2b < __ldg(&P->thr_bits));
            if (__any_sync(kFull, act)) {
              double v = __ldg(&P->coef) * ebuf[__ldg(&P->ent) * 32 + lane];
              v = keep_if(act, v);
              t0 += v;
              if constexpr (NC == 5) {
                const double ar2 = __ldg(&P->expo) * r2;
                const double two_a = __ldg(&P->m2a) * v;
                g += two_a;
                h = fma(two_a, ar2, h);
              }
            }
          }
        } else {
          for (int pi = sh.prim_begin; pi < sh.prim_end; ++pi) {
            const bool act = !scr && (r2b < __ldg(&a.prims[pi].thr_bits));
            if (__any_sync(kFull, act)) {
              const double expo = __ldg(&a.prims[pi].expo);
              const double ar2 = expo * r2;
              const double e = exp_neg(ar2, thi, tlo);
              double v = __ldg(&a.prims[pi].coef) * e;
              v = keep_if(act, v);
              t0 += v;
              if constexpr (NC == 5) {
                const double two_a = __ldg(&a.prims[pi].m2a) * v;
                g += two_a;
                h = fma(two_a, ar2, h);
              }
            }
          }
        }
        if (nan_warp) {
          // every primitive of a NaN lane is NaN in the reference; the outputs follow by arithmetic
          if (nanr && sh.prim_end > sh.prim_begin) t0 = g = h = __longlong_as_double(0x7FF8000000000000ll);
        } else if (kSkipDead && !__any_sync(kFull, ((bits_of(t0) | bits_of(g) | bits_of(h)) << 1) != 0)) {
          // no lane has a nonzero radial sum: the shell's AOs are zero in every component,
          // written without the assembly
          w.emit_zeros((sh.l + 1) * (sh.l + 2) / 2);
          continue;
        }
        ShellVals sv;
        sv.R = t0;
        if constexpr (NC == 5) {
          sv.t1 = g * x;
          sv.t2 = g * y;
          sv.t3 = g * z;
          // a shell without primitives has a zero radial gradient in the reference, also at a NaN
          // coordinate (where g * x would be NaN)
          if (nan_warp && nanr && sh.prim_end == sh.prim_begin) sv.t1 = sv.t2 = sv.t3 = 0.0;
          const double t4 = fma(-2.0, h, 3.0 * g);
          sv.Rt = fma(kTwoL[sh.l], g, t4);
        } else {
          sv.t1 = sv.t2 = sv.t3 = sv.Rt = 0.0;
        }
        const PolyZero pz{};
        switch (sh.l) {
          case 0: shell_fixed<O, 0>(w, make_pows<O, 0>(x, y, z, 0.f, 0.f, 0.f), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          case 1: shell_fixed<O, 1>(w, make_pows<O, 1>(x, y, z, 0.f, 0.f, 0.f), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          case 2: shell_fixed<O, 2>(w, make_pows<O, 2>(x, y, z, 0.f, 0.f, 0.f), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          case 3: shell_fixed<O, 3>(w, make_pows<O, 3>(x, y, z, 0.f, 0.f, 0.f), sv, a.aof, sh.ao_begin, sh.unit_aof != 0, scr, pz); break;
          default:
            if constexpr (G) shell_generic<O>(w, x, y, z, sh.l, sv, a.aof, sh.ao_begin, scr);
            break;
        }
      }
    }
  }
  // BF16 planes are padded to a multiple of 64 columns; the last chunk zeroes the padding
  if constexpr (O == Out::Planes) {
    if (cj.ao_end == a.ao_num) w.emit_zeros((int)(a.row_len - a.ao_num));
  }
  w.flush();
}

// Task `task` of a single-molecule launch: its segment (the last one starting at or before it,
// selected with constant indices so that the kernel-parameter arrays are read in place), then
// its point group and chunk.
template <Out O, bool G, bool B, bool S>
__device__ __forceinline__ void ao_task(const FusedArgs& a, int64_t task, Stage<ncomp<O>()>* st,
                                        const double* __restrict__ thi, const double* __restrict__ tlo,
                                        const float2* __restrict__ fine, double* __restrict__ ebuf, int lane) {
  int64_t t0 = a.seg_task[0], g0 = a.seg_group[0];
  const NucleusChunk* c0 = a.seg_chunks[0];
  int cn = a.seg_chunk_num[0];
#pragma unroll
  for (int k = 1; k < FusedArgs::kMaxSegments; ++k) {
    if (k < a.nseg && task >= a.seg_task[k]) {
      t0 = a.seg_task[k];
      g0 = a.seg_group[k];
      c0 = a.seg_chunks[k];
      cn = a.seg_chunk_num[k];
    }
  }
  const int64_t t = task - t0;
  const int64_t g = t / cn;
  ao_task_at<O, G, B, S>(a, g0 + g, c0 + (t - g * cn), st, thi, tlo, fine, ebuf, lane);
}

// Dynamic shared memory of the fused kernels: tables, staging buffers (ao_vgl / ao_value), then
// with shared exponentials one column of ent_cap doubles per lane.
template <Out O>
__host__ __device__ constexpr size_t fused_smem(int ent_cap = 0) {
  const size_t base = O == Out::Planes ? stage_offset<O>() : stage_offset<O>() + sizeof(Stage<ncomp<O>()>) * kWarps;
  return base + (size_t)kWarps * 32 * sizeof(double) * (size_t)(ent_cap > 0 ? ent_cap : 0);
}

// Per-CTA setup shared by the kernels: the exponential's tables into shared memory, and this
// warp's staging buffer and exponential buffer.
template <Out O>
struct CtaSmem {
  double *thi, *tlo, *ebuf;
  float2* fine;
  Stage<ncomp<O>()>* st;
  __device__ __forceinline__ CtaSmem(unsigned char* raw, const ExpTable* tab, int ent_cap, int warp) {
    thi = reinterpret_cast<double*>(raw);
    tlo = thi + 32;
    fine = reinterpret_cast<float2*>(thi + 64);  // split-BF16 planes only
    load_exp_table(tab->hi, tab->lo, thi, tlo);
    if constexpr (O == Out::Planes)
      for (int i = threadIdx.x; i < kFine; i += blockDim.x) fine[i] = tab->fine[i];
    st = reinterpret_cast<Stage<ncomp<O>()>*>(raw + stage_offset<O>()) + warp;
    ebuf = reinterpret_cast<double*>(raw + fused_smem<O>(0)) + (size_t)warp * 32 * (ent_cap > 0 ? ent_cap : 0);
  }
};

// One molecule. counter null: warp task = blockIdx.x * kWarps + warp. Otherwise persistent:
// each warp takes the next task from *counter (zeroed before the launch) until none is left,
// so that every SM gets the same share of the FP64 work whatever the grid's tail.
// G: shells with l >= 4 exist; B: shared exponentials (a.ent non-null).
template <Out O, bool G, bool B, bool S>
__global__ void __launch_bounds__(kWarps * 32, min_ctas<O>()) ao_fused_kernel(const FusedArgs a,
                                                                              unsigned long long* counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const CtaSmem<O> sm(smem_raw, a.exp_table, B ? a.ent_cap : 0, warp);
  __syncthreads();
  if (!counter) {
    const int64_t task = (int64_t)blockIdx.x * kWarps + warp;
    if (task < a.task_num) ao_task<O, G, B, S>(a, task, sm.st, sm.thi, sm.tlo, sm.fine, sm.ebuf, lane);  // warp-uniform
    return;
  }
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(counter, 1ull);
    t = __shfl_sync(kFull, t, 0);
    if (t >= (unsigned long long)a.task_num) break;
    ao_task<O, G, B, S>(a, (int64_t)t, sm.st, sm.thi, sm.tlo, sm.fine, sm.ebuf, lane);
  }
}

// Many molecules, persistent: each warp takes the next task from a global counter until the
// tasks of every molecule are done (uneven molecules balance themselves). ent_cap: the largest
// AoTables::ent_cap of the molecules with shared exponentials (B).
template <Out O, bool G, bool B>
__global__ void __launch_bounds__(kWarps * 32, min_ctas<O>()) ao_batch_kernel(const FusedArgs* __restrict__ mols,
                                                                const int64_t* __restrict__ task_begin, int nmol,
                                                                int64_t total, unsigned long long* counter,
                                                                int ent_cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const CtaSmem<O> sm(smem_raw, mols[0].exp_table, B ? ent_cap : 0, warp);
  __syncthreads();
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(counter, 1ull);
    t = __shfl_sync(kFull, t, 0);
    if (t >= (unsigned long long)total) break;
    const int64_t task = (int64_t)t;
    int lo = 0, hi = nmol - 1;  // last molecule whose first task is <= task
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (task_begin[mid] <= task) lo = mid;
      else hi = mid - 1;
    }
    const FusedArgs& a = mols[lo];  // fields read from global memory as needed (registers)
    const int64_t local = task - task_begin[lo];  // one segment per molecule
    const int cn = a.chunk_num;
    const int64_t g = local / cn;
    // the FP64 outputs skip shells that are zero on every lane (64-molecule ao_vgl 6.06 -> 5.33 ms);
    // the planes do not: there the test cost the batch kernel more than it saved (2.26 ms without,
    // 2.38 ms with it, also with the arguments copied to shared memory; with the FP32 pair radials
    // 1.392 ms without, 1.434 ms with it)
    ao_task_at<O, G, B, false, O != Out::Planes || kBatchPlanesSkipDead>(a, g, a.chunks + (local - g * cn), sm.st,
                                                                          sm.thi, sm.tlo, sm.fine,
                                                 sm.ebuf, lane);
  }
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
  if (!QG_STORE_OK(kSiteShellVgl, ip * 5 * shell_num + os + 4 * shell_num, point_num * 5 * shell_num)) return;
  // NaN r2 screens nothing, as the reference's `>` tests (every primitive then gives NaN)
  const bool nanr = (bits_of(r2) << 1) > 0xFFE0000000000000ull;
  if (bits_of(r2) > N.screen_bits && !nanr) {
    o[0] = o[shell_num] = o[2 * shell_num] = o[3 * shell_num] = o[4 * shell_num] = 0.0;
    return;
  }
  const ShellEntry S = shells[si];
  double t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0;
  for (int pi = S.prim_begin; pi < S.prim_end; ++pi) {
    const PrimEntry Pr = prims[pi];
    if (bits_of(r2) >= Pr.thr_bits && !nanr) continue;
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

// ---------------------------------------------------------------- point order
__device__ __forceinline__ int morton_key(double x, double y, double z, const double* origin, double inv_cell);

// 15-bit Morton key of a point's cell on the 32^3 grid; one counter per cell.
__global__ void morton_key_kernel(const double* __restrict__ coord, int64_t ld, int64_t P, double ox, double oy,
                                  double oz, double inv_cell, int32_t* __restrict__ keys, int32_t* __restrict__ counts) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const double origin[3] = {ox, oy, oz};
  const int key = morton_key(coord[p], coord[ld + p], coord[2 * ld + p], origin, inv_cell);
  keys[p] = key;
  atomicAdd(&counts[key], 1);
}

// In-place exclusive prefix sum of kOrderCells counters per CTA of 1024 threads (CTA b scans
// the counters of molecule b): each thread scans 32 consecutive counters read as eight 16-byte
// vectors, a warp scans its threads' sums by shuffles, warp 0 the 32 warp sums.
__global__ void __launch_bounds__(1024) cell_scan_kernel(int32_t* __restrict__ counts_all) {
  static_assert(kOrderCells == 1024 * 32, "one thread per 32 counters");
  int4* __restrict__ counts = reinterpret_cast<int4*>(counts_all + (int64_t)blockIdx.x * kOrderCells);
  __shared__ int32_t warp_sum[32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  int4 v[8];
  int32_t s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    v[i] = counts[t * 8 + i];
    s += v[i].x + v[i].y + v[i].z + v[i].w;
  }
  int32_t incl = s;  // inclusive scan of the thread sums within the warp
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int32_t u = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += u;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int32_t w = warp_sum[lane];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += u;
    }
    warp_sum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int32_t run = (warp > 0 ? warp_sum[warp - 1] : 0) + incl - s;  // exclusive start of this thread
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int4 o;
    o.x = run;
    run += v[i].x;
    o.y = run;
    run += v[i].y;
    o.z = run;
    run += v[i].z;
    o.w = run;
    run += v[i].w;
    counts[t * 8 + i] = o;
  }
}

__global__ void cell_scatter_kernel(const int32_t* __restrict__ keys, int64_t P, int32_t* __restrict__ offsets,
                                    int32_t* __restrict__ perm) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int pos = atomicAdd(&offsets[keys[p]], 1);
  if (QG_STORE_OK(kSitePointPerm, pos, P)) perm[pos] = (int32_t)p;
}

// Picks the first nucleus-chunk level with at least `target` warp tasks; when none has that
// many, the pieces (level index ao_level_count(t)) if allowed and there are more of them. The
// FP64 outputs do not take pieces as their level: a piece's AO columns start and end inside the
// 8-AO windows they are stored in, and those partial windows cost more than the balance gains
// (CHBrClF, 40,960 points: ao_vgl 0.72 ms with pieces against 0.57 ms; the planes kernel, which
// stores whole 64-byte segments per AO, 0.058 against 0.116 ms).
int pick_level(const AoTables& t, int64_t groups, int64_t target, bool pieces) {
  const int levels = (int)t.level_offsets.size();
  for (int lv = 0; lv < levels; ++lv)
    if (groups * (int64_t)t.level_sizes[lv] >= target) return lv;
  return pieces && t.piece_num > t.level_sizes[levels - 1] ? levels : levels - 1;
}


// Resident CTAs per SM of a kernel with `smem` bytes of dynamic shared memory.
template <class K>
int resident_per_sm(K kernel, size_t smem) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kWarps * 32, smem) != cudaSuccess) n = 1;
  cudaGetLastError();
  return n > 0 ? n : 1;
}

template <Out O, bool G, bool B>
cudaError_t launch_fused_g(Ctx* ctx, const AoTables& t, const double* coord, const int32_t* perm, int64_t point_num,
                           double* out, __nv_bfloat16* planes, int64_t row_len, const char* name, int64_t coord_ld) {
  const int64_t groups = (point_num + 31) / 32;
  const size_t smem = fused_smem<O>(B ? t.ent_cap : 0);
  static size_t cached_smem = 0;
  static int cached_per_sm = 0;
  if (cached_smem != smem || cached_per_sm == 0) {
    cached_per_sm = resident_per_sm(ao_fused_kernel<O, G, B, false>, smem);
    cached_smem = smem;
  }
  constexpr bool kPieces = O == Out::Planes;  // the FP64 outputs never take pieces (see pick_level)
  const int per_sm = cached_per_sm;
  const int64_t resident_warps = (int64_t)t.sm_count * per_sm * kWarps;
  // tasks taken from a counter, two or more per resident warp for the FP64 outputs: with one task
  // per warp the SMs that receive one CTA more than the others set the time (4 or 5 CTAs per SM on
  // the medium workload, 16 % idle FP64 issue); the planes' shorter tasks balance with one
  const int level = pick_level(t, groups, (O == Out::Planes ? kPlanesTasksPerWarp : kTasksPerWarp) * resident_warps,
                               kPieces);
  FusedArgs a = make_fused_args(t, level, coord, perm, point_num, out, planes, row_len);
  // the last tasks at ever finer nucleus-chunk levels: a warp's last task is short, so the launch
  // ends with every warp busy nearly to the end (a task at the coarse level takes ~1/3 of the
  // launch, and a lone warp runs a nucleus's FP64 work on one sub-partition's FP64 unit).
  // Measured on the medium workload's planes (40,960 points): 0.968 ms against 1.005 ms for one
  // segment; ending with pieces too 0.980 ms (the kernel with clamped shell ranges is slower);
  // with about 4 or 16 times as many tail tasks 1.010 / 1.062 ms, and with 4, 8 or 32 tasks per
  // warp at the coarse level 1.05 / 1.09 / 1.36 ms (finer tasks cost more than they balance:
  // every task takes a global counter and reloads its points).
  plan_segments(a, t, level, resident_warps, kTailSegments, false);
  bool pieces = false;  // some task evaluates a piece of a nucleus: the kernel with clamped shell ranges
  for (int i = 0; i < a.nseg; ++i) pieces = pieces || a.seg_chunks[i] == t.chunks + t.piece_offset;
  if (coord_ld >= 0) a.coord_ld = coord_ld;
  a.ent = B ? t.ent : nullptr;
  a.ent_cap = B ? t.ent_cap : 0;
  unsigned long long* counter = nullptr;
  int64_t blocks = (a.task_num + kWarps - 1) / kWarps;
  if (a.task_num > resident_warps) {
    if (!ctx->task_counter)
      ctx->task_counter = static_cast<unsigned long long*>(dalloc(ctx, sizeof(unsigned long long)));
    if (!ctx->task_counter) return cudaErrorMemoryAllocation;
    counter = ctx->task_counter;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream);
    if (e != cudaSuccess) return e;
    blocks = (int64_t)t.sm_count * per_sm;
  }
  LaunchScope scope(ctx, name);
  if constexpr (kPieces) {
    if (pieces) {
      cudaFuncSetAttribute(ao_fused_kernel<O, G, B, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      ao_fused_kernel<O, G, B, true><<<(unsigned)blocks, kWarps * 32, smem, ctx->stream>>>(a, counter);
      return cudaGetLastError();
    }
  }
  cudaFuncSetAttribute(ao_fused_kernel<O, G, B, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  ao_fused_kernel<O, G, B, false><<<(unsigned)blocks, kWarps * 32, smem, ctx->stream>>>(a, counter);
  return cudaGetLastError();
}

// Without an explicit request, sharing serves the FP64 outputs only (the tables exist only
// when the basis passes the activity-weighted test at build time). Measured on 40960 points:
// generally contracted basis (26 distinct exponents for 103 primitives per nucleus) ao_vgl
// 3.19 -> 2.60 ms although the buffer halves the resident CTAs, but the split-BF16 planes
// 1.44 -> 1.50 ms (their folded primitive costs 10 FP64 instructions against 18, so less is
// saved); CHBrClF (repeats mostly among steep, mostly screened primitives) ao_vgl 0.58 -> 0.72.
template <Out O>
bool share_by_default() {
  return O != Out::Planes;
}

template <Out O>
cudaError_t launch_fused(Ctx* ctx, const AoTables& t, const double* coord, const int32_t* perm, int64_t point_num,
                         double* out, __nv_bfloat16* planes, int64_t row_len, const char* name, int64_t coord_ld = -1) {
  if (point_num <= 0 || t.ao_num <= 0) return cudaSuccess;
  const bool g = t.lmax > 3, b = t.ent != nullptr && (t.ent_forced || share_by_default<O>());
  if (g && b) return launch_fused_g<O, true, true>(ctx, t, coord, perm, point_num, out, planes, row_len, name, coord_ld);
  if (g) return launch_fused_g<O, true, false>(ctx, t, coord, perm, point_num, out, planes, row_len, name, coord_ld);
  if (b) return launch_fused_g<O, false, true>(ctx, t, coord, perm, point_num, out, planes, row_len, name, coord_ld);
  return launch_fused_g<O, false, false>(ctx, t, coord, perm, point_num, out, planes, row_len, name, coord_ld);
}

__device__ __forceinline__ int morton_key(double x, double y, double z, const double* origin, double inv_cell) {
  const double c[3] = {(x - origin[0]) * inv_cell, (y - origin[1]) * inv_cell, (z - origin[2]) * inv_cell};
  int key = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int q = c[d] > 0.0 ? (c[d] < 31.0 ? (int)c[d] : 31) : 0;  // NaN goes to cell 0
#pragma unroll
    for (int b = 0; b < 5; ++b) key |= ((q >> b) & 1) << (3 * b + d);
  }
  return key;
}

// Molecule owning global point gp: the last m with point_begin[m] <= gp.
__device__ __forceinline__ int owner_of(const int64_t* __restrict__ point_begin, int nmol, int64_t gp) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (point_begin[mid] <= gp) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void batch_key_kernel(const OrderDesc* __restrict__ desc, const int64_t* __restrict__ point_begin, int nmol,
                                 int64_t total, int32_t* __restrict__ counts) {
  const int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gp >= total) return;
  const int m = owner_of(point_begin, nmol, gp);
  const OrderDesc& d = desc[m];
  const int64_t p = gp - point_begin[m];
  const int64_t P = d.point_num;
  const int key = morton_key(d.coord[p], d.coord[P + p], d.coord[2 * P + p], d.origin, d.inv_cell);
  d.keys[p] = key;
  atomicAdd(&counts[(int64_t)m * kOrderCells + key], 1);
}

__global__ void batch_scatter_kernel(const OrderDesc* __restrict__ desc, const int64_t* __restrict__ point_begin,
                                     int nmol, int64_t total, int32_t* __restrict__ offsets) {
  const int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gp >= total) return;
  const int m = owner_of(point_begin, nmol, gp);
  const OrderDesc& d = desc[m];
  const int64_t p = gp - point_begin[m];
  const int pos = atomicAdd(&offsets[(int64_t)m * kOrderCells + d.keys[p]], 1);
  if (QG_STORE_OK(kSitePointPerm, pos, d.point_num)) d.perm[pos] = (int32_t)p;
}

// The range of point p among nr consecutive ranges: the last r with bounds[r] <= p.
__device__ __forceinline__ int range_of(const int64_t* __restrict__ bounds, int nr, int64_t p) {
  int lo = 0, hi = nr - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bounds[mid] <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void range_key_kernel(const double* __restrict__ coord, int64_t P, double ox, double oy, double oz,
                                 double inv_cell, const int64_t* __restrict__ bounds, int nr,
                                 int32_t* __restrict__ keys, int32_t* __restrict__ counts) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const double origin[3] = {ox, oy, oz};
  const int key = morton_key(coord[p], coord[P + p], coord[2 * P + p], origin, inv_cell);
  keys[p] = key;
  atomicAdd(&counts[(int64_t)range_of(bounds, nr, p) * kOrderCells + key], 1);
}

__global__ void range_scatter_kernel(const int32_t* __restrict__ keys, int64_t P, const int64_t* __restrict__ bounds,
                                     int nr, int32_t* __restrict__ offsets, int32_t* __restrict__ perm) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int r = range_of(bounds, nr, p);
  const int64_t at = bounds[r] + atomicAdd(&offsets[(int64_t)r * kOrderCells + keys[p]], 1);
  if (QG_STORE_OK(kSitePointPerm, at, P)) perm[at] = (int32_t)(p - bounds[r]);
}

}  // namespace

int ao_level_count(const AoTables& t) { return (int)t.level_offsets.size(); }

bool ao_shared_exponentials(const AoTables& t, bool planes) {
  if (!t.ent) return false;
  if (planes && !t.fold) return false;  // the planes share exponentials in the folded evaluation only
  return t.ent_forced || (planes ? share_by_default<Out::Planes>() : share_by_default<Out::Vgl>());
}

FusedArgs make_fused_args(const AoTables& t, int level, const double* coord, const int32_t* perm, int64_t point_num,
                          double* out, void* planes, int64_t row_len) {
  const int levels = (int)t.level_offsets.size();
  const bool pieces = level >= levels && t.piece_num > 0;
  const int lv = level < 0 ? 0 : (level >= levels ? levels - 1 : level);
  FusedArgs a;
  a.nuclei = t.nuclei;
  a.shells = t.shells;
  a.prims = t.prims;
  a.aof = t.ao_factor;
  a.chunk_num = pieces ? t.piece_num : t.level_sizes[lv];
  a.chunks = t.chunks + (pieces ? t.piece_offset : t.level_offsets[lv]);
  a.exp_table = t.exp_table;
  a.fold = t.fold;
  const bool share = ao_shared_exponentials(t, planes != nullptr);
  a.ent = share ? t.ent : nullptr;
  a.ent_cap = share ? t.ent_cap : 0;
  a.coord = coord;
  a.perm = perm;
  a.out = out;
  a.planes = planes;
  a.point_num = point_num;
  a.ao_num = t.ao_num;
  a.row_len = row_len;
  a.plane_pp = (point_num + 63) / 64 * 64;
  a.coord_ld = point_num;
  a.task_num = ((point_num + 31) / 32) * a.chunk_num;
  a.nseg = 1;
  a.seg_task[0] = 0;
  a.seg_task[1] = a.task_num;
  a.seg_group[0] = 0;
  a.seg_chunks[0] = a.chunks;
  a.seg_chunk_num[0] = a.chunk_num;
  return a;
}

void plan_segments(FusedArgs& a, const AoTables& t, int level, int64_t tail_tasks, int max_segments, bool pieces) {
  const int64_t groups = (a.point_num + 31) / 32;
  if (max_segments > FusedArgs::kMaxSegments) max_segments = FusedArgs::kMaxSegments;
  // finer partitions from the finest up: the pieces, then the levels finer than a's
  struct Part {
    const NucleusChunk* chunks;
    int num;
  };
  std::vector<Part> finer;
  if (pieces && t.piece_num > a.chunk_num) finer.push_back(Part{t.chunks + t.piece_offset, t.piece_num});
  for (int lv = (int)t.level_offsets.size() - 1; lv > level; --lv)
    if (t.level_sizes[lv] > a.chunk_num && (finer.empty() || t.level_sizes[lv] < finer.back().num))
      finer.push_back(Part{t.chunks + t.level_offsets[lv], t.level_sizes[lv]});
  // groups of each finer segment (about tail_tasks tasks), finest first, at most half of all
  std::vector<int64_t> take;
  int64_t used = 0;
  for (const Part& p : finer) {
    if ((int)take.size() + 1 >= max_segments) break;
    int64_t g = (tail_tasks + p.num - 1) / p.num;
    if (used + g > groups / 2) g = groups / 2 - used;
    if (g <= 0) break;
    take.push_back(g);
    used += g;
  }
  a.nseg = 1;
  int64_t group = groups - used, task = group * a.chunk_num;
  for (int k = (int)take.size() - 1; k >= 0; --k) {  // coarse to fine
    const int i = a.nseg++;
    a.seg_task[i] = task;
    a.seg_group[i] = group;
    a.seg_chunks[i] = finer[k].chunks;
    a.seg_chunk_num[i] = finer[k].num;
    group += take[k];
    task += take[k] * finer[k].num;
  }
  a.seg_task[a.nseg] = task;
  a.task_num = task;
}

template <Out O, bool G, bool B>
int batch_per_sm(int ent_cap) {
  return resident_per_sm(ao_batch_kernel<O, G, B>, fused_smem<O>(B ? ent_cap : 0));
}

template <Out O>
int batch_per_sm_of(bool high_l, int ent_cap) {
  if (high_l) return ent_cap > 0 ? batch_per_sm<O, true, true>(ent_cap) : batch_per_sm<O, true, false>(0);
  return ent_cap > 0 ? batch_per_sm<O, false, true>(ent_cap) : batch_per_sm<O, false, false>(0);
}

int ao_batch_resident_ctas(bool planes, bool high_l, int ent_cap) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaGetLastError();
  const int per_sm = planes ? batch_per_sm_of<Out::Planes>(high_l, ent_cap) : batch_per_sm_of<Out::Vgl>(high_l, ent_cap);
  return sms * per_sm;
}

template <Out O, bool G, bool B>
void launch_batch_g(cudaStream_t stream, const FusedArgs* mols, const int64_t* task_begin, int nmol, int64_t total,
                    unsigned long long* counter, int grid, int ent_cap) {
  const size_t smem = fused_smem<O>(B ? ent_cap : 0);
  cudaFuncSetAttribute(ao_batch_kernel<O, G, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  ao_batch_kernel<O, G, B><<<grid, kWarps * 32, smem, stream>>>(mols, task_begin, nmol, total, counter, ent_cap);
}

template <Out O>
void launch_batch_of(cudaStream_t stream, bool high_l, int ent_cap, const FusedArgs* mols, const int64_t* task_begin,
                     int nmol, int64_t total, unsigned long long* counter, int grid) {
  if (high_l && ent_cap > 0) launch_batch_g<O, true, true>(stream, mols, task_begin, nmol, total, counter, grid, ent_cap);
  else if (high_l) launch_batch_g<O, true, false>(stream, mols, task_begin, nmol, total, counter, grid, 0);
  else if (ent_cap > 0) launch_batch_g<O, false, true>(stream, mols, task_begin, nmol, total, counter, grid, ent_cap);
  else launch_batch_g<O, false, false>(stream, mols, task_begin, nmol, total, counter, grid, 0);
}

cudaError_t launch_ao_batch(cudaStream_t stream, bool planes, bool high_l, int ent_cap, const FusedArgs* mols,
                            const int64_t* task_begin, int nmol, int64_t total, unsigned long long* counter,
                            int grid) {
  if (nmol <= 0 || total <= 0) return cudaSuccess;
  if (grid <= 0) grid = ao_batch_resident_ctas(planes, high_l, ent_cap);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  if (planes) launch_batch_of<Out::Planes>(stream, high_l, ent_cap, mols, task_begin, nmol, total, counter, grid);
  else launch_batch_of<Out::Vgl>(stream, high_l, ent_cap, mols, task_begin, nmol, total, counter, grid);
  return cudaGetLastError();
}

cudaError_t launch_order_batch(cudaStream_t stream, const OrderDesc* desc, const int64_t* point_begin, int nmol,
                               int64_t total_points, int32_t* counts) {
  if (nmol <= 0 || total_points <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int32_t) * kOrderCells * (size_t)nmol, stream);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((total_points + 255) / 256);
  batch_key_kernel<<<blocks, 256, 0, stream>>>(desc, point_begin, nmol, total_points, counts);
  cell_scan_kernel<<<nmol, 1024, 0, stream>>>(counts);
  batch_scatter_kernel<<<blocks, 256, 0, stream>>>(desc, point_begin, nmol, total_points, counts);
  return cudaGetLastError();
}

cudaError_t launch_point_order(Ctx* ctx, const AoTables& t, const double* coord, int64_t coord_ld, int64_t point_num,
                               int32_t* keys, int32_t* counts, int32_t* perm) {
  if (point_num <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int32_t) * kOrderCells, ctx->stream);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((point_num + 255) / 256);
  {
    LaunchScope scope(ctx, "point_order_keys");
    morton_key_kernel<<<blocks, 256, 0, ctx->stream>>>(coord, coord_ld, point_num, t.grid_origin[0], t.grid_origin[1],
                                                       t.grid_origin[2], t.grid_inv_cell, keys, counts);
  }
  {
    LaunchScope scope(ctx, "point_order_scan");
    cell_scan_kernel<<<1, 1024, 0, ctx->stream>>>(counts);
  }
  LaunchScope scope(ctx, "point_order_scatter");
  cell_scatter_kernel<<<blocks, 256, 0, ctx->stream>>>(keys, point_num, counts, perm);
  return cudaGetLastError();
}

cudaError_t launch_point_order_ranges(Ctx* ctx, const AoTables& t, const double* coord, int64_t point_num,
                                      const int64_t* bounds, int nr, int32_t* keys, int32_t* counts, int32_t* perm) {
  if (point_num <= 0 || nr <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int32_t) * kOrderCells * (size_t)nr, ctx->stream);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((point_num + 255) / 256);
  {
    LaunchScope scope(ctx, "point_order_keys");
    range_key_kernel<<<blocks, 256, 0, ctx->stream>>>(coord, point_num, t.grid_origin[0], t.grid_origin[1],
                                                      t.grid_origin[2], t.grid_inv_cell, bounds, nr, keys, counts);
  }
  {
    LaunchScope scope(ctx, "point_order_scan");
    cell_scan_kernel<<<nr, 1024, 0, ctx->stream>>>(counts);
  }
  LaunchScope scope(ctx, "point_order_scatter");
  range_scatter_kernel<<<blocks, 256, 0, ctx->stream>>>(keys, point_num, bounds, nr, counts, perm);
  return cudaGetLastError();
}

cudaError_t launch_ao_vgl(Ctx* ctx, const AoTables& t, const double* coord, const int32_t* perm, int64_t point_num,
                          double* ao_vgl) {
  return launch_fused<Out::Vgl>(ctx, t, coord, perm, point_num, ao_vgl, nullptr, t.ao_num, "ao_vgl_fused");
}

cudaError_t launch_ao_value(Ctx* ctx, const AoTables& t, const double* coord, const int32_t* perm,
                            int64_t point_num, double* ao_value) {
  return launch_fused<Out::Value>(ctx, t, coord, perm, point_num, ao_value, nullptr, t.ao_num, "ao_value_fused");
}

cudaError_t launch_ao_planes(Ctx* ctx, const AoTables& t, const double* coord, int64_t coord_ld, const int32_t* perm,
                             int64_t point_num, int64_t kp, void* planes) {
  return launch_fused<Out::Planes>(ctx, t, coord, perm, point_num, nullptr, static_cast<__nv_bfloat16*>(planes), kp,
                                   "ao_vgl_fused_bf16_planes", coord_ld);
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

// ---------------------------------------------------------------- exponential check
namespace {
__global__ void exp_check_kernel(const double* __restrict__ x, int64_t n, const ExpTable* __restrict__ tab,
                                 double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[2 * i] = exp_neg(x[i], tab->hi, tab->lo);
  out[2 * i + 1] = exp(-x[i]);
}
}  // namespace

namespace {
// Primitive values coef * e^(-expo r2) as the split-BF16 form's AO kernel evaluates them (the
// folded FP32 pair evaluation, hi + lo as a double, or the FP64 form's when the tables have no
// folded list), zero where the primitive is screened; out[i][prim_orig[k]] for packed
// primitive k.
__global__ void prim_check_kernel(const PrimFold* __restrict__ fold, const PrimEntry* __restrict__ prims,
                                  const ExpTable* __restrict__ tab, const int32_t* __restrict__ prim_orig,
                                  const double* __restrict__ r2, int64_t n, int packed, int64_t prim_num,
                                  double* __restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * packed) return;
  const int64_t i = idx / packed;
  const int k = (int)(idx - i * packed);
  const double r = r2[i];
  double v = 0.0;
  if (fold) {
    if (bits_of(r) < fold[k].thr_bits) {
      const float rh = f64_to_f32(r);
      const F2 p = prim_pair(load_fold(fold + k), rh, f64_to_f32(r - f32_to_f64(rh)), tab->fine);
      v = f32_to_f64(p.h) + f32_to_f64(p.l);
    }
  } else if (bits_of(r) < prims[k].thr_bits) {
    v = prims[k].coef * exp_neg(prims[k].expo * r, tab->hi, tab->lo);
  }
  out[i * prim_num + prim_orig[k]] = v;
}
}  // namespace

cudaError_t launch_prim_check(Ctx* ctx, const AoTables& t, const double* r2, int64_t n, int64_t prim_num,
                              double* out) {
  if (n <= 0 || prim_num <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * n * prim_num, ctx->stream);
  if (e != cudaSuccess || t.prim_num == 0) return e;
  const int64_t total = n * t.prim_num;
  LaunchScope scope(ctx, "prim_check");
  prim_check_kernel<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(t.fold, t.prims, t.exp_table,
                                                                              t.prim_orig, r2, n, t.prim_num,
                                                                              prim_num, out);
  return cudaGetLastError();
}

cudaError_t launch_exp_check(Ctx* ctx, const ExpTable* tab, const double* x, int64_t n, double* out) {
  if (n <= 0) return cudaSuccess;
  LaunchScope scope(ctx, "exp_check");
  exp_check_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(x, n, tab, out);
  return cudaGetLastError();
}

}  // namespace qg
