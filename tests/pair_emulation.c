/* CPU emulation of the split-BF16 AO kernel's FP32 pair arithmetic, for the error-bound test
 * tests/test_pair_emulation.py (test infrastructure; nothing in the library uses it).
 *
 * It restates, in binary32 C arithmetic (fmaf is correctly rounded, and the file is compiled with
 * -ffp-contract=off so that no other product is fused), the device functions prim_pair, acc_prim,
 * mul_pair and add_pair of qmckl_sycl_gb300/csrc/ao_kernels.cu and the host record of
 * fold_entry in qmckl_sycl_gb300/csrc/ao_basis.cpp, then compares with long double:
 *   - every primitive value c e^(-a r2) over random r2 in the active range a r2 <= 27.63
 *     (relative error);
 *   - per synthetic shell (1..6 primitives of mixed-sign coefficients, l = 0..3) the FP32 values
 *     of R = sum v, the radial gradient factor 2 G = sum -2 a v and the Laplacian's radial part
 *     Rt = 2 ((3 + 2l) G + 2 r2 H), each against sum |terms| (the cancellation-aware measure).
 *
 * Input (stdin): K, then K pairs (exponent, normalised coefficient) as doubles, binary.
 * Output: "prim <max rel err> <evaluations>" and "shell <R> <2G> <Rt>" lines. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define KFINE_BITS 10
#define KFINE (1 << KFINE_BITS)
static const double kCutoff = 27.631021115928547;

static float Th[KFINE], Tl[KFINE];
static float kInvLFinef, kLh, kLm;

static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static int32_t f2i(float f) { int32_t i; memcpy(&i, &f, 4); return i; }

typedef struct { float h, l; } F2;
typedef struct { float nah, nal, dh; uint32_t jeb; } Rec;

static Rec fold_entry(double expo, double coef) {
  Rec r;
  memset(&r, 0, sizeof r);
  r.nah = (float)(-expo);
  r.nal = (float)(-expo - (double)r.nah);
  int e2 = 0;
  const double m = frexp(fabs(coef), &e2);
  const int k = e2 - 1;
  const long double L = logl(2.0L) / (long double)KFINE;
  const long double lnm = logl(2.0L * (long double)m);
  const long double jm = roundl(lnm / L);
  r.dh = (float)(lnm - jm * L);
  r.jeb = ((uint32_t)(k + 127) << 23) | (signbit(coef) ? 0x80000000u : 0u) | ((uint32_t)jm & 0xFFFu);
  return r;
}

static F2 prim_pair(const Rec* F, float r2h, float r2l) {
  const float ph = F->nah * r2h;
  const float pe = fmaf(F->nah, r2h, -ph);
  const float pl = fmaf(F->nah, r2l, fmaf(F->nal, r2h, pe));
  const float tf = fmaf(ph, kInvLFinef, 12582912.0f);
  const int n1 = f2i(tf) - 0x4B400000;
  const float nf = tf - 12582912.0f;
  const float t1 = fmaf(nf, -kLh, ph);
  const float rl = fmaf(nf, -kLm, pl + F->dh);
  const float rr = t1 + rl;
  const float pp = fmaf(rr * rr, fmaf(rr, 1.0f / 6.0f, 0.5f), rl);
  const int n = n1 + (int)(F->jeb & 0xFFFu);
  const float tx = Th[n & (KFINE - 1)], ty = Tl[n & (KFINE - 1)];
  const float ah = tx * t1;
  const float al = fmaf(tx, t1, -ah);
  const float s = tx + ah;
  const float e = ah - (s - tx);
  const float vl = (e + al) + fmaf(tx, pp, fmaf(ty, t1, ty));
  const float sc = u2f((F->jeb & ~0xFFFu) + ((uint32_t)(n >> KFINE_BITS) << 23));
  F2 v = {s * sc, vl * sc};
  return v;
}

static F2 mul_pair(float xh, float xl, float yh, float yl) {
  const float p = xh * yh;
  const float e = fmaf(xh, yh, -p);
  F2 r = {p, fmaf(xh, yl, fmaf(xl, yh, e))};
  return r;
}

static void add_pair(F2* s, F2 b) {
  const float t = s->h + b.h;
  const float bb = t - s->h;
  const float err = (s->h - (t - bb)) + (b.h - bb);
  s->l = s->l + (err + b.l);
  s->h = t;
}

static double urand(void) { return (double)rand() / (double)RAND_MAX; }

int main(void) {
  const double kLFine = 0.6931471805599453094 / KFINE;
  kInvLFinef = (float)(KFINE / 0.6931471805599453094);
  kLh = (float)kLFine;
  kLm = (float)(kLFine - (double)kLh);
  for (int j = 0; j < KFINE; ++j) {
    const long double t = exp2l((long double)j / KFINE);
    Th[j] = (float)t;
    Tl[j] = (float)(t - (long double)Th[j]);
  }
  int64_t K = 0;
  if (fread(&K, sizeof K, 1, stdin) != 1 || K <= 0) return 2;
  double* d = (double*)malloc(sizeof(double) * 2 * (size_t)K);
  if (!d || fread(d, sizeof(double), 2 * (size_t)K, stdin) != 2 * (size_t)K) return 2;
  srand(1);
  double worst = 0.0;
  long evals = 0;
  for (int64_t p = 0; p < K; ++p) {
    const double a = d[2 * p], c = d[2 * p + 1];
    if (c == 0.0) continue;
    const Rec F = fold_entry(a, c);
    for (int t = 0; t < 400; ++t) {
      const double u = urand();
      const double r2 = (t % 2) ? u * kCutoff / a : exp(log(1e-12) + u * (log(kCutoff / a) - log(1e-12)));
      if (a * r2 > kCutoff) continue;
      const float r2h = (float)r2, r2l = (float)(r2 - (double)r2h);
      const F2 v = prim_pair(&F, r2h, r2l);
      const long double ex = (long double)c * expl(-(long double)a * (long double)r2);
      const double rel = (double)fabsl(((long double)v.h + (long double)v.l - ex) / ex);
      if (rel > worst) worst = rel;
      ++evals;
    }
  }
  printf("prim %.6e %ld\n", worst, evals);
  double wR = 0.0, wg = 0.0, wt = 0.0;
  for (int trial = 0; trial < 20000; ++trial) {
    const int np = 1 + rand() % 6, l = rand() % 4;
    double ea[6], ec[6];
    for (int i = 0; i < np; ++i) {
      ea[i] = exp(log(0.03) + urand() * (log(1e5) - log(0.03)));
      ec[i] = (urand() * 2.0 - 1.0) * pow(10.0, (double)(rand() % 6) - 2.0);
    }
    const double r2 = urand() * 30.0 / ea[0];
    const float r2h = (float)r2, r2l = (float)(r2 - (double)r2h);
    F2 R = {0.f, 0.f}, G = {0.f, 0.f}, H = {0.f, 0.f};
    long double eR = 0, eg = 0, et = 0, aR = 0, ag = 0, at = 0;
    for (int i = 0; i < np; ++i) {
      if (ea[i] * r2 > kCutoff) continue;
      const Rec F = fold_entry(ea[i], ec[i]);
      const F2 v = prim_pair(&F, r2h, r2l);
      add_pair(&R, v);
      const F2 m = mul_pair(F.nah, F.nal, v.h, v.l);
      add_pair(&G, m);
      add_pair(&H, mul_pair(F.nah, F.nal, m.h, m.l));
      const long double V = (long double)ec[i] * expl(-(long double)ea[i] * (long double)r2);
      eR += V;
      aR += fabsl(V);
      eg += -2.0L * ea[i] * V;
      ag += fabsl(2.0L * ea[i] * V);
      et += V * (4.0L * ea[i] * ea[i] * r2 - 2.0L * ea[i] * (3 + 2 * l));
      at += fabsl(V * 4.0L * ea[i] * ea[i] * r2) + fabsl(V * 2.0L * ea[i] * (3 + 2 * l));
    }
    if (aR == 0) continue;
    const float Rf = R.h + R.l, gf = 2.f * (G.h + G.l);
    F2 rt = mul_pair((float)(3 + 2 * l), 0.f, G.h, G.l);
    const F2 rh = mul_pair(r2h, r2l, H.h, H.l);
    const F2 rh2 = {2.f * rh.h, 2.f * rh.l};
    add_pair(&rt, rh2);
    const float Rtf = 2.f * (rt.h + rt.l);
    const double e1 = (double)(fabsl((long double)Rf - eR) / aR);
    const double e2 = (double)(fabsl((long double)gf - eg) / ag);
    const double e3 = (double)(fabsl((long double)Rtf - et) / at);
    if (e1 > wR) wR = e1;
    if (e2 > wg) wg = e2;
    if (e3 > wt) wt = e3;
  }
  printf("shell %.6e %.6e %.6e\n", wR, wg, wt);
  free(d);
  return 0;
}
