// AO basis: setters/getters with the reference's mask, finalize and exit-code semantics
// (src/qmckl_ao.cpp:402-1765 of qmckl_sycl), the finalize step (src/qmckl_ao_sycl.cpp:
// 1067-1236) done on the host, the packed tables for the fused kernels, and the lazy,
// date-stamped provide chain (src/qmckl_ao.cpp:47-199, src/qmckl_ao_sycl.cpp:748-849).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.hpp"

using namespace qg;

namespace {

constexpr int32_t kAoMaskAll = (1 << 14) - 1;

Ctx* checked(qmckl_context_device c) {
  return qmckl_context_check_device(c) == QMCKL_NULL_CONTEXT_DEVICE ? nullptr : ctx_of(c);
}

template <class T>
std::vector<T> to_host(Ctx* ctx, qmckl_context_device c, const T* d, int64_t n, qmckl_exit_code_device* rc) {
  std::vector<T> h((size_t)std::max<int64_t>(n, 0));
  if (n > 0) *rc = copy(ctx, c, h.data(), d, sizeof(T) * (size_t)n, "qmckl_finalize_ao_basis_device", true);
  return h;
}

template <class T>
T* to_device(Ctx* ctx, const std::vector<T>& h) {
  T* d = static_cast<T*>(dalloc(ctx, sizeof(T) * std::max<size_t>(h.size(), 1)));
  if (d && !h.empty() &&
      cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    dfree(ctx, d);
    return nullptr;
  }
  return d;
}

uint64_t bits_of(double x) {
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
}

// Smallest non-negative double r2 with fl(expo * r2) > cutoff, as a bit pattern; the
// primitive test of src/qmckl_ao_sycl.cpp:72 is then `bits(r2) >= thr`. fl(expo*r2) is
// monotone non-decreasing in r2, so the set of screened r2 is an up-set.
uint64_t prim_threshold(double expo) {
  const double inf = HUGE_VAL;
  if (!(expo > 0.0)) return bits_of(inf);  // never screened (the reference's test is false)
  if (std::isinf(expo)) return bits_of(std::nextafter(0.0, 1.0));
  volatile double e = expo;  // keep every product a plain, separately rounded multiply
  double c = kCutoff / expo;
  if (!std::isfinite(c)) c = std::numeric_limits<double>::max();
  for (int i = 0; i < 64 && c > 0.0 && e * std::nextafter(c, 0.0) > kCutoff; ++i) c = std::nextafter(c, 0.0);
  for (int i = 0; i < 64 && !(e * c > kCutoff); ++i) c = std::nextafter(c, inf);
  return bits_of(c);
}

// The split-BF16 form's record of one primitive (or, with coef 1, one distinct exponent):
// -expo as an FP32 pair, |coef| = mant 2^k with ln(mant) = jm L + dh (L = ln 2 / kFine, jm the
// nearest integer), sign * 2^k as float bits packed with jm, and coef as an FP32 pair (a
// distinct exponent keeps -expo as a double there instead). The remainders are formed in long
// double, then rounded once to float.
PrimFold fold_entry(double expo, double coef, uint64_t thr_bits, bool distinct_exponent) {
  PrimFold f{};
  f.thr_bits = thr_bits;
  f.nah = (float)(-expo);
  f.nal = (float)(-expo - (double)f.nah);  // the difference is exact in double
  if (distinct_exponent) {
    f.na = -expo;
  } else {
    f.c.ch = (float)coef;
    f.c.cl = (float)(coef - (double)f.c.ch);
  }
  if (coef != 0.0 && std::isfinite(coef)) {
    int e2 = 0;
    const double m = std::frexp(std::fabs(coef), &e2);  // |coef| = m 2^e2, m in [0.5, 1)
    const int k = e2 - 1;
    const long double L = logl(2.0L) / (long double)kFine;
    const long double lnm = logl(2.0L * (long double)m);
    const long double jm = roundl(lnm / L);
    f.dh = (float)(lnm - jm * L);
    const uint32_t ebase =
        ((uint32_t)(std::min(std::max(k, -126), 127) + 127) << 23) | (std::signbit(coef) ? 0x80000000u : 0u);
    f.jeb = ebase | ((uint32_t)jm & kFoldJmMask);
  }
  return f;
}

int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Per-nucleus exponent tables of src/qmckl_ao_sycl.cpp:855-1065: each nucleus' primitives
// sorted by exponent (a bubble sort exchanging on a strict '<', as the reference's, so that
// ties keep the shell order and the result is the reference's for any input), runs of equal
// exponents merged into one entry whose per-shell coefficient is the sum of the run's
// coefficients of that shell in sorted order (the entry keeps the run's last exponent value).
// A nucleus without primitives reports one zero entry, like the reference.
struct HpcTables {
  int64_t prim_max = 0, shell_max = 0;
  std::vector<int32_t> num;
  std::vector<double> expo, coef;
};

HpcTables hpc_tables(int64_t N, const std::vector<int64_t>& nidx, const std::vector<int64_t>& nsh,
                     const std::vector<int64_t>& spi, const std::vector<int64_t>& spn,
                     const std::vector<double>& expo, const std::vector<double>& cn) {
  HpcTables h;
  for (int64_t n = 0; n < N; ++n) {
    int64_t k = 0;
    for (int64_t s = nidx[n]; s < nidx[n] + nsh[n]; ++s) k += spn[s];
    h.prim_max = std::max(h.prim_max, k);
    h.shell_max = std::max(h.shell_max, nsh[n]);
  }
  const int64_t PM = h.prim_max, SM = h.shell_max;
  h.num.assign((size_t)N, 0);
  h.expo.assign((size_t)(N * PM), 0.0);
  h.coef.assign((size_t)(N * SM * PM), 0.0);
  if (PM == 0) return h;
  struct Entry {
    double e;
    int32_t shell;  // nucleus-local shell
    int64_t prim;   // user primitive index
  };
  std::vector<Entry> v;
  for (int64_t n = 0; n < N; ++n) {
    v.clear();
    for (int64_t j = 0; j < nsh[n]; ++j) {
      const int64_t s = nidx[n] + j;
      for (int64_t p = spi[s]; p < spi[s] + spn[s]; ++p) v.push_back(Entry{expo[p], (int32_t)j, p});
    }
    const size_t k = v.size();
    for (size_t pass = 1; pass < k; ++pass) {
      bool swapped = false;
      for (size_t j = 0; j + pass < k; ++j)
        if (v[j + 1].e < v[j].e) {
          std::swap(v[j], v[j + 1]);
          swapped = true;
        }
      if (!swapped) break;
    }
    double* ex = h.expo.data() + n * PM;
    double* co = h.coef.data() + n * SM * PM;
    int64_t u = 0;
    for (size_t i = 0; i < k; ++i) {
      if (i > 0 && v[i].e != v[i - 1].e) ++u;
      ex[u] = v[i].e;
      co[v[i].shell * PM + u] += cn[(size_t)v[i].prim];
    }
    h.num[(size_t)n] = (int32_t)(u + 1);
  }
  return h;
}

// Stores the tables in the context (device arrays), replacing earlier ones.
qmckl_exit_code_device store_hpc(Ctx* ctx, qmckl_context_device c, const HpcTables& h, const char* fn) {
  AoBasisData& ao = ctx->ao_basis;
  dfree(ctx, ao.prim_num_per_nucleus);
  dfree(ctx, ao.expo_per_nucleus);
  dfree(ctx, ao.coef_per_nucleus);
  ao.prim_num_per_nucleus = to_device(ctx, h.num);
  ao.expo_per_nucleus = to_device(ctx, h.expo);
  ao.coef_per_nucleus = to_device(ctx, h.coef);
  ao.hpc_prim_max = h.prim_max;
  ao.hpc_shell_max = h.shell_max;
  if (!ao.prim_num_per_nucleus || !ao.expo_per_nucleus || !ao.coef_per_nucleus)
    return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  return QMCKL_SUCCESS_DEVICE;
}

void free_tables(Ctx* ctx, AoTables& t) {
  dfree(ctx, t.nuclei);
  dfree(ctx, t.shells);
  dfree(ctx, t.prims);
  dfree(ctx, t.ao_factor);
  dfree(ctx, t.shell_orig);
  dfree(ctx, t.shell_nucl);
  dfree(ctx, t.prim_orig);
  dfree(ctx, t.chunks);
  dfree(ctx, t.exp_table);
  dfree(ctx, t.fold);
  dfree(ctx, t.ent);
  t.exp_table = nullptr;
  t.fold = nullptr;
  t.ent = nullptr;
  t.ent_cap = 0;
  t.ent_forced = false;
  t.nuclei = nullptr;
  t.shells = nullptr;
  t.prims = nullptr;
  t.ao_factor = nullptr;
  t.shell_orig = t.shell_nucl = t.prim_orig = nullptr;
  t.chunks = nullptr;
  t.valid = false;
}

// Splits nuclei [0, n) into `parts` contiguous chunks of near-equal cost.
void split_chunks(const std::vector<NucleusEntry>& nuc, const std::vector<double>& cost, int parts,
                  std::vector<NucleusChunk>& out) {
  const int n = (int)nuc.size();
  double total = 0;
  for (double c : cost) total += c;
  int begin = 0;
  double acc = 0;
  for (int k = 0; k < parts && begin < n; ++k) {
    const double target = total * (k + 1) / parts;
    int end = begin;
    while (end < n && (end == begin || acc + cost[end] <= target + 1e-9 || k == parts - 1)) {
      acc += cost[end];
      ++end;
      if (k < parts - 1 && acc >= target) break;
    }
    if (end == begin) end = begin + 1;
    out.push_back(NucleusChunk{begin, end, nuc[begin].ao_begin, nuc[end - 1].ao_end, nuc[begin].shell_begin,
                               nuc[end - 1].shell_end});
    begin = end;
  }
  if (begin < n) {  // leftovers go to the last chunk
    out.back().nucl_end = n;
    out.back().ao_end = nuc[n - 1].ao_end;
    out.back().shell_hi = nuc[n - 1].shell_end;
  }
}

// Pieces: each nucleus's shells in consecutive ranges of cost about `target` (at least one shell
// each; nuclei without shells have none), appended to out.
void split_pieces(const std::vector<NucleusEntry>& nuc, const std::vector<ShellEntry>& shells,
                  const std::vector<double>& shell_cost, double target, std::vector<NucleusChunk>& out) {
  for (int n = 0; n < (int)nuc.size(); ++n) {
    int s = nuc[n].shell_begin;
    while (s < nuc[n].shell_end) {
      const int lo = s;
      double acc = shell_cost[s++];
      while (s < nuc[n].shell_end && acc + shell_cost[s] <= target) acc += shell_cost[s++];
      const int ao_hi = s < nuc[n].shell_end ? shells[s].ao_begin : nuc[n].ao_end;
      out.push_back(NucleusChunk{n, n + 1, shells[lo].ao_begin, ao_hi, lo, s});
    }
  }
}

}  // namespace

namespace qg {

// Builds the packed tables from the host copies of the basis and the nucleus coordinates.
qmckl_exit_code_device build_tables(Ctx* ctx, qmckl_context_device c) {
  AoBasisData& ao = ctx->ao_basis;
  const char* fn = "qmckl_finalize_ao_basis_device";
  if (ctx->nucleus.uninitialized & (1 << 2))
    return fail(c, QMCKL_NOT_PROVIDED_DEVICE, fn, "nucleus coordinates are not set");
  const int64_t N = ctx->nucleus.num, S = ao.shell_num, K = ao.prim_num, A = ao.ao_num;
  qmckl_exit_code_device rc = QMCKL_SUCCESS_DEVICE;
  auto nidx = to_host(ctx, c, ao.nucleus_index, N, &rc);
  auto nsh = to_host(ctx, c, ao.nucleus_shell_num, N, &rc);
  auto lam = to_host(ctx, c, ao.shell_ang_mom, S, &rc);
  auto spn = to_host(ctx, c, ao.shell_prim_num, S, &rc);
  auto spi = to_host(ctx, c, ao.shell_prim_index, S, &rc);
  auto expo = to_host(ctx, c, ao.exponent, K, &rc);
  auto cn = to_host(ctx, c, ao.coefficient_normalized, K, &rc);
  auto aof = to_host(ctx, c, ao.ao_factor, A, &rc);
  auto ncoord = to_host(ctx, c, ctx->nucleus.coord, 3 * N, &rc);
  auto nrange = to_host(ctx, c, ao.nucleus_range, N, &rc);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  AoTables& t = ao.tables;
  free_tables(ctx, t);
  t.h_nuclei.clear();
  t.h_shells.clear();
  t.h_prims.clear();
  t.h_fold.clear();
  t.h_ent.clear();
  t.h_chunks.clear();
  t.h_shell_orig.clear();
  t.h_prim_orig.clear();
  t.h_shell_nucl.clear();
  t.level_offsets.clear();
  t.level_sizes.clear();
  std::vector<double> cost, shell_cost;
  int ao_counter = 0, lmax = 0;
  for (int64_t n = 0; n < N; ++n) {
    NucleusEntry e{};
    e.x = ncoord[n];
    e.y = ncoord[N + n];
    e.z = ncoord[2 * N + n];
    e.screen_bits = bits_of(kCutoff * nrange[n]);
    e.shell_begin = (int32_t)t.h_shells.size();
    e.ao_begin = ao_counter;
    e.lmax = 0;
    double w = 0;
    if (nidx[n] < 0 || nsh[n] < 0 || nidx[n] + nsh[n] > S)
      return fail(c, QMCKL_FAILURE_DEVICE, fn, "nucleus_index/nucleus_shell_num out of range");
    for (int64_t s = nidx[n]; s < nidx[n] + nsh[n]; ++s) {
      const int l = lam[s];
      if (l < 0 || l > kMaxL) return fail(c, QMCKL_FAILURE_DEVICE, fn, "shell_ang_mom out of range (0..19)");
      if (spi[s] < 0 || spn[s] < 0 || spi[s] + spn[s] > K)
        return fail(c, QMCKL_FAILURE_DEVICE, fn, "shell_prim_index/shell_prim_num out of range");
      ShellEntry se{};
      se.prim_begin = (int32_t)t.h_prims.size();
      for (int64_t p = spi[s]; p < spi[s] + spn[s]; ++p) {
        PrimEntry pe{};
        pe.expo = expo[p];
        pe.coef = cn[p];
        pe.m2a = -2.0 * expo[p];
        pe.m2a2 = -2.0 * (expo[p] * expo[p]);
        pe.thr_bits = prim_threshold(expo[p]);
        t.h_prims.push_back(pe);
        t.h_prim_orig.push_back((int32_t)p);
      }
      se.prim_end = (int32_t)t.h_prims.size();
      se.ao_begin = ao_counter;
      se.l = (int16_t)l;
      se.unit_aof = 1;
      for (int i = 0; i < ncart(l); ++i)
        if (ao_counter + i >= A || !(aof[(size_t)(ao_counter + i)] == 1.0)) se.unit_aof = 0;
      ao_counter += ncart(l);
      e.lmax = std::max(e.lmax, l);
      w += (double)spn[s] + 0.5 * ncart(l);
      shell_cost.push_back((double)spn[s] + 0.5 * ncart(l));
      t.h_shells.push_back(se);
      t.h_shell_orig.push_back((int32_t)s);
      t.h_shell_nucl.push_back((int32_t)n);
    }
    e.shell_end = (int32_t)t.h_shells.size();
    e.ao_end = ao_counter;
    lmax = std::max(lmax, e.lmax);
    t.h_nuclei.push_back(e);
    cost.push_back(w + 1.0);
  }
  if (ao_counter != A)
    return fail(c, QMCKL_FAILURE_DEVICE, fn, "ao_num does not match the number of Cartesian functions of the shells");
  if ((int64_t)t.h_prims.size() > (int64_t)INT32_MAX || A > (int64_t)INT32_MAX)
    return fail(c, QMCKL_FAILURE_DEVICE, fn, "basis too large");
  for (int parts = 1;; parts *= 2) {
    const int p = (int)std::min<int64_t>(parts, N);
    t.level_offsets.push_back((int32_t)t.h_chunks.size());
    const size_t before = t.h_chunks.size();
    split_chunks(t.h_nuclei, cost, p, t.h_chunks);
    t.level_sizes.push_back((int32_t)(t.h_chunks.size() - before));
    if (p >= N) break;
  }
  {
    double total = 0.0;
    for (double c : cost) total += c - 1.0;
    t.piece_offset = (int32_t)t.h_chunks.size();
    split_pieces(t.h_nuclei, t.h_shells, shell_cost, total / (4.0 * (double)N), t.h_chunks);
    t.piece_num = (int32_t)t.h_chunks.size() - t.piece_offset;
  }
  t.h_ao_factor = aof;
  // 2^(j/32) to ~64 bits: hi = nearest double, lo = remainder (long double on the host)
  std::vector<ExpTable> et(1);
  for (int j = 0; j < 32; ++j) {
    const long double v = exp2l((long double)j / 32.0L);
    et[0].hi[j] = (double)v;
    et[0].lo[j] = (double)(v - (long double)et[0].hi[j]);
  }
  for (int j = 0; j < kFine; ++j) {
    const long double v = exp2l((long double)j / (long double)kFine);
    et[0].fine[j].x = (float)v;
    et[0].fine[j].y = (float)(v - (long double)et[0].fine[j].x);
  }
  // the split-BF16 form's folded primitives, evaluated in FP32 pair arithmetic: every exponent
  // within 2^+-60 (so that -expo and expo r2 over the active range are normal floats) and every
  // coefficient zero or of binary exponent within +-64 (so that sign * 2^k * e^y, y in
  // [-27.7, ln 2), and the products of the shared-exponential path stay normal floats)
  bool fold_ok = true;
  t.h_fold.resize(t.h_prims.size());
  for (size_t i = 0; i < t.h_prims.size(); ++i) {
    const PrimEntry& pe = t.h_prims[i];
    if (!(pe.expo >= 0x1p-60) || !(pe.expo <= 0x1p60) || !std::isfinite(pe.coef)) fold_ok = false;
    t.h_fold[i] = fold_entry(pe.expo, pe.coef, pe.coef == 0.0 ? 0 : pe.thr_bits, false);
    if (pe.coef != 0.0 && std::isfinite(pe.coef)) {
      int e2 = 0;
      std::frexp(pe.coef, &e2);
      if (e2 - 1 < -64 || e2 - 1 > 64) fold_ok = false;
    }
  }
  // point-grouping grid over the nuclei plus a 4-bohr margin, 32 cells along the longest side
  {
    double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    for (int64_t n = 0; n < N; ++n)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], ncoord[d * N + n]);
        hi[d] = std::max(hi[d], ncoord[d * N + n]);
      }
    const double margin = 4.0;
    double ext = 0.0;
    for (int d = 0; d < 3; ++d) {
      t.grid_origin[d] = std::isfinite(lo[d]) ? lo[d] - margin : 0.0;
      ext = std::max(ext, std::isfinite(hi[d] - lo[d]) ? hi[d] - lo[d] + 2 * margin : 0.0);
    }
    const double cell = std::max(ext / 32.0, 0.25);
    t.grid_inv_cell = 1.0 / cell;
  }
  t.nucl_num = (int32_t)N;
  t.shell_num = (int32_t)t.h_shells.size();
  t.prim_num = (int32_t)t.h_prims.size();
  t.ao_num = (int32_t)A;
  t.lmax = lmax;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
    t.sm_count = sms;
  cudaGetLastError();
  // distinct exponents per nucleus. Worth sharing when they save most of the exponentials that
  // points actually evaluate: a primitive is active within r2 <= 27.6 / a, a volume ~ a^-1.5,
  // so the measure is sum over distinct exponents of a^-1.5 / sum over primitives of a^-1.5
  // (CHBrClF 0.75: its repeated exponents are mostly steep; generally contracted bases ~0.25);
  // every exponent positive and finite
  {
    bool ok = true;
    int64_t total = 0;
    int32_t cap = 0;
    double w_all = 0.0, w_ent = 0.0;
    for (const PrimEntry& pe : t.h_prims)
      if (!(pe.expo > 0.0) || !std::isfinite(pe.expo)) ok = false;
    std::vector<double> ex;
    for (size_t n = 0; ok && n < t.h_nuclei.size(); ++n) {
      NucleusEntry& e = t.h_nuclei[n];
      const int32_t p0 = e.shell_end > e.shell_begin ? t.h_shells[(size_t)e.shell_begin].prim_begin : 0;
      const int32_t p1 = e.shell_end > e.shell_begin ? t.h_shells[(size_t)e.shell_end - 1].prim_end : 0;
      ex.clear();
      for (int32_t p = p0; p < p1; ++p) ex.push_back(t.h_prims[(size_t)p].expo);
      std::sort(ex.begin(), ex.end());
      ex.erase(std::unique(ex.begin(), ex.end()), ex.end());
      e.ent_begin = (int32_t)t.h_ent.size();
      e.ent_num = (int32_t)ex.size();
      for (int32_t p = p0; p < p1; ++p) w_all += std::pow(t.h_prims[(size_t)p].expo, -1.5);
      for (double a : ex) {
        w_ent += std::pow(a, -1.5);
        t.h_ent.push_back(fold_entry(a, 1.0, prim_threshold(a), true));
      }
      for (int32_t p = p0; p < p1; ++p)
        t.h_prims[(size_t)p].ent =
            (int32_t)(std::lower_bound(ex.begin(), ex.end(), t.h_prims[(size_t)p].expo) - ex.begin());
      total += (int64_t)ex.size();
      cap = std::max(cap, (int32_t)ex.size());
    }
    const int32_t mode = ctx->shared_exp;
    const bool worth = w_all > 0.0 && w_ent <= 0.5 * w_all;
    if (ok && cap > 0 && cap <= 64 && mode != QMCKL_SHARED_EXP_OFF_DEVICE &&
        (worth || mode == QMCKL_SHARED_EXP_ON_DEVICE)) {
      t.ent_cap = cap;
      t.ent_forced = mode == QMCKL_SHARED_EXP_ON_DEVICE;
    } else {
      t.h_ent.clear();
      t.ent_cap = 0;
    }
  }
  t.nuclei = to_device(ctx, t.h_nuclei);
  t.shells = to_device(ctx, t.h_shells);
  t.prims = to_device(ctx, t.h_prims);
  t.ao_factor = to_device(ctx, t.h_ao_factor);
  t.shell_orig = to_device(ctx, t.h_shell_orig);
  t.shell_nucl = to_device(ctx, t.h_shell_nucl);
  t.prim_orig = to_device(ctx, t.h_prim_orig);
  {
    std::vector<char> seen((size_t)K, 0);
    t.prims_unique = true;
    for (int32_t q : t.h_prim_orig) {
      if (seen[(size_t)q]) t.prims_unique = false;
      seen[(size_t)q] = 1;
    }
  }
  t.chunks = to_device(ctx, t.h_chunks);
  t.exp_table = to_device(ctx, et);
  if (t.ent_cap > 0) {
    t.ent = to_device(ctx, t.h_ent);
    if (!t.ent) {
      free_tables(ctx, t);
      return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "kernel tables");
    }
  }
  if (fold_ok && !t.h_fold.empty()) {
    t.fold = to_device(ctx, t.h_fold);
    if (!t.fold) {
      free_tables(ctx, t);
      return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "kernel tables");
    }
  }
  if (!t.nuclei || !t.shells || !t.prims || !t.ao_factor || !t.shell_orig || !t.shell_nucl || !t.chunks ||
      !t.exp_table || (!t.h_prim_orig.empty() && !t.prim_orig)) {
    free_tables(ctx, t);
    return fail(c, QMCKL_ALLOCATION_FAILED_DEVICE, fn, "kernel tables");
  }
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, QMCKL_FAILURE_DEVICE, fn, "table upload failed");
  }
  t.valid = true;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device ensure_tables(Ctx* ctx, qmckl_context_device c) {
  // Slater-type bases are accepted by the setter but not computed (src/qmckl_ao.cpp:103-108)
  if (ctx->ao_basis.type != 'G')
    return fail(c, QMCKL_FAILURE_DEVICE, "compute_ao_basis_shell_vgl", "Not yet implemented for basis type != 'G'");
  if (ctx->ao_basis.tables.valid) return QMCKL_SUCCESS_DEVICE;
  return build_tables(ctx, c);
}

// The processing order of the current points for the fused AO kernels (recomputed when the
// point set changes).
const int32_t* point_order(Ctx* ctx) {
  AoBasisData& ao = ctx->ao_basis;
  const int64_t P = ctx->point.num;
  if (P <= 0 || P > (int64_t)INT32_MAX - 64) return nullptr;
  if (ao.point_perm && ao.perm_date == ctx->point.date) return ao.point_perm;
  void* perm = ao.point_perm;
  void* keys = ao.point_keys;
  void* counts = ao.cell_counts;
  if (!ensure_raw(ctx, &perm, &ao.perm_cap, sizeof(int32_t) * P) ||
      !ensure_raw(ctx, &keys, &ao.keys_cap, sizeof(int32_t) * P) ||
      !ensure_raw(ctx, &counts, &ao.counts_cap, sizeof(int32_t) * kOrderCells)) {
    ao.point_perm = static_cast<int32_t*>(perm);
    ao.point_keys = static_cast<int32_t*>(keys);
    ao.cell_counts = static_cast<int32_t*>(counts);
    return nullptr;  // fall back to the identity order
  }
  ao.point_perm = static_cast<int32_t*>(perm);
  ao.point_keys = static_cast<int32_t*>(keys);
  ao.cell_counts = static_cast<int32_t*>(counts);
  if (launch_point_order(ctx, ao.tables, ctx->point.coord, P, P, ao.point_keys, ao.cell_counts, ao.point_perm) !=
      cudaSuccess)
    return nullptr;
  ao.perm_date = ctx->point.date;
  return ao.point_perm;
}

// Clears the AO and MO caches (after a basis change).
void invalidate_caches(Ctx* ctx) {
  ctx->ao_basis.shell_vgl_date = ctx->ao_basis.ao_vgl_date = ctx->ao_basis.ao_value_date = 0;
  ctx->mo_basis.mo_vgl_date = ctx->mo_basis.mo_value_date = 0;
}

}  // namespace qg

extern "C" qmckl_exit_code_device qmckl_finalize_ao_basis_device(qmckl_context_device context);

namespace {

static qmckl_exit_code_device after_set(qmckl_context_device context, Ctx* ctx, int32_t mask) {
  ctx->ao_basis.uninitialized &= ~mask;
  ctx->ao_basis.provided = ctx->ao_basis.uninitialized == 0;
  if (ctx->ao_basis.provided) return qmckl_finalize_ao_basis_device(context);
  return QMCKL_SUCCESS_DEVICE;
}

// Shared body of the array setters: checks the governing count, copies into a
// context-owned array (from device or host memory) and clears the mask bit.
template <class T>
static qmckl_exit_code_device set_array(qmckl_context_device context, T** field, const T* src, int64_t count,
                                        int64_t size_max, int32_t mask, const char* fn, const char* count_msg,
                                        qmckl_exit_code_device too_small_code) {
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  if (count <= 0) return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, count_msg);
  if (size_max < count) return qmckl_failwith_device(context, too_small_code, fn, "input array too small");
  if (!src) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (!ensure_device(ctx)) return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, fn, "no usable CUDA device");
  if (*field) {
    qmckl_exit_code_device rc = qmckl_free_device(context, *field);
    if (rc != QMCKL_SUCCESS_DEVICE) return qmckl_failwith_device(context, rc, fn, nullptr);
    *field = nullptr;
  }
  T* a = static_cast<T*>(dalloc(ctx, sizeof(T) * (size_t)count));
  if (!a) return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  qmckl_exit_code_device rc = copy(ctx, context, a, src, sizeof(T) * (size_t)count, fn, true);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  *field = a;
  ctx->ao_basis.tables.valid = false;
  return after_set(context, ctx, mask);
}

template <class T>
static qmckl_exit_code_device get_array(qmckl_context_device context, T* dst, const T* src, int64_t count,
                                        int64_t size_max, int32_t mask, const char* fn, const char* small_msg) {
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  if (ctx->ao_basis.uninitialized & mask) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  if (!dst) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (size_max < count) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, small_msg);
  if (!src) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  return copy(ctx, context, dst, src, sizeof(T) * (size_t)count, fn, true);
}

}  // namespace

extern "C" {

// src/qmckl_ao_sycl.cpp:1067-1231, computed on the host with the same operations.
qmckl_exit_code_device qmckl_finalize_ao_basis_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_finalize_ao_basis_device");
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_finalize_ao_basis_device", nullptr);
  int64_t N = 0;
  qmckl_exit_code_device rc = qmckl_get_nucleus_num_device(context, &N);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  AoBasisData& ao = ctx->ao_basis;
  const int64_t S = ao.shell_num, K = ao.prim_num;
  auto nidx = to_host(ctx, context, ao.nucleus_index, N, &rc);
  auto nsh = to_host(ctx, context, ao.nucleus_shell_num, N, &rc);
  auto lam = to_host(ctx, context, ao.shell_ang_mom, S, &rc);
  auto spn = to_host(ctx, context, ao.shell_prim_num, S, &rc);
  auto spi = to_host(ctx, context, ao.shell_prim_index, S, &rc);
  auto expo = to_host(ctx, context, ao.exponent, K, &rc);
  auto coef = to_host(ctx, context, ao.coefficient, K, &rc);
  auto pf = to_host(ctx, context, ao.prim_factor, K, &rc);
  auto sf = to_host(ctx, context, ao.shell_factor, S, &rc);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  const char* fn = "qmckl_finalize_ao_basis_device";
  for (int64_t n = 0; n < N; ++n)
    if (nidx[n] < 0 || nsh[n] < 0 || nidx[n] + nsh[n] > S)
      return fail(context, QMCKL_FAILURE_DEVICE, fn, "nucleus_index/nucleus_shell_num out of range");
  for (int64_t s = 0; s < S; ++s)
    if (spi[s] < 0 || spn[s] < 0 || spi[s] + spn[s] > K)
      return fail(context, QMCKL_FAILURE_DEVICE, fn, "shell_prim_index/shell_prim_num out of range");

  std::vector<int64_t> npi((size_t)N + 1);
  for (int64_t i = 0; i < N; ++i) npi[i] = (nidx[i] < S && S > 0) ? spi[nidx[i]] : 0;  // :1105-1109
  npi[N] = K;
  std::vector<double> cn((size_t)K, 0.0);
  for (int64_t s = 0; s < S; ++s)
    for (int64_t p = spi[s]; p < spi[s] + spn[s]; ++p) {
      volatile double prod = coef[p] * pf[p];  // coefficient * prim_factor * shell_factor, :1142-1144
      cn[p] = prod * sf[s];
    }
  std::vector<int32_t> nmax((size_t)N, 0);
  for (int64_t n = 0; n < N; ++n)
    for (int64_t s = nidx[n]; s < nidx[n] + nsh[n]; ++s) nmax[n] = std::max(nmax[n], lam[s]);  // :1168-1179
  std::vector<double> nrange((size_t)N, 0.0);
  for (int64_t n = 0; n < N; ++n)
    for (int64_t s = nidx[n]; s < nidx[n] + nsh[n]; ++s)
      for (int64_t p = spi[s]; p < spi[s] + spn[s]; ++p) {
        const double range = 1.0 / expo[p];  // :1222-1225
        nrange[n] = nrange[n] > range ? nrange[n] : range;
      }
  dfree(ctx, ao.nucleus_prim_index);
  dfree(ctx, ao.coefficient_normalized);
  dfree(ctx, ao.nucleus_max_ang_mom);
  dfree(ctx, ao.nucleus_range);
  ao.nucleus_prim_index = to_device(ctx, npi);
  ao.coefficient_normalized = to_device(ctx, cn);
  ao.nucleus_max_ang_mom = to_device(ctx, nmax);
  ao.nucleus_range = to_device(ctx, nrange);
  if (!ao.nucleus_prim_index || !ao.coefficient_normalized || !ao.nucleus_max_ang_mom || !ao.nucleus_range)
    return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  // the reference ends its finalize with the per-nucleus tables (src/qmckl_ao_sycl.cpp:1233)
  rc = store_hpc(ctx, context, hpc_tables(N, nidx, nsh, spi, spn, expo, cn), fn);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(context, QMCKL_FAILURE_DEVICE, fn, "upload failed");
  }
  ao.tables.valid = false;
  invalidate_caches(ctx);
  // Build the kernel tables now when the nuclei are placed; otherwise at first use.
  if (ao.type == 'G' && !(ctx->nucleus.uninitialized & (1 << 2))) return build_tables(ctx, context);
  return QMCKL_SUCCESS_DEVICE;
}

// src/qmckl_ao_sycl.cpp:855-1065: recomputes the per-nucleus tables of the finalized basis.
qmckl_exit_code_device qmckl_finalize_ao_basis_hpc_device(qmckl_context_device context) {
  const char* fn = "qmckl_finalize_ao_basis_hpc_device";
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  AoBasisData& ao = ctx->ao_basis;
  if (!ao.provided || !ao.coefficient_normalized) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  const int64_t N = ctx->nucleus.num, S = ao.shell_num, K = ao.prim_num;
  qmckl_exit_code_device rc = QMCKL_SUCCESS_DEVICE;
  auto nidx = to_host(ctx, context, ao.nucleus_index, N, &rc);
  auto nsh = to_host(ctx, context, ao.nucleus_shell_num, N, &rc);
  auto spn = to_host(ctx, context, ao.shell_prim_num, S, &rc);
  auto spi = to_host(ctx, context, ao.shell_prim_index, S, &rc);
  auto expo = to_host(ctx, context, ao.exponent, K, &rc);
  auto cn = to_host(ctx, context, ao.coefficient_normalized, K, &rc);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rc = store_hpc(ctx, context, hpc_tables(N, nidx, nsh, spi, spn, expo, cn), fn);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(context, QMCKL_FAILURE_DEVICE, fn, "upload failed");
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_ao_basis_hpc_dims_device(qmckl_context_device context, int64_t* prim_max,
                                                          int64_t* shell_max) {
  const char* fn = "qmckl_get_ao_basis_hpc_dims_device";
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  if (!ctx->ao_basis.provided || !ctx->ao_basis.prim_num_per_nucleus)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  if (!prim_max) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (!shell_max) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "NULL pointer");
  *prim_max = ctx->ao_basis.hpc_prim_max;
  *shell_max = ctx->ao_basis.hpc_shell_max;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_ao_basis_prim_num_per_nucleus_device(qmckl_context_device context,
                                                                      int32_t* prim_num_per_nucleus, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, prim_num_per_nucleus, ctx->ao_basis.prim_num_per_nucleus, ctx->nucleus.num, size_max,
                   ctx->ao_basis.provided ? 0 : kAoMaskAll, "qmckl_get_ao_basis_prim_num_per_nucleus_device",
                   "Array too small. Expected nucl_num");
}

qmckl_exit_code_device qmckl_get_ao_basis_expo_per_nucleus_device(qmckl_context_device context,
                                                                  double* expo_per_nucleus, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, expo_per_nucleus, ctx->ao_basis.expo_per_nucleus,
                   ctx->nucleus.num * ctx->ao_basis.hpc_prim_max, size_max, ctx->ao_basis.provided ? 0 : kAoMaskAll,
                   "qmckl_get_ao_basis_expo_per_nucleus_device", "Array too small. Expected nucl_num * prim_max");
}

qmckl_exit_code_device qmckl_get_ao_basis_coef_per_nucleus_device(qmckl_context_device context,
                                                                  double* coef_per_nucleus, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, coef_per_nucleus, ctx->ao_basis.coef_per_nucleus,
                   ctx->nucleus.num * ctx->ao_basis.hpc_shell_max * ctx->ao_basis.hpc_prim_max, size_max,
                   ctx->ao_basis.provided ? 0 : kAoMaskAll, "qmckl_get_ao_basis_coef_per_nucleus_device",
                   "Array too small. Expected nucl_num * shell_max * prim_max");
}

qmckl_exit_code_device qmckl_set_ao_shared_exponentials_device(qmckl_context_device context, int32_t mode) {
  const char* fn = "qmckl_set_ao_shared_exponentials_device";
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  if (mode != QMCKL_SHARED_EXP_AUTO_DEVICE && mode != QMCKL_SHARED_EXP_OFF_DEVICE && mode != QMCKL_SHARED_EXP_ON_DEVICE)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "mode must be AUTO (-1), OFF (0) or ON (1)");
  if (ctx->shared_exp != mode) {
    ctx->shared_exp = mode;
    ctx->ao_basis.tables.valid = false;  // rebuilt at the next evaluation
    invalidate_caches(ctx);
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_ao_shared_exponentials_device(qmckl_context_device context, int32_t* active) {
  const char* fn = "qmckl_get_ao_shared_exponentials_device";
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  if (!active) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (!ctx->ao_basis.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  qmckl_exit_code_device rc = ensure_tables(ctx, context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  *active = ao_shared_exponentials(ctx->ao_basis.tables, ctx->precision == QMCKL_PRECISION_SPLIT_BF16_DEVICE) ? 1 : 0;
  return QMCKL_SUCCESS_DEVICE;
}

bool qmckl_ao_basis_provided_device(qmckl_context_device context) {
  Ctx* ctx = checked(context);
  return ctx ? ctx->ao_basis.provided : false;
}

// ---------------------------------------------------------------- setters
qmckl_exit_code_device qmckl_set_ao_basis_type_device(qmckl_context_device context, char basis_type) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (basis_type != 'G' && basis_type != 'S')
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_type_device", nullptr);
  ctx->ao_basis.type = basis_type;
  return after_set(context, ctx, 1);
}

qmckl_exit_code_device qmckl_set_ao_basis_shell_num_device(qmckl_context_device context, int64_t shell_num) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (shell_num <= 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_shell_num_device",
                                 "shell_num <= 0");
  const int64_t prim_num = ctx->ao_basis.prim_num;
  if (0 < prim_num && prim_num < shell_num)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_shell_num_device",
                                 "shell_num > prim_num");
  ctx->ao_basis.shell_num = shell_num;
  return after_set(context, ctx, 1 << 1);
}

qmckl_exit_code_device qmckl_set_ao_basis_prim_num_device(qmckl_context_device context, int64_t prim_num) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (prim_num <= 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_prim_num_device",
                                 "prim_num must be positive");
  const int64_t shell_num = ctx->ao_basis.shell_num;
  if (shell_num <= 0)
    return qmckl_failwith_device(context, QMCKL_FAILURE_DEVICE, "qmckl_set_ao_basis_prim_num_device",
                                 "shell_num is not set");
  if (prim_num < shell_num)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_prim_num_device",
                                 "prim_num < shell_num");
  ctx->ao_basis.prim_num = prim_num;
  return after_set(context, ctx, 1 << 2);
}

qmckl_exit_code_device qmckl_set_ao_basis_ao_num_device(qmckl_context_device context, int64_t ao_num) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (ao_num <= 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_shell_num_device",
                                 "ao_num must be positive");
  const int64_t shell_num = ctx->ao_basis.shell_num;
  if (shell_num <= 0)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_shell_num_device",
                                 "shell_num is not set");
  if (ao_num < shell_num)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_set_ao_basis_shell_num_device",
                                 "ao_num < shell_num");
  ctx->ao_basis.ao_num = ao_num;
  return after_set(context, ctx, 1 << 12);
}

qmckl_exit_code_device qmckl_set_ao_basis_nucleus_index_device(qmckl_context_device context, int64_t* nucleus_index,
                                                               int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  // the reference reports a short array as QMCKL_FAILURE_DEVICE here (src/qmckl_ao.cpp:598-603)
  return set_array(context, &ctx->ao_basis.nucleus_index, nucleus_index, ctx->nucleus.num, size_max, 1 << 4,
                   "qmckl_set_ao_basis_nucleus_index_device", "nucl_num is not set", QMCKL_FAILURE_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_nucleus_shell_num_device(qmckl_context_device context,
                                                                   int64_t* nucleus_shell_num, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.nucleus_shell_num, nucleus_shell_num, ctx->nucleus.num, size_max, 1 << 3,
                   "qmckl_set_ao_basis_nucleus_shell_num_device", "shell_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_shell_ang_mom_device(qmckl_context_device context, int32_t* shell_ang_mom,
                                                               int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.shell_ang_mom, shell_ang_mom, ctx->ao_basis.shell_num, size_max, 1 << 5,
                   "qmckl_set_ao_basis_shell_ang_mom_device", "shell_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_shell_prim_num_device(qmckl_context_device context,
                                                                int64_t* shell_prim_num, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.shell_prim_num, shell_prim_num, ctx->ao_basis.shell_num, size_max, 1 << 6,
                   "qmckl_set_ao_basis_shell_prim_num_device", "shell_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_shell_prim_index_device(qmckl_context_device context,
                                                                  int64_t* shell_prim_index, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.shell_prim_index, shell_prim_index, ctx->ao_basis.shell_num, size_max,
                   1 << 7, "qmckl_set_ao_basis_shell_prim_index_device", "shell_num is not set",
                   QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_shell_factor_device(qmckl_context_device context, double* shell_factor,
                                                              int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.shell_factor, shell_factor, ctx->ao_basis.shell_num, size_max, 1 << 8,
                   "qmckl_set_ao_basis_shell_factor_device", "shell_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_exponent_device(qmckl_context_device context, double* exponent,
                                                          int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.exponent, exponent, ctx->ao_basis.prim_num, size_max, 1 << 9,
                   "qmckl_set_ao_basis_exponent_device", "prim_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_coefficient_device(qmckl_context_device context, double* coefficient,
                                                             int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.coefficient, coefficient, ctx->ao_basis.prim_num, size_max, 1 << 10,
                   "qmckl_set_ao_basis_coefficient_device", "prim_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_prim_factor_device(qmckl_context_device context, double* prim_factor,
                                                             int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.prim_factor, prim_factor, ctx->ao_basis.prim_num, size_max, 1 << 11,
                   "qmckl_set_ao_basis_prim_factor_device", "prim_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}
qmckl_exit_code_device qmckl_set_ao_basis_ao_factor_device(qmckl_context_device context, double* ao_factor,
                                                           int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return set_array(context, &ctx->ao_basis.ao_factor, ao_factor, ctx->ao_basis.ao_num, size_max, 1 << 13,
                   "qmckl_set_ao_basis_ao_factor_device", "ao_num is not set", QMCKL_INVALID_ARG_3_DEVICE);
}

// ---------------------------------------------------------------- getters
static qmckl_exit_code_device scalar_check(qmckl_context_device context, int32_t mask, const char* fn) {
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  if (ctx->ao_basis.uninitialized & mask) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_ao_basis_type_device(qmckl_context_device context, char* const basis_type) {
  qmckl_exit_code_device rc = scalar_check(context, 1, "qmckl_get_ao_basis_type");
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!basis_type) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_ao_basis_type", "NULL pointer");
  basis_type[0] = ctx_of(context)->ao_basis.type;
  return QMCKL_SUCCESS_DEVICE;
}
qmckl_exit_code_device qmckl_get_ao_basis_shell_num_device(qmckl_context_device context, int64_t* const shell_num) {
  qmckl_exit_code_device rc = scalar_check(context, 1 << 1, "qmckl_get_ao_basis_shell_num");
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!shell_num) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_ao_basis_shell_num", "NULL pointer");
  *shell_num = ctx_of(context)->ao_basis.shell_num;
  return QMCKL_SUCCESS_DEVICE;
}
qmckl_exit_code_device qmckl_get_ao_basis_prim_num_device(qmckl_context_device context, int64_t* prim_num) {
  qmckl_exit_code_device rc = scalar_check(context, 1 << 2, "qmckl_get_ao_basis_prim_num");
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!prim_num) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_ao_basis_prim_num", "NULL pointer");
  *prim_num = ctx_of(context)->ao_basis.prim_num;
  return QMCKL_SUCCESS_DEVICE;
}
qmckl_exit_code_device qmckl_get_ao_basis_ao_num_device(qmckl_context_device context, int64_t* ao_num) {
  qmckl_exit_code_device rc = scalar_check(context, 1 << 12, "qmckl_get_ao_basis_ao_num");
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!ao_num) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_ao_basis_ao_num", "NULL pointer");
  *ao_num = ctx_of(context)->ao_basis.ao_num;
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_get_ao_basis_nucleus_shell_num_device(qmckl_context_device context,
                                                                   int64_t* nucleus_shell_num, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, nucleus_shell_num, ctx->ao_basis.nucleus_shell_num, ctx->nucleus.num, size_max, 1 << 3,
                   "qmckl_get_ao_basis_nucleus_shell_num_device", "Array too small. Expected nucl_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_nucleus_index_device(qmckl_context_device context, int64_t* nucleus_index,
                                                               int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, nucleus_index, ctx->ao_basis.nucleus_index, ctx->nucleus.num, size_max, 1 << 4,
                   "qmckl_get_ao_basis_nucleus_index_device", "Array too small. Expected shell_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_shell_ang_mom_device(qmckl_context_device context, int32_t* shell_ang_mom,
                                                               int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, shell_ang_mom, ctx->ao_basis.shell_ang_mom, ctx->ao_basis.shell_num, size_max, 1 << 5,
                   "qmckl_get_ao_basis_shell_ang_mom_device", "Array too small. Expected shell_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_shell_factor_device(qmckl_context_device context, double* shell_factor,
                                                              int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, shell_factor, ctx->ao_basis.shell_factor, ctx->ao_basis.shell_num, size_max, 1 << 8,
                   "qmckl_get_ao_basis_shell_factor_device", "Array too small. Expected shell_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_shell_prim_num_device(qmckl_context_device context,
                                                                int64_t* shell_prim_num, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, shell_prim_num, ctx->ao_basis.shell_prim_num, ctx->ao_basis.shell_num, size_max, 1 << 6,
                   "qmckl_get_ao_basis_shell_prim_num_device", "Array too small. Expected shell_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_shell_prim_index_device(qmckl_context_device context,
                                                                  int64_t* shell_prim_index, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, shell_prim_index, ctx->ao_basis.shell_prim_index, ctx->ao_basis.shell_num, size_max,
                   1 << 7, "qmckl_get_ao_basis_shell_prim_index_device", "Array too small. Expected shell_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_exponent_device(qmckl_context_device context, double* exponent,
                                                          int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, exponent, ctx->ao_basis.exponent, ctx->ao_basis.prim_num, size_max, 1 << 9,
                   "qmckl_get_ao_basis_exponent_device", "Array too small. Expected prim_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_coefficient_device(qmckl_context_device context, double* coefficient,
                                                             int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, coefficient, ctx->ao_basis.coefficient, ctx->ao_basis.prim_num, size_max, 1 << 10,
                   "qmckl_get_ao_basis_coefficient_device", "Array too small. Expected prim_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_prim_factor_device(qmckl_context_device context, double* prim_factor,
                                                             int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, prim_factor, ctx->ao_basis.prim_factor, ctx->ao_basis.prim_num, size_max, 1 << 11,
                   "qmckl_get_ao_basis_prim_factor_device", "Array too small. Expected prim_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_ao_factor_device(qmckl_context_device context, double* ao_factor,
                                                           int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  return get_array(context, ao_factor, ctx->ao_basis.ao_factor, ctx->ao_basis.ao_num, size_max, 1 << 13,
                   "qmckl_get_ao_basis_ao_factor_device", "Array too small. Expected ao_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_nucleus_range_device(qmckl_context_device context, double* nucleus_range,
                                                               int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!ctx->ao_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_get_ao_basis_nucleus_range_device", nullptr);
  return get_array(context, nucleus_range, ctx->ao_basis.nucleus_range, ctx->nucleus.num, size_max, 0,
                   "qmckl_get_ao_basis_nucleus_range_device", "Array too small. Expected nucl_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_nucleus_max_ang_mom_device(qmckl_context_device context,
                                                                     int32_t* nucleus_max_ang_mom, int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!ctx->ao_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_get_ao_basis_nucleus_max_ang_mom_device",
                                 nullptr);
  return get_array(context, nucleus_max_ang_mom, ctx->ao_basis.nucleus_max_ang_mom, ctx->nucleus.num, size_max, 0,
                   "qmckl_get_ao_basis_nucleus_max_ang_mom_device", "Array too small. Expected nucl_num");
}
qmckl_exit_code_device qmckl_get_ao_basis_coefficient_normalized_device(qmckl_context_device context,
                                                                        double* coefficient_normalized,
                                                                        int64_t size_max) {
  Ctx* ctx = checked(context);
  if (!ctx) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!ctx->ao_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE,
                                 "qmckl_get_ao_basis_coefficient_normalized_device", nullptr);
  return get_array(context, coefficient_normalized, ctx->ao_basis.coefficient_normalized, ctx->ao_basis.prim_num,
                   size_max, 0, "qmckl_get_ao_basis_coefficient_normalized_device",
                   "Array too small. Expected prim_num");
}

// ---------------------------------------------------------------- provides
qmckl_exit_code_device qmckl_provide_ao_basis_shell_vgl_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_provide_ao_basis_shell_vgl_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_provide_ao_basis_shell_vgl_device";
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  AoBasisData& ao = ctx->ao_basis;
  if (!ao.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  if (ctx->point.date > ao.shell_vgl_date) {
    qmckl_exit_code_device rc = ensure_tables(ctx, context);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    if (!ensure(ctx, &ao.shell_vgl, &ao.shell_vgl_cap, sizeof(double) * 5 * ao.shell_num * ctx->point.num))
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
    launch_shell_vgl(ctx, ao.tables, ctx->point.coord, ctx->point.num, ao.shell_num, ao.shell_vgl);
    rc = finish(ctx, context, fn);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    ao.shell_vgl_date = ctx->date;
  }
  return QMCKL_SUCCESS_DEVICE;
}

// Computes AO vgl for the current points into `dst` (no cache bookkeeping).
static qmckl_exit_code_device compute_ao_vgl(Ctx* ctx, qmckl_context_device context, double* dst, const char* fn) {
  qmckl_exit_code_device rc = ensure_tables(ctx, context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  launch_ao_vgl(ctx, ctx->ao_basis.tables, ctx->point.coord, point_order(ctx), ctx->point.num, dst);
  return finish(ctx, context, fn);
}

static qmckl_exit_code_device compute_ao_value(Ctx* ctx, qmckl_context_device context, double* dst, const char* fn) {
  AoBasisData& ao = ctx->ao_basis;
  if (ctx->point.date <= ao.ao_vgl_date && ao.ao_vgl) {
    // src/qmckl_ao_sycl.cpp:790-808: ao_vgl is fresh, copy its value rows
    launch_strided_copy(ctx, ao.ao_vgl, 5 * ao.ao_num, dst, ao.ao_num, ctx->point.num, ao.ao_num);
    return finish(ctx, context, fn);
  }
  qmckl_exit_code_device rc = ensure_tables(ctx, context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  launch_ao_value(ctx, ao.tables, ctx->point.coord, point_order(ctx), ctx->point.num, dst);
  return finish(ctx, context, fn);
}

qmckl_exit_code_device qmckl_provide_ao_basis_ao_vgl_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_provide_ao_basis_ao_vgl_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_provide_ao_basis_ao_vgl_device";
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  AoBasisData& ao = ctx->ao_basis;
  if (!ao.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_ao_basis_ao_vgl_device", nullptr);
  if (ctx->point.date > ao.ao_vgl_date) {
    if (!ensure(ctx, &ao.ao_vgl, &ao.ao_vgl_cap, sizeof(double) * 5 * ao.ao_num * ctx->point.num))
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_ao_basis_ao_vgl", nullptr);
    qmckl_exit_code_device rc = compute_ao_vgl(ctx, context, ao.ao_vgl, fn);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    ao.ao_vgl_date = ctx->date;
  }
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device qmckl_provide_ao_basis_ao_value_device(qmckl_context_device context) {
  QG_NVTX_RANGE("qmckl_provide_ao_basis_ao_value_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_provide_ao_basis_ao_value";
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  AoBasisData& ao = ctx->ao_basis;
  if (!ao.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  if (ctx->point.date > ao.ao_value_date) {
    if (!ensure(ctx, &ao.ao_value, &ao.ao_value_cap, sizeof(double) * ao.ao_num * ctx->point.num))
      return qmckl_failwith_device(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
    qmckl_exit_code_device rc = compute_ao_value(ctx, context, ao.ao_value, fn);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
    ao.ao_value_date = ctx->date;
  }
  return QMCKL_SUCCESS_DEVICE;
}

// ---------------------------------------------------------------- results
qmckl_exit_code_device qmckl_get_ao_basis_shell_vgl_device(qmckl_context_device context, double* const shell_vgl,
                                                           const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_ao_basis_shell_vgl_device");
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_get_ao_basis_shell_vgl_device", nullptr);
  qmckl_exit_code_device rc = qmckl_provide_ao_basis_shell_vgl_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  const int64_t sze = ctx->ao_basis.shell_num * 5 * ctx->point.num;
  if (size_max < sze)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_ao_basis_shell_vgl",
                                 "input array too small");
  if (!shell_vgl) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_ao_basis_shell_vgl", "NULL pointer");
  return copy(ctx, context, shell_vgl, ctx->ao_basis.shell_vgl, sizeof(double) * (size_t)sze,
              "qmckl_get_ao_basis_shell_vgl", true);
}

qmckl_exit_code_device qmckl_get_ao_basis_ao_vgl_device(qmckl_context_device context, double* const ao_vgl,
                                                        const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_ao_basis_ao_vgl_device");
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_get_ao_basis_ao_vgl_device", nullptr);
  qmckl_exit_code_device rc = qmckl_provide_ao_basis_ao_vgl_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  const int64_t sze = ctx->ao_basis.ao_num * 5 * ctx->point.num;
  if (size_max < sze)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_ao_basis_ao_vgl_device",
                                 "input array too small");
  if (!ao_vgl) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_ao_basis_ao_vgl_device", "NULL pointer");
  return copy(ctx, context, ao_vgl, ctx->ao_basis.ao_vgl, sizeof(double) * (size_t)sze,
              "qmckl_get_ao_basis_ao_vgl_device", true);
}

// The reference swaps the user's buffer into the context, provides, and swaps back
// (src/qmckl_ao.cpp:277-318), which leaves the internal cache dated fresh but stale;
// here the result goes straight to the user's buffer and the cache date is untouched.
qmckl_exit_code_device qmckl_get_ao_basis_ao_vgl_inplace_device(qmckl_context_device context, double* const ao_vgl,
                                                                const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_ao_basis_ao_vgl_inplace_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_get_ao_basis_ao_vgl_inplace_device";
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  const int64_t sze = ctx->ao_basis.ao_num * 5 * ctx->point.num;
  if (size_max < sze) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "input array too small");
  qmckl_exit_code_device rc = qmckl_context_touch_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!ctx->ao_basis.provided)
    return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, "qmckl_ao_basis_ao_vgl_device", nullptr);
  if (!ao_vgl) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (gpu_accessible(ao_vgl)) return compute_ao_vgl(ctx, context, ao_vgl, fn);
  rc = qmckl_provide_ao_basis_ao_vgl_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  return copy(ctx, context, ao_vgl, ctx->ao_basis.ao_vgl, sizeof(double) * (size_t)sze, fn, true);
}

qmckl_exit_code_device qmckl_get_ao_basis_ao_value_device(qmckl_context_device context, double* const ao_value,
                                                          const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_ao_basis_ao_value_device");
  Ctx* ctx = checked(context);
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, "qmckl_get_ao_basis_ao_value_device", nullptr);
  qmckl_exit_code_device rc = qmckl_provide_ao_basis_ao_value_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  const int64_t sze = ctx->ao_basis.ao_num * ctx->point.num;
  if (size_max < sze)
    return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, "qmckl_get_ao_basis_ao_value_device",
                                 "input array too small");
  if (!ao_value) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, "qmckl_get_ao_basis_ao_value_device", "NULL pointer");
  return copy(ctx, context, ao_value, ctx->ao_basis.ao_value, sizeof(double) * (size_t)sze,
              "qmckl_get_ao_basis_ao_value_device", true);
}

qmckl_exit_code_device qmckl_get_ao_basis_ao_value_inplace_device(qmckl_context_device context,
                                                                  double* const ao_value, const int64_t size_max) {
  QG_NVTX_RANGE("qmckl_get_ao_basis_ao_value_inplace_device");
  Ctx* ctx = checked(context);
  const char* fn = "qmckl_get_ao_basis_ao_value_inplace_device";
  if (!ctx) return qmckl_failwith_device(context, QMCKL_INVALID_CONTEXT_DEVICE, fn, nullptr);
  const int64_t sze = ctx->ao_basis.ao_num * ctx->point.num;
  if (size_max < sze) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "input array too small");
  qmckl_exit_code_device rc = qmckl_context_touch_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  if (!ctx->ao_basis.provided) return qmckl_failwith_device(context, QMCKL_NOT_PROVIDED_DEVICE, fn, nullptr);
  if (!ao_value) return qmckl_failwith_device(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL pointer");
  if (gpu_accessible(ao_value)) return compute_ao_value(ctx, context, ao_value, fn);
  rc = qmckl_provide_ao_basis_ao_value_device(context);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  return copy(ctx, context, ao_value, ctx->ao_basis.ao_value, sizeof(double) * (size_t)sze, fn, true);
}

}  // extern "C"
