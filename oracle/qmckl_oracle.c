/*
 * CPU oracle for the QMCkl basis-evaluation path (AO vgl, AO value, MO vgl, MO value).
 *
 * TEST INFRASTRUCTURE ONLY. This file restates, in plain C and on the host, the
 * arithmetic of the reference library (qmckl_sycl) so that the CUDA product can be
 * checked against it. Only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * --impl reference legs of bench.py load it, and only as the checker or the timed CPU
 * baseline; the product never calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks this oracle against the
 * reference's own golden file (tests/mo_reference.txt, all 152,320 MO vgl values at
 * 1e-14 absolute, as tests/test_qmckl_mo.cpp:382-405 does) and known answers
 * (tests/test_qmckl_ao.cpp:440-448, tests/test_qmckl_mo.cpp:250-259), and, where the
 * reference sources are available, bit for bit against the unmodified reference built
 * on the host (oracle/Makefile.ref).
 *
 * Every value is computed with the same operations in the same order as the reference
 * kernels, and this file must be compiled without floating-point contraction
 * (-ffp-contract=off) so that no multiply-add is fused. Loops are reordered only where
 * each output slot is still produced by the same sequence of operations (the point
 * loop is outermost so that points can be spread over host threads).
 *
 * Layouts (C index order, as the reference indexes them):
 *   coord      [3][point_num]      (ctx->point.coord, qmckl_point.cpp:124-129)
 *   nucl_coord [3][nucl_num]
 *   shell_vgl  [point_num][5][shell_num]
 *   ao_vgl     [point_num][5][ao_num],  ao_value [point_num][ao_num]
 *   coef_t     [ao_num][mo_num]    (transpose of the user's [mo_num][ao_num])
 *   mo_vgl     [point_num][5][mo_num],  mo_value [point_num][mo_num]
 * Output slots that the reference never writes (screened nuclei) are left untouched;
 * callers pass zeroed arrays, which is what a fresh reference allocation holds.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* -ln(1e-12), hard-coded by the reference at src/qmckl_ao_sycl.cpp:22,117,449. */
static const double ORACLE_CUTOFF = 27.631021115928547;

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/*
 * Derived AO tables, src/qmckl_ao_sycl.cpp:1067-1231 (qmckl_finalize_ao_basis_device):
 *   nucleus_prim_index[n] = shell_prim_index[nucleus_index[n]], [nucl_num] = prim_num (:1105-1109)
 *   coefficient_normalized[p] = coefficient[p] * prim_factor[p] * shell_factor[s]  (:1142-1144)
 *   nucleus_max_ang_mom[n] = max over the nucleus' shells of shell_ang_mom        (:1168-1179)
 *   nucleus_range[n] = max over the nucleus' primitives of 1/exponent             (:1211-1227)
 */
void oracle_finalize_ao(int64_t nucl_num, int64_t shell_num, int64_t prim_num, const int64_t* nucleus_index,
                        const int64_t* nucleus_shell_num, const int32_t* shell_ang_mom,
                        const int64_t* shell_prim_index, const int64_t* shell_prim_num, const double* exponent,
                        const double* coefficient, const double* prim_factor, const double* shell_factor,
                        int64_t* nucleus_prim_index, double* coefficient_normalized, int32_t* nucleus_max_ang_mom,
                        double* nucleus_range) {
  for (int64_t i = 0; i < nucl_num; ++i) nucleus_prim_index[i] = shell_prim_index[nucleus_index[i]];
  nucleus_prim_index[nucl_num] = prim_num;
  for (int64_t s = 0; s < shell_num; ++s)
    for (int64_t p = shell_prim_index[s]; p < shell_prim_index[s] + shell_prim_num[s]; ++p)
      coefficient_normalized[p] = coefficient[p] * prim_factor[p] * shell_factor[s];
  for (int64_t n = 0; n < nucl_num; ++n) {
    int32_t m = 0;
    for (int64_t s = nucleus_index[n]; s < nucleus_index[n] + nucleus_shell_num[n]; ++s)
      m = m > shell_ang_mom[s] ? m : shell_ang_mom[s];
    nucleus_max_ang_mom[n] = m;
  }
  for (int64_t n = 0; n < nucl_num; ++n) {
    double r = 0.;
    for (int64_t s = nucleus_index[n]; s < nucleus_index[n] + nucleus_shell_num[n]; ++s)
      for (int64_t p = shell_prim_index[s]; p < shell_prim_index[s] + shell_prim_num[s]; ++p) {
        double range = 1. / exponent[p];
        r = r > range ? r : range;
      }
    nucleus_range[n] = r;
  }
}

/*
 * Per-nucleus exponent tables, src/qmckl_ao_sycl.cpp:855-1065 (qmckl_finalize_ao_basis_hpc_device,
 * run by the reference at the end of qmckl_finalize_ao_basis_device, :1233):
 *   hpc_dims(): shell_max = max nucleus_shell_num, prim_max = max over nuclei of the
 *     nucleus' primitive count (:873-900);
 *   for each nucleus: its primitives' exponents in shell order, sorted ascending by a
 *     bubble sort that swaps only on a strict '<' (stable, :941-962); coef[j][i] = the
 *     coefficient_normalized of sorted primitive i when it belongs to the nucleus' shell j,
 *     else 0 (:964-984); consecutive equal exponents merge into one entry whose coefficient
 *     per shell is the sum over the merged ones in sorted order (:988-1009, the entry keeps
 *     the last merged exponent value, :1011-1013); prim_num_per_nucleus = number of entries
 *     (1 for a nucleus without primitives, :989-1015).
 * Outputs: prim_num_per_nucleus [nucl_num], expo_per_nucleus [nucl_num][prim_max],
 * coef_per_nucleus [nucl_num][shell_max][prim_max] (zero where not written).
 */
void oracle_hpc_dims(int64_t nucl_num, const int64_t* nucleus_index, const int64_t* nucleus_shell_num,
                     const int64_t* shell_prim_num, int64_t* prim_max, int64_t* shell_max) {
  int64_t pm = 0, sm = 0;
  for (int64_t n = 0; n < nucl_num; ++n) {
    int64_t k = 0;
    for (int64_t s = nucleus_index[n]; s < nucleus_index[n] + nucleus_shell_num[n]; ++s) k += shell_prim_num[s];
    if (nucleus_shell_num[n] > sm) sm = nucleus_shell_num[n];
    if (k > pm) pm = k;
  }
  *prim_max = pm;
  *shell_max = sm;
}

void oracle_finalize_hpc(int64_t nucl_num, const int64_t* nucleus_index, const int64_t* nucleus_shell_num,
                         const int64_t* shell_prim_index, const int64_t* shell_prim_num, const double* exponent,
                         const double* coefficient_normalized, int64_t prim_max, int64_t shell_max,
                         int32_t* prim_num_per_nucleus, double* expo_per_nucleus, double* coef_per_nucleus) {
  for (int64_t i = 0; i < nucl_num * prim_max; ++i) expo_per_nucleus[i] = 0.0;
  for (int64_t i = 0; i < nucl_num * shell_max * prim_max; ++i) coef_per_nucleus[i] = 0.0;
  if (prim_max == 0) {
    for (int64_t n = 0; n < nucl_num; ++n) prim_num_per_nucleus[n] = 0;
    return;
  }
  double* ex = (double*)calloc((size_t)prim_max, sizeof(double));
  int64_t* pos = (int64_t*)calloc((size_t)prim_max, sizeof(int64_t));  /* nucleus-local index of sorted entry */
  int64_t* grp = (int64_t*)calloc((size_t)prim_max, sizeof(int64_t));  /* merged entry of sorted entry */
  double* cs = (double*)calloc((size_t)(shell_max * prim_max), sizeof(double));
  double* acc = (double*)calloc((size_t)prim_max, sizeof(double));
  for (int64_t n = 0; n < nucl_num; ++n) {
    const int64_t s0 = nucleus_index[n], ns = nucleus_shell_num[n];
    int64_t k = 0;
    for (int64_t s = s0; s < s0 + ns; ++s)
      for (int64_t p = shell_prim_index[s]; p < shell_prim_index[s] + shell_prim_num[s]; ++p) {
        ex[k] = exponent[p];
        pos[k] = k;
        ++k;
      }
    for (int64_t pass = 0; pass + 1 < k; ++pass)
      for (int64_t j = 0; j + 1 < k - pass; ++j)
        if (ex[j + 1] < ex[j]) {
          const double te = ex[j];
          ex[j] = ex[j + 1];
          ex[j + 1] = te;
          const int64_t tp = pos[j];
          pos[j] = pos[j + 1];
          pos[j + 1] = tp;
        }
    /* coefficient of sorted entry i for shell j: nonzero only if the entry is one of j's */
    for (int64_t j = 0; j < ns; ++j) {
      int64_t first = 0;
      for (int64_t s = s0; s < s0 + j; ++s) first += shell_prim_num[s];
      const int64_t last = first + shell_prim_num[s0 + j];
      for (int64_t i = 0; i < k; ++i)
        cs[j * prim_max + i] =
            (pos[i] >= first && pos[i] < last) ? coefficient_normalized[shell_prim_index[s0 + j] + (pos[i] - first)]
                                               : 0.0;
    }
    int64_t g = 0;
    if (k > 0) grp[0] = 0;
    for (int64_t i = 1; i < k; ++i) {
      if (ex[i] != ex[i - 1]) ++g;
      grp[i] = g;
    }
    for (int64_t j = 0; j < ns; ++j) {
      for (int64_t i = 0; i < k; ++i) acc[i] = 0.0;
      for (int64_t i = 0; i < k; ++i) acc[grp[i]] += cs[j * prim_max + i];
      for (int64_t i = 0; i < k; ++i) cs[j * prim_max + i] = acc[i];
    }
    for (int64_t i = 0; i < k; ++i) ex[grp[i]] = ex[i];
    const int64_t u = g + 1;
    prim_num_per_nucleus[n] = (int32_t)u;
    for (int64_t i = 0; i < u; ++i) expo_per_nucleus[n * prim_max + i] = k > 0 ? ex[i] : 0.0;
    for (int64_t j = 0; j < ns; ++j)
      for (int64_t i = 0; i < u; ++i)
        coef_per_nucleus[(n * shell_max + j) * prim_max + i] = k > 0 ? cs[j * prim_max + i] : 0.0;
  }
  free(ex);
  free(pos);
  free(grp);
  free(cs);
  free(acc);
}

/* shell -> nucleus map, src/qmckl_ao_sycl.cpp:30-37 */
static void shell_to_nucleus(int64_t nucl_num, const int64_t* nucleus_index, const int64_t* nucleus_shell_num,
                             int64_t shell_num, int32_t* s2n) {
  for (int64_t s = 0; s < shell_num; ++s) s2n[s] = 0;
  for (int64_t n = 0; n < nucl_num; ++n)
    for (int64_t s = nucleus_index[n]; s <= nucleus_index[n] + nucleus_shell_num[n] - 1; ++s) s2n[s] = (int32_t)n;
}

/*
 * Shell radial vgl for one point, src/qmckl_ao_sycl.cpp:40-95: displacement (:47-51),
 * nucleus screen (:53-55, slot not written), primitive screen (:72-75), accumulation
 * (:77-84), store (:87-95).
 */
static void shell_vgl_point(int64_t ip, int64_t point_num, int64_t nucl_num, int64_t shell_num, const int32_t* s2n,
                            const double* nucleus_range, const int64_t* shell_prim_index,
                            const int64_t* shell_prim_num, const double* coord, const double* nucl_coord,
                            const double* expo, const double* coef_normalized, double* shell_vgl) {
  for (int64_t is = 0; is < shell_num; ++is) {
    const int64_t in = s2n[is];
    const double x = coord[ip] - nucl_coord[in];
    const double y = coord[ip + point_num] - nucl_coord[in + nucl_num];
    const double z = coord[ip + 2 * point_num] - nucl_coord[in + 2 * nucl_num];
    const double r2 = x * x + y * y + z * z;
    if (r2 > ORACLE_CUTOFF * nucleus_range[in]) continue;
    double t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0;
    for (int64_t p = shell_prim_index[is]; p <= shell_prim_index[is] + shell_prim_num[is] - 1; ++p) {
      const double ar2 = expo[p] * r2;
      if (ar2 > ORACLE_CUTOFF) continue;
      const double v = coef_normalized[p] * exp(-ar2);
      const double two_a = -2 * expo[p] * v;
      t0 += v;
      t1 += two_a * x;
      t2 += two_a * y;
      t3 += two_a * z;
      t4 += two_a * (3 - 2 * ar2);
    }
    double* out = shell_vgl + ip * shell_num * 5;
    out[is + 0 * shell_num] = t0;
    out[is + 1 * shell_num] = t1;
    out[is + 2 * shell_num] = t2;
    out[is + 3 * shell_num] = t3;
    out[is + 4 * shell_num] = t4;
  }
}

void oracle_shell_vgl(int64_t point_num, int64_t nucl_num, int64_t shell_num, const int64_t* nucleus_index,
                      const int64_t* nucleus_shell_num, const double* nucleus_range, const int64_t* shell_prim_index,
                      const int64_t* shell_prim_num, const double* coord, const double* nucl_coord,
                      const double* expo, const double* coef_normalized, double* shell_vgl) {
  int32_t* s2n = (int32_t*)malloc(sizeof(int32_t) * (size_t)(shell_num > 0 ? shell_num : 1));
  shell_to_nucleus(nucl_num, nucleus_index, nucleus_shell_num, shell_num, s2n);
#pragma omp parallel for schedule(dynamic, 8)
  for (int64_t ip = 0; ip < point_num; ++ip)
    shell_vgl_point(ip, point_num, nucl_num, shell_num, s2n, nucleus_range, shell_prim_index, shell_prim_num, coord,
                    nucl_coord, expo, coef_normalized, shell_vgl);
  free(s2n);
}

/*
 * Cartesian polynomial vgl of one (point, nucleus), src/qmckl_ao_sycl.cpp:221-331.
 * pows[i + (llmax+3)*j] holds x_j^(i-2) for i >= 2 and 1 for i < 2 (:246-264);
 * poly[5*n + c] is component c of monomial n, monomials ordered by degree, then a
 * descending, then b descending (:293-305).
 */
static void poly_vgl_point(double x, double y, double z, int llmax, double* pows, double* poly) {
  if (llmax == 0) {
    poly[0] = 1.;
    poly[1] = 0.;
    poly[2] = 0.;
    poly[3] = 0.;
    poly[4] = 0.;
    return;
  }
  const int L = llmax + 3;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) pows[i + L * j] = 1.;
  for (int i = 3; i < llmax + 3; ++i) {
    pows[i] = pows[i - 1] * x;
    pows[i + L] = pows[i - 1 + L] * y;
    pows[i + 2 * L] = pows[i - 1 + 2 * L] * z;
  }
  for (int i = 0; i < 20; ++i) poly[i] = 0.;
  poly[0] = 1.;
  poly[5] = pows[3];
  poly[6] = 1.;
  poly[10] = pows[3 + L];
  poly[12] = 1.;
  poly[15] = pows[3 + 2 * L];
  poly[18] = 1.;
  int n = 3;
  double dd = 2.;
  for (int d = 2; d <= llmax; d++) {
    double da = dd;
    for (int a = d; a >= 0; a--) {
      double db = dd - da;
      for (int b = d - a; b >= 0; b--) {
        const int c = d - a - b;
        const double dc = dd - da - db;
        n = n + 1;
        double xy = pows[a + 2] * pows[(b + 2) + L];
        double yz = pows[(b + 2) + L] * pows[(c + 2) + 2 * L];
        double xz = pows[a + 2] * pows[(c + 2) + 2 * L];
        poly[5 * n] = xy * pows[c + 2 + 2 * L];
        xy = dc * xy;
        xz = db * xz;
        yz = da * yz;
        poly[1 + 5 * n] = pows[a + 1] * yz;
        poly[2 + 5 * n] = pows[b + 1 + L] * xz;
        poly[3 + 5 * n] = pows[c + 1 + 2 * L] * xy;
        poly[4 + 5 * n] = (da - 1.) * pows[a] * yz + (db - 1.) * pows[b + L] * xz + (dc - 1.) * pows[c + 2 * L] * xy;
        db -= 1.;
      }
      da -= 1.;
    }
    dd += 1.;
  }
}

static int64_t lstart(int l) { return (int64_t)l * (l + 1) * (l + 2) / 6 + 1; } /* :159-163 */

/* first AO (0-based) of each shell, walking nuclei in order, src/qmckl_ao_sycl.cpp:166-188 */
static void shell_ao_index(int64_t nucl_num, const int64_t* nucleus_index, const int64_t* nucleus_shell_num,
                           const int32_t* shell_ang_mom, int64_t* ao_index) {
  int64_t k = 1;
  for (int64_t n = 0; n < nucl_num; ++n)
    for (int64_t s = nucleus_index[n]; s <= nucleus_index[n] + nucleus_shell_num[n] - 1; ++s) {
      const int l = shell_ang_mom[s];
      ao_index[s] = k - 1;
      k += lstart(l + 1) - lstart(l);
    }
}

static int max_lmax(int64_t nucl_num, const int32_t* nucleus_max_ang_mom) {
  int m = 0;
  for (int64_t n = 0; n < nucl_num; ++n) m = m > nucleus_max_ang_mom[n] ? m : nucleus_max_ang_mom[n];
  return m;
}

/*
 * AO vgl (value_only = 0) or AO value (value_only = 1) for one point: polynomial part
 * src/qmckl_ao_sycl.cpp:195-334 (value: :527-677) and assembly :337-422 (value:
 * :684-727). shell_vgl is this point's [5][shell_num] block.
 */
static void ao_point(int64_t ip, int value_only, int64_t point_num, int64_t nucl_num, int64_t shell_num,
                     int64_t ao_num, const int32_t* s2n, const int64_t* ao_index, const double* coord,
                     const double* nucl_coord, const double* nucleus_range, const int32_t* nucleus_max_ang_mom,
                     const int32_t* shell_ang_mom, const double* ao_factor, const double* shell_vgl, double* pows,
                     double* poly_all, int* screened, double* out) {
  const int lm = max_lmax(nucl_num, nucleus_max_ang_mom);
  const int64_t npoly = 5 * lstart(lm + 1);
  for (int64_t n = 0; n < nucl_num; ++n) {
    const double x = coord[ip] - nucl_coord[n];
    const double y = coord[ip + point_num] - nucl_coord[n + nucl_num];
    const double z = coord[ip + 2 * point_num] - nucl_coord[n + 2 * nucl_num];
    const double r2 = x * x + y * y + z * z;
    screened[n] = r2 > ORACLE_CUTOFF * nucleus_range[n];
    if (!screened[n]) poly_vgl_point(x, y, z, nucleus_max_ang_mom[n], pows, poly_all + n * npoly);
  }
  for (int64_t is = 0; is < shell_num; ++is) {
    const int64_t n = s2n[is];
    if (screened[n]) continue;
    const double* poly = poly_all + n * npoly;
    const double s0 = shell_vgl[is + 0 * shell_num];
    int64_t k = ao_index[is];
    const int l = shell_ang_mom[is];
    if (value_only) {
      for (int64_t il = lstart(l) - 1; il <= lstart(l + 1) - 2; il++) {
        out[k] = poly[il * 5] * s0 * ao_factor[k];
        k = k + 1;
      }
      continue;
    }
    const double s1 = shell_vgl[is + 1 * shell_num];
    const double s2 = shell_vgl[is + 2 * shell_num];
    const double s3 = shell_vgl[is + 3 * shell_num];
    const double s4 = shell_vgl[is + 4 * shell_num];
    for (int64_t il = lstart(l) - 1; il <= lstart(l + 1) - 2; il++) {
      const double* pp = poly + il * 5;
      out[k + 0 * ao_num] = pp[0] * s0 * ao_factor[k];
      out[k + 1 * ao_num] = (pp[1] * s0 + pp[0] * s1) * ao_factor[k];
      out[k + 2 * ao_num] = (pp[2] * s0 + pp[0] * s2) * ao_factor[k];
      out[k + 3 * ao_num] = (pp[3] * s0 + pp[0] * s3) * ao_factor[k];
      out[k + 4 * ao_num] = (pp[4] * s0 + pp[0] * s4 + 2.0 * (pp[1] * s1 + pp[2] * s2 + pp[3] * s3)) * ao_factor[k];
      k = k + 1;
    }
  }
}

static void ao_all(int value_only, int64_t point_num, int64_t nucl_num, int64_t shell_num, int64_t ao_num,
                   const int64_t* nucleus_index, const int64_t* nucleus_shell_num, const double* coord,
                   const double* nucl_coord, const double* nucleus_range, const int32_t* nucleus_max_ang_mom,
                   const int32_t* shell_ang_mom, const double* ao_factor, const double* shell_vgl, double* out) {
  int32_t* s2n = (int32_t*)malloc(sizeof(int32_t) * (size_t)shell_num);
  int64_t* ao_index = (int64_t*)malloc(sizeof(int64_t) * (size_t)shell_num);
  shell_to_nucleus(nucl_num, nucleus_index, nucleus_shell_num, shell_num, s2n);
  shell_ao_index(nucl_num, nucleus_index, nucleus_shell_num, shell_ang_mom, ao_index);
  const int lm = max_lmax(nucl_num, nucleus_max_ang_mom);
  const int64_t npoly = 5 * lstart(lm + 1);
  const int64_t stride = value_only ? ao_num : 5 * ao_num;
#pragma omp parallel
  {
    double* pows = (double*)malloc(sizeof(double) * 3 * (size_t)(lm + 3));
    double* poly = (double*)malloc(sizeof(double) * (size_t)(npoly * nucl_num));
    int* screened = (int*)malloc(sizeof(int) * (size_t)nucl_num);
#pragma omp for schedule(dynamic, 8)
    for (int64_t ip = 0; ip < point_num; ++ip)
      ao_point(ip, value_only, point_num, nucl_num, shell_num, ao_num, s2n, ao_index, coord, nucl_coord,
               nucleus_range, nucleus_max_ang_mom, shell_ang_mom, ao_factor, shell_vgl + ip * 5 * shell_num, pows,
               poly, screened, out + ip * stride);
    free(pows);
    free(poly);
    free(screened);
  }
  free(s2n);
  free(ao_index);
}

void oracle_ao_vgl(int64_t point_num, int64_t nucl_num, int64_t shell_num, int64_t ao_num,
                   const int64_t* nucleus_index, const int64_t* nucleus_shell_num, const double* coord,
                   const double* nucl_coord, const double* nucleus_range, const int32_t* nucleus_max_ang_mom,
                   const int32_t* shell_ang_mom, const double* ao_factor, const double* shell_vgl, double* ao_vgl) {
  ao_all(0, point_num, nucl_num, shell_num, ao_num, nucleus_index, nucleus_shell_num, coord, nucl_coord,
         nucleus_range, nucleus_max_ang_mom, shell_ang_mom, ao_factor, shell_vgl, ao_vgl);
}

void oracle_ao_value(int64_t point_num, int64_t nucl_num, int64_t shell_num, int64_t ao_num,
                     const int64_t* nucleus_index, const int64_t* nucleus_shell_num, const double* coord,
                     const double* nucl_coord, const double* nucleus_range, const int32_t* nucleus_max_ang_mom,
                     const int32_t* shell_ang_mom, const double* ao_factor, const double* shell_vgl,
                     double* ao_value) {
  ao_all(1, point_num, nucl_num, shell_num, ao_num, nucleus_index, nucleus_shell_num, coord, nucl_coord,
         nucleus_range, nucleus_max_ang_mom, shell_ang_mom, ao_factor, shell_vgl, ao_value);
}

/*
 * MO vgl, src/qmckl_mo_sycl.cpp:24-50: zero the point's block (:27-33), then for each
 * AO k and component l, skip when the AO *value* is exactly zero (:40), else
 * mo[l][i] = mo[l][i] + coef_t[k][i] * ao[l][k] (:42-47).
 */
void oracle_mo_vgl(int64_t ao_num, int64_t mo_num, int64_t point_num, const double* coef_t, const double* ao_vgl,
                   double* mo_vgl) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t j = 0; j < point_num; ++j) {
    double* mo = mo_vgl + mo_num * 5 * j;
    const double* ao = ao_vgl + ao_num * 5 * j;
    for (int64_t i = 0; i < 5 * mo_num; ++i) mo[i] = 0.;
    for (int64_t k = 0; k < ao_num; k++)
      for (int64_t l = 0; l < 5; l++)
        if (ao[k] != 0.) {
          const double c1 = ao[k + ao_num * l];
          const double* ct = coef_t + mo_num * k;
          double* m = mo + mo_num * l;
          for (int64_t i = 0; i < mo_num; i++) m[i] = m[i] + ct[i] * c1;
        }
  }
}

/*
 * MO value, src/qmckl_mo_sycl.cpp:77-129: gather the non-zero AOs of the point, then
 * accumulate four at a time while n < nidx - 4 (:102-118, left-to-right sum), and the
 * remainder one at a time (:120-128).
 */
void oracle_mo_value(int64_t ao_num, int64_t mo_num, int64_t point_num, const double* coef_t, const double* ao_value,
                     double* mo_value) {
#pragma omp parallel
  {
    double* av1 = (double*)malloc(sizeof(double) * (size_t)ao_num);
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)ao_num);
#pragma omp for schedule(dynamic, 4)
    for (int64_t ip = 0; ip < point_num; ++ip) {
      double* vgl1 = mo_value + ip * mo_num;
      const double* avgl1 = ao_value + ip * ao_num;
      for (int64_t i = 0; i < mo_num; ++i) vgl1[i] = 0.;
      int64_t nidx = 0;
      for (int64_t k = 0; k < ao_num; ++k)
        if (avgl1[k] != 0.) {
          idx[nidx] = k;
          av1[nidx] = avgl1[k];
          ++nidx;
        }
      int64_t n = 0;
      for (n = 0; n < nidx - 4; n += 4) {
        const double* ck1 = coef_t + idx[n] * mo_num;
        const double* ck2 = coef_t + idx[n + 1] * mo_num;
        const double* ck3 = coef_t + idx[n + 2] * mo_num;
        const double* ck4 = coef_t + idx[n + 3] * mo_num;
        const double a11 = av1[n], a21 = av1[n + 1], a31 = av1[n + 2], a41 = av1[n + 3];
        for (int64_t i = 0; i < mo_num; ++i) vgl1[i] = vgl1[i] + ck1[i] * a11 + ck2[i] * a21 + ck3[i] * a31 + ck4[i] * a41;
      }
      for (int64_t m = n; m < nidx; m++) {
        const double* ck = coef_t + idx[m] * mo_num;
        const double a1 = av1[m];
        for (int64_t i = 0; i < mo_num; ++i) vgl1[i] += ck[i] * a1;
      }
    }
    free(av1);
    free(idx);
  }
}

/* Coefficient transpose, src/qmckl_mo_sycl.cpp:178-183: coef_t[i][j] = coef[j][i]. */
void oracle_transpose_mo(int64_t ao_num, int64_t mo_num, const double* coef, double* coef_t) {
  for (int64_t i = 0; i < ao_num; ++i)
    for (int64_t j = 0; j < mo_num; ++j) coef_t[i * mo_num + j] = coef[j * ao_num + i];
}

/*
 * Whole forward path from the user's inputs, in the order the provide chain runs it
 * (src/qmckl_mo.cpp:114-181 -> src/qmckl_ao.cpp:123-199 -> src/qmckl_ao.cpp:47-119).
 * Any output pointer may be NULL. ao_vgl / ao_value must arrive zeroed.
 * coord is [3][point_num]; mo_coef is [mo_num][ao_num].
 */
int oracle_forward(int64_t nucl_num, const double* nucl_coord, int64_t shell_num, int64_t prim_num, int64_t ao_num,
                   const int64_t* nucleus_index, const int64_t* nucleus_shell_num, const int32_t* shell_ang_mom,
                   const int64_t* shell_prim_num, const int64_t* shell_prim_index, const double* shell_factor,
                   const double* exponent, const double* coefficient, const double* prim_factor,
                   const double* ao_factor, int64_t mo_num, const double* mo_coef, int64_t point_num,
                   const double* coord, double* ao_vgl, double* ao_value, double* mo_vgl, double* mo_value) {
  int64_t* nucleus_prim_index = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nucl_num + 1));
  double* coef_norm = (double*)malloc(sizeof(double) * (size_t)prim_num);
  int32_t* nmax = (int32_t*)malloc(sizeof(int32_t) * (size_t)nucl_num);
  double* nrange = (double*)malloc(sizeof(double) * (size_t)nucl_num);
  oracle_finalize_ao(nucl_num, shell_num, prim_num, nucleus_index, nucleus_shell_num, shell_ang_mom,
                     shell_prim_index, shell_prim_num, exponent, coefficient, prim_factor, shell_factor,
                     nucleus_prim_index, coef_norm, nmax, nrange);
  double* shell_vgl = (double*)calloc((size_t)(point_num * 5 * shell_num), sizeof(double));
  oracle_shell_vgl(point_num, nucl_num, shell_num, nucleus_index, nucleus_shell_num, nrange, shell_prim_index,
                   shell_prim_num, coord, nucl_coord, exponent, coef_norm, shell_vgl);
  double* ao_tmp = ao_vgl;
  if (!ao_tmp && mo_vgl) ao_tmp = (double*)calloc((size_t)(point_num * 5 * ao_num), sizeof(double));
  if (ao_tmp)
    oracle_ao_vgl(point_num, nucl_num, shell_num, ao_num, nucleus_index, nucleus_shell_num, coord, nucl_coord, nrange,
                  nmax, shell_ang_mom, ao_factor, shell_vgl, ao_tmp);
  double* aov_tmp = ao_value;
  if (!aov_tmp && mo_value) aov_tmp = (double*)calloc((size_t)(point_num * ao_num), sizeof(double));
  if (aov_tmp)
    oracle_ao_value(point_num, nucl_num, shell_num, ao_num, nucleus_index, nucleus_shell_num, coord, nucl_coord,
                    nrange, nmax, shell_ang_mom, ao_factor, shell_vgl, aov_tmp);
  if ((mo_vgl || mo_value) && mo_num > 0) {
    double* ct = (double*)malloc(sizeof(double) * (size_t)(ao_num * mo_num));
    oracle_transpose_mo(ao_num, mo_num, mo_coef, ct);
    if (mo_vgl) oracle_mo_vgl(ao_num, mo_num, point_num, ct, ao_tmp, mo_vgl);
    if (mo_value) oracle_mo_value(ao_num, mo_num, point_num, ct, aov_tmp, mo_value);
    free(ct);
  }
  if (ao_tmp != ao_vgl) free(ao_tmp);
  if (aov_tmp != ao_value) free(aov_tmp);
  free(shell_vgl);
  free(nucleus_prim_index);
  free(coef_norm);
  free(nmax);
  free(nrange);
  return 0;
}

/* ======================================================================================
 * FP64 reference gradient of L = sum_{p,l,m} w[p][l][m] * mo_vgl[p][l][m] (the adjoint form).
 * The reference library has no derivatives; this is the oracle's own restatement, written
 * per primitive (each primitive's contribution c e^{-a r^2} P(x,y,z) differentiated on its
 * own), so that it shares no aggregation with the GPU kernels. Forward quantities come from
 * the functions above (the reference's arithmetic); the MO kernel's zero-value skip
 * (src/qmckl_mo_sycl.cpp:40) is a constant mask: where ao_vgl[p][0][k] == 0 no component of
 * AO k contributes, so no gradient flows through it. Screening decisions are held fixed.
 *
 *   d_coef [mo_num][ao_num]  dL/dC for the user's coefficient layout
 *   d_expo [prim_num]        dL/dexponent (user primitive order)
 *   d_coord [point_num][3]   dL/d(point coordinates)
 * ====================================================================================== */

/* d^(dx+dy+dz) (x^a y^b z^c) / dx^dx dy^dy dz^dz */
static double mono_deriv(int a, int b, int c, int dx, int dy, int dz, double x, double y, double z) {
  if (dx > a || dy > b || dz > c) return 0.0;
  double f = 1.0;
  for (int i = 0; i < dx; ++i) f *= (double)(a - i);
  for (int i = 0; i < dy; ++i) f *= (double)(b - i);
  for (int i = 0; i < dz; ++i) f *= (double)(c - i);
  for (int i = 0; i < a - dx; ++i) f *= x;
  for (int i = 0; i < b - dy; ++i) f *= y;
  for (int i = 0; i < c - dz; ++i) f *= z;
  return f;
}

/* derivative multi-index of axis j added to (d0,d1,d2) */
#define OR_D(P, d0, d1, d2) mono_deriv(a, b, c, (d0), (d1), (d2), x, y, z)

int oracle_vjp_mo_vgl(int64_t nucl_num, const double* nucl_coord, int64_t shell_num, int64_t prim_num, int64_t ao_num,
                      const int64_t* nucleus_index, const int64_t* nucleus_shell_num, const int32_t* shell_ang_mom,
                      const int64_t* shell_prim_num, const int64_t* shell_prim_index, const double* shell_factor,
                      const double* exponent, const double* coefficient, const double* prim_factor,
                      const double* ao_factor, int64_t mo_num, const double* mo_coef, int64_t point_num,
                      const double* coord, const double* w, double* d_coef, double* d_expo, double* d_coord) {
  int64_t* nucleus_prim_index = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nucl_num + 1));
  double* coef_norm = (double*)malloc(sizeof(double) * (size_t)prim_num);
  int32_t* nmax = (int32_t*)malloc(sizeof(int32_t) * (size_t)nucl_num);
  double* nrange = (double*)malloc(sizeof(double) * (size_t)nucl_num);
  oracle_finalize_ao(nucl_num, shell_num, prim_num, nucleus_index, nucleus_shell_num, shell_ang_mom,
                     shell_prim_index, shell_prim_num, exponent, coefficient, prim_factor, shell_factor,
                     nucleus_prim_index, coef_norm, nmax, nrange);
  double* shell_vgl = (double*)calloc((size_t)(point_num * 5 * shell_num), sizeof(double));
  oracle_shell_vgl(point_num, nucl_num, shell_num, nucleus_index, nucleus_shell_num, nrange, shell_prim_index,
                   shell_prim_num, coord, nucl_coord, exponent, coef_norm, shell_vgl);
  double* ao = (double*)calloc((size_t)(point_num * 5 * ao_num), sizeof(double));
  oracle_ao_vgl(point_num, nucl_num, shell_num, ao_num, nucleus_index, nucleus_shell_num, coord, nucl_coord, nrange,
                nmax, shell_ang_mom, ao_factor, shell_vgl, ao);
  int32_t* s2n = (int32_t*)malloc(sizeof(int32_t) * (size_t)shell_num);
  int64_t* ao_index = (int64_t*)malloc(sizeof(int64_t) * (size_t)shell_num);
  shell_to_nucleus(nucl_num, nucleus_index, nucleus_shell_num, shell_num, s2n);
  shell_ao_index(nucl_num, nucleus_index, nucleus_shell_num, shell_ang_mom, ao_index);
  const int nthreads = oracle_num_threads();
  double* dc_all = d_coef ? (double*)calloc((size_t)nthreads * (size_t)(mo_num * ao_num), sizeof(double)) : NULL;
  double* de_all = d_expo ? (double*)calloc((size_t)nthreads * (size_t)prim_num, sizeof(double)) : NULL;

#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double* gbar = (double*)malloc(sizeof(double) * (size_t)(5 * ao_num));
    double* dc = dc_all ? dc_all + (size_t)tid * (size_t)(mo_num * ao_num) : NULL;
    double* de = de_all ? de_all + (size_t)tid * (size_t)prim_num : NULL;
#pragma omp for schedule(dynamic, 4)
    for (int64_t p = 0; p < point_num; ++p) {
      const double* a_p = ao + p * 5 * ao_num;
      const double* w_p = w + p * 5 * mo_num;
      /* adjoint of the AO values: gbar[l][k] = sum_m w[l][m] C[m][k], masked */
      for (int64_t l = 0; l < 5; ++l)
        for (int64_t k = 0; k < ao_num; ++k) {
          double s = 0.0;
          if (a_p[k] != 0.0)
            for (int64_t m = 0; m < mo_num; ++m) s += w_p[l * mo_num + m] * mo_coef[m * ao_num + k];
          gbar[l * ao_num + k] = s;
        }
      if (dc)
        for (int64_t k = 0; k < ao_num; ++k) {
          if (a_p[k] == 0.0) continue;
          for (int64_t l = 0; l < 5; ++l) {
            const double av = a_p[l * ao_num + k];
            for (int64_t m = 0; m < mo_num; ++m) dc[m * ao_num + k] += w_p[l * mo_num + m] * av;
          }
        }
      if (!de && !d_coord) continue;
      double gc[3] = {0.0, 0.0, 0.0};
      for (int64_t is = 0; is < shell_num; ++is) {
        const int64_t n = s2n[is];
        const double x = coord[p] - nucl_coord[n];
        const double y = coord[p + point_num] - nucl_coord[n + nucl_num];
        const double z = coord[p + 2 * point_num] - nucl_coord[n + 2 * nucl_num];
        const double r2 = x * x + y * y + z * z;
        if (r2 > ORACLE_CUTOFF * nrange[n]) continue;
        const double xv[3] = {x, y, z};
        const int L = shell_ang_mom[is];
        for (int64_t q = shell_prim_index[is]; q < shell_prim_index[is] + shell_prim_num[is]; ++q) {
          const double al = exponent[q];
          const double ar2 = al * r2;
          if (ar2 > ORACLE_CUTOFF) continue;
          const double v = coef_norm[q] * exp(-ar2);
          /* v and its derivatives: dv_j = -2 a x_j v; d2v_jd = (4 a^2 x_j x_d - 2 a delta_jd) v;
             lap v = (4 a^2 r2 - 6 a) v; d_j lap v = (8 a^2 x_j + (4 a^2 r2 - 6 a)(-2 a x_j)) v */
          double dv[3], d2v[3][3], dlapv[3];
          const double lapv = (4.0 * al * al * r2 - 6.0 * al) * v;
          for (int j = 0; j < 3; ++j) {
            dv[j] = -2.0 * al * xv[j] * v;
            for (int d = 0; d < 3; ++d) d2v[j][d] = (4.0 * al * al * xv[j] * xv[d] - (j == d ? 2.0 * al : 0.0)) * v;
            dlapv[j] = 8.0 * al * al * xv[j] * v + (4.0 * al * al * r2 - 6.0 * al) * dv[j];
          }
          /* derivatives with respect to the exponent */
          const double v_a = -r2 * v;
          double dv_a[3];
          for (int j = 0; j < 3; ++j) dv_a[j] = -2.0 * xv[j] * v - 2.0 * al * xv[j] * v_a;
          const double lapv_a = (8.0 * al * r2 - 6.0) * v + (4.0 * al * al * r2 - 6.0 * al) * v_a;
          int64_t k = ao_index[is];
          for (int a = L; a >= 0; --a)
            for (int b = L - a; b >= 0; --b, ++k) {
              const int c = L - a - b;
              const double f = ao_factor[k];
              const double g0 = gbar[k], g1 = gbar[ao_num + k], g2 = gbar[2 * ao_num + k],
                           g3 = gbar[3 * ao_num + k], g4 = gbar[4 * ao_num + k];
              if (g0 == 0.0 && g1 == 0.0 && g2 == 0.0 && g3 == 0.0 && g4 == 0.0) continue;
              const double gd[3] = {g1, g2, g3};
              const double P = OR_D(P, 0, 0, 0);
              const double Pj[3] = {OR_D(P, 1, 0, 0), OR_D(P, 0, 1, 0), OR_D(P, 0, 0, 1)};
              double Pjd[3][3];
              for (int j = 0; j < 3; ++j)
                for (int d = 0; d < 3; ++d) {
                  int e[3] = {0, 0, 0};
                  e[j] += 1;
                  e[d] += 1;
                  Pjd[j][d] = OR_D(P, e[0], e[1], e[2]);
                }
              const double lapP = Pjd[0][0] + Pjd[1][1] + Pjd[2][2];
              if (de) {
                /* outputs of this primitive: phi = P v, d_d phi, lap phi; their exponent derivatives */
                double s = g0 * P * v_a;
                for (int d = 0; d < 3; ++d) s += gd[d] * (Pj[d] * v_a + P * dv_a[d]);
                double lap_a = lapP * v_a + P * lapv_a;
                for (int d = 0; d < 3; ++d) lap_a += 2.0 * Pj[d] * dv_a[d];
                s += g4 * lap_a;
                de[q] += f * s;
              }
              if (d_coord)
                for (int j = 0; j < 3; ++j) {
                  double dlapP = 0.0;
                  for (int d = 0; d < 3; ++d) {
                    int e[3] = {0, 0, 0};
                    e[j] += 1;
                    e[d] += 2;
                    dlapP += OR_D(P, e[0], e[1], e[2]);
                  }
                  double s = g0 * (Pj[j] * v + P * dv[j]);
                  for (int d = 0; d < 3; ++d)
                    s += gd[d] * (Pjd[j][d] * v + Pj[d] * dv[j] + Pj[j] * dv[d] + P * d2v[j][d]);
                  double t = dlapP * v + lapP * dv[j] + Pj[j] * lapv + P * dlapv[j];
                  for (int d = 0; d < 3; ++d) t += 2.0 * (Pjd[d][j] * dv[d] + Pj[d] * d2v[d][j]);
                  s += g4 * t;
                  gc[j] += f * s;
                }
            }
        }
      }
      if (d_coord)
        for (int j = 0; j < 3; ++j) d_coord[p * 3 + j] = gc[j];
    }
    free(gbar);
  }
  if (d_coef) {
    for (int64_t i = 0; i < mo_num * ao_num; ++i) {
      double s = 0.0;
      for (int t = 0; t < nthreads; ++t) s += dc_all[(size_t)t * (size_t)(mo_num * ao_num) + i];
      d_coef[i] = s;
    }
  }
  if (d_expo) {
    for (int64_t q = 0; q < prim_num; ++q) {
      double s = 0.0;
      for (int t = 0; t < nthreads; ++t) s += de_all[(size_t)t * (size_t)prim_num + q];
      d_expo[q] = s;
    }
  }
  free(dc_all);
  free(de_all);
  free(s2n);
  free(ao_index);
  free(ao);
  free(shell_vgl);
  free(nucleus_prim_index);
  free(coef_norm);
  free(nmax);
  free(nrange);
  return 0;
}
#undef OR_D

/* ======================================================================================
 * Distances: the intended result of src/qmckl_electron.cpp:373-552 (qmckl_distance_device), which
 * the reference's kernel garbles (every work-item takes square roots of a whole column of C):
 * C[i + j*ldc] = sqrt((x*x + y*y) + z*z), x = A_i - B_j per coordinate, point i of A stored as
 * A[d + i*lda] ('N') or A[i + d*lda] ('T'), same for B.
 * ====================================================================================== */
void oracle_distance(char transa, char transb, int64_t m, int64_t n, const double* A, int64_t lda, const double* B,
                     int64_t ldb, double* C, int64_t ldc) {
  const int ta = transa == 'T' || transa == 't', tb = transb == 'T' || transb == 't';
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < m; ++i) {
      double d[3];
      for (int k = 0; k < 3; ++k) {
        const double a = ta ? A[i + k * lda] : A[k + i * lda];
        const double b = tb ? B[j + k * ldb] : B[k + j * ldb];
        d[k] = a - b;
      }
      C[i + j * ldc] = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    }
}
