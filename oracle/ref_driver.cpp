// C-ABI driver around the UNMODIFIED reference library (qmckl_sycl src/*.cpp built
// against the host SYCL shim in oracle/sycl_shim). Test infrastructure only: it lets
// the Python tests run the reference's own API sequence (tests/test_qmckl_mo.cpp:56-300)
// on arbitrary inputs and compare the oracle restatement against it.
//
// Inputs are host arrays in the reference's layouts:
//   nucl_coord [3][nucl_num] (set with transp 'T', tests/test_qmckl_ao.cpp:70)
//   coord      [point_num][3] (set with transp 'N', tests/test_qmckl_mo.cpp:85)
//   mo_coef    [mo_num][ao_num]
// Outputs (any may be NULL): ao_vgl [P][5][A], ao_value [P][A], mo_vgl [P][5][M],
// mo_value [P][M]. Returns 0 on success, otherwise the first failing exit code.
#include <chrono>
#include <cstring>
#include <vector>

#include "qmckl_gpu.hpp"

namespace {

template <class T> T* up(qmckl_context_device ctx, const T* h, int64_t n) {
  T* d = static_cast<T*>(qmckl_malloc_device(ctx, sizeof(T) * (size_t)n));
  qmckl_memcpy_H2D(ctx, d, const_cast<T*>(h), sizeof(T) * (size_t)n);
  return d;
}

#define REF_CHECK(x)            \
  do {                          \
    qmckl_exit_code_device r_ = (x); \
    if (r_ != QMCKL_SUCCESS_DEVICE) return r_; \
  } while (0)

int setup(qmckl_context_device ctx, int64_t nucl_num, const double* nucl_charge, const double* nucl_coord,
          int64_t shell_num, int64_t prim_num, int64_t ao_num, const int64_t* nucleus_index,
          const int64_t* nucleus_shell_num, const int32_t* shell_ang_mom, const int64_t* shell_prim_num,
          const int64_t* shell_prim_index, const double* shell_factor, const double* exponent,
          const double* coefficient, const double* prim_factor, const double* ao_factor, int64_t mo_num,
          const double* mo_coef, int64_t point_num, const double* coord) {
  double* coord_d = up(ctx, coord, 3 * point_num);
  REF_CHECK(qmckl_set_point_device(ctx, 'N', point_num, coord_d, 3 * point_num));
  REF_CHECK(qmckl_set_nucleus_num_device(ctx, nucl_num));
  REF_CHECK(qmckl_set_nucleus_coord_device(ctx, 'T', up(ctx, nucl_coord, 3 * nucl_num), 3 * nucl_num));
  REF_CHECK(qmckl_set_nucleus_charge_device(ctx, up(ctx, nucl_charge, nucl_num), nucl_num));
  REF_CHECK(qmckl_set_ao_basis_type_device(ctx, 'G'));
  REF_CHECK(qmckl_set_ao_basis_shell_num_device(ctx, shell_num));
  REF_CHECK(qmckl_set_ao_basis_prim_num_device(ctx, prim_num));
  REF_CHECK(qmckl_set_ao_basis_nucleus_index_device(ctx, up(ctx, nucleus_index, nucl_num), nucl_num));
  REF_CHECK(qmckl_set_ao_basis_nucleus_shell_num_device(ctx, up(ctx, nucleus_shell_num, nucl_num), nucl_num));
  REF_CHECK(qmckl_set_ao_basis_shell_ang_mom_device(ctx, up(ctx, shell_ang_mom, shell_num), shell_num));
  REF_CHECK(qmckl_set_ao_basis_shell_factor_device(ctx, up(ctx, shell_factor, shell_num), shell_num));
  REF_CHECK(qmckl_set_ao_basis_shell_prim_num_device(ctx, up(ctx, shell_prim_num, shell_num), shell_num));
  REF_CHECK(qmckl_set_ao_basis_shell_prim_index_device(ctx, up(ctx, shell_prim_index, shell_num), shell_num));
  REF_CHECK(qmckl_set_ao_basis_exponent_device(ctx, up(ctx, exponent, prim_num), prim_num));
  REF_CHECK(qmckl_set_ao_basis_coefficient_device(ctx, up(ctx, coefficient, prim_num), prim_num));
  REF_CHECK(qmckl_set_ao_basis_prim_factor_device(ctx, up(ctx, prim_factor, prim_num), prim_num));
  REF_CHECK(qmckl_set_ao_basis_ao_num_device(ctx, ao_num));
  REF_CHECK(qmckl_set_ao_basis_ao_factor_device(ctx, up(ctx, ao_factor, ao_num), ao_num));
  if (mo_num > 0) {
    REF_CHECK(qmckl_set_mo_basis_mo_num_device(ctx, mo_num));
    REF_CHECK(qmckl_set_mo_basis_coefficient_device(ctx, up(ctx, mo_coef, mo_num * ao_num)));
  }
  return 0;
}

template <class T> int down(qmckl_context_device ctx, T* dst, T* src_d, int64_t n) {
  return qmckl_memcpy_D2H(ctx, dst, src_d, sizeof(T) * (size_t)n);
}

}  // namespace

extern "C" int ref_run(int64_t nucl_num, const double* nucl_charge, const double* nucl_coord, int64_t shell_num,
                       int64_t prim_num, int64_t ao_num, const int64_t* nucleus_index,
                       const int64_t* nucleus_shell_num, const int32_t* shell_ang_mom,
                       const int64_t* shell_prim_num, const int64_t* shell_prim_index, const double* shell_factor,
                       const double* exponent, const double* coefficient, const double* prim_factor,
                       const double* ao_factor, int64_t mo_num, const double* mo_coef, int64_t point_num,
                       const double* coord, double* ao_vgl, double* ao_value, double* mo_vgl, double* mo_value) {
  sycl::queue q;
  qmckl_context_device ctx = qmckl_context_create_device(q);
  int rc = setup(ctx, nucl_num, nucl_charge, nucl_coord, shell_num, prim_num, ao_num, nucleus_index,
                 nucleus_shell_num, shell_ang_mom, shell_prim_num, shell_prim_index, shell_factor, exponent,
                 coefficient, prim_factor, ao_factor, mo_num, mo_coef, point_num, coord);
  if (rc) return rc;
  const int64_t P = point_num;
  if (ao_vgl) {
    double* d = (double*)qmckl_malloc_device(ctx, sizeof(double) * 5 * P * ao_num);
    REF_CHECK(qmckl_get_ao_basis_ao_vgl_device(ctx, d, 5 * P * ao_num));
    down(ctx, ao_vgl, d, 5 * P * ao_num);
  }
  if (ao_value) {
    double* d = (double*)qmckl_malloc_device(ctx, sizeof(double) * P * ao_num);
    REF_CHECK(qmckl_get_ao_basis_ao_value_device(ctx, d, P * ao_num));
    down(ctx, ao_value, d, P * ao_num);
  }
  if (mo_vgl && mo_num > 0) {
    double* d = (double*)qmckl_malloc_device(ctx, sizeof(double) * 5 * P * mo_num);
    REF_CHECK(qmckl_get_mo_basis_mo_vgl_device(ctx, d, 5 * P * mo_num));
    down(ctx, mo_vgl, d, 5 * P * mo_num);
  }
  if (mo_value && mo_num > 0) {
    // Fresh date so that mo_value is computed from ao_value, not copied from mo_vgl
    // (mo.cpp:232 vs mo.cpp:263).
    REF_CHECK(qmckl_context_touch_device(ctx));
    double* d = (double*)qmckl_malloc_device(ctx, sizeof(double) * P * mo_num);
    REF_CHECK(qmckl_get_mo_basis_mo_value_device(ctx, d, P * mo_num));
    down(ctx, mo_value, d, P * mo_num);
  }
  return qmckl_context_destroy_device(ctx);
}

// Times `reps` calls of touch + get_mo_basis_mo_vgl (the recompute a QMC step pays),
// after one untimed warm-up call; seconds[i] receives each call's wall time.
extern "C" int ref_time_mo_vgl(int64_t nucl_num, const double* nucl_charge, const double* nucl_coord,
                               int64_t shell_num, int64_t prim_num, int64_t ao_num, const int64_t* nucleus_index,
                               const int64_t* nucleus_shell_num, const int32_t* shell_ang_mom,
                               const int64_t* shell_prim_num, const int64_t* shell_prim_index,
                               const double* shell_factor, const double* exponent, const double* coefficient,
                               const double* prim_factor, const double* ao_factor, int64_t mo_num,
                               const double* mo_coef, int64_t point_num, const double* coord, int reps,
                               double* seconds) {
  sycl::queue q;
  qmckl_context_device ctx = qmckl_context_create_device(q);
  int rc = setup(ctx, nucl_num, nucl_charge, nucl_coord, shell_num, prim_num, ao_num, nucleus_index,
                 nucleus_shell_num, shell_ang_mom, shell_prim_num, shell_prim_index, shell_factor, exponent,
                 coefficient, prim_factor, ao_factor, mo_num, mo_coef, point_num, coord);
  if (rc) return rc;
  const int64_t n = 5 * point_num * mo_num;
  double* d = (double*)qmckl_malloc_device(ctx, sizeof(double) * n);
  REF_CHECK(qmckl_get_mo_basis_mo_vgl_device(ctx, d, n));
  for (int r = 0; r < reps; ++r) {
    auto t0 = std::chrono::steady_clock::now();
    REF_CHECK(qmckl_context_touch_device(ctx));
    REF_CHECK(qmckl_get_mo_basis_mo_vgl_device(ctx, d, n));
    auto t1 = std::chrono::steady_clock::now();
    seconds[r] = std::chrono::duration<double>(t1 - t0).count();
  }
  return qmckl_context_destroy_device(ctx);
}

// Per-nucleus exponent tables the reference leaves in its context after finalize
// (qmckl_finalize_ao_basis_hpc_device, src/qmckl_ao_sycl.cpp:855-1065, run at :1233):
// dims[0] = prim_max, dims[1] = shell_max; prim_num_per_nucleus [nucl_num],
// expo [nucl_num][prim_max], coef [nucl_num][shell_max][prim_max] are copied out when
// capacity (in doubles) suffices for both arrays. Returns 0 on success, -1 when too small.
extern "C" int ref_hpc(int64_t nucl_num, const double* nucl_charge, const double* nucl_coord, int64_t shell_num,
                       int64_t prim_num, int64_t ao_num, const int64_t* nucleus_index,
                       const int64_t* nucleus_shell_num, const int32_t* shell_ang_mom,
                       const int64_t* shell_prim_num, const int64_t* shell_prim_index, const double* shell_factor,
                       const double* exponent, const double* coefficient, const double* prim_factor,
                       const double* ao_factor, int64_t* dims, int32_t* prim_num_per_nucleus, double* expo,
                       double* coef, int64_t capacity) {
  sycl::queue q;
  qmckl_context_device ctx = qmckl_context_create_device(q);
  const double coord[3] = {0.0, 0.0, 0.0};
  int rc = setup(ctx, nucl_num, nucl_charge, nucl_coord, shell_num, prim_num, ao_num, nucleus_index,
                 nucleus_shell_num, shell_ang_mom, shell_prim_num, shell_prim_index, shell_factor, exponent,
                 coefficient, prim_factor, ao_factor, 0, nullptr, 1, coord);
  if (rc) return rc;
  const qmckl_context_struct_device* c = reinterpret_cast<const qmckl_context_struct_device*>(ctx);
  const int64_t pm = c->ao_basis.expo_per_nucleus.size[0];
  const int64_t sm = c->ao_basis.coef_per_nucleus.size[1];
  dims[0] = pm;
  dims[1] = sm;
  if (capacity < nucl_num * pm || capacity < nucl_num * sm * pm) {
    qmckl_context_destroy_device(ctx);
    return -1;
  }
  std::memcpy(prim_num_per_nucleus, c->ao_basis.prim_num_per_nucleus, sizeof(int32_t) * (size_t)nucl_num);
  std::memcpy(expo, c->ao_basis.expo_per_nucleus.data, sizeof(double) * (size_t)(nucl_num * pm));
  std::memcpy(coef, c->ao_basis.coef_per_nucleus.data, sizeof(double) * (size_t)(nucl_num * sm * pm));
  return qmckl_context_destroy_device(ctx);
}
