/*
 * qmckl_gpu.h — C ABI of the GB300 (sm_103a) implementation of the QMCkl basis-evaluation
 * path: electron-nucleus displacement, Gaussian shell radials with exponent-cutoff
 * screening, Cartesian AO polynomial vgl, and the MO vgl contraction.
 *
 * Drop-in for the `*_device` context API of the reference library (qmckl_sycl,
 * include/qmckl_gpu.hpp): same function names, argument lists, exit codes and error
 * behaviour. Every array argument is a pointer that the GPU can reach (device memory,
 * or host memory through unified addressing); the library copies what it keeps. Every
 * call that launches work waits for it before returning, like the reference's
 * `q.wait()`, unless the context was switched to asynchronous mode.
 *
 * The one signature change: contexts are created on a CUDA device ordinal (or on a
 * caller-provided cudaStream_t) instead of a sycl::queue
 * (reference: src/qmckl_context.cpp:187).
 *
 * Layouts are C index order, exactly as the reference indexes them:
 *   ao_vgl [point][5][ao], ao_value [point][ao], mo_vgl [point][5][mo],
 *   mo_value [point][mo], shell_vgl [point][5][shell]; component 0 is the value,
 *   1..3 the gradient (x, y, z), 4 the Laplacian.
 */
#ifndef QMCKL_GPU_H
#define QMCKL_GPU_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Types and exit codes (reference: include/qmckl_types.hpp:24-57,74,116) ---- */
typedef int32_t qmckl_exit_code_device;
typedef int64_t qmckl_context_device;

#define QMCKL_NULL_CONTEXT_DEVICE ((qmckl_context_device)0)

#define QMCKL_SUCCESS_DEVICE ((qmckl_exit_code_device)0)
#define QMCKL_INVALID_ARG_1_DEVICE ((qmckl_exit_code_device)1)
#define QMCKL_INVALID_ARG_2_DEVICE ((qmckl_exit_code_device)2)
#define QMCKL_INVALID_ARG_3_DEVICE ((qmckl_exit_code_device)3)
#define QMCKL_INVALID_ARG_4_DEVICE ((qmckl_exit_code_device)4)
#define QMCKL_INVALID_ARG_5_DEVICE ((qmckl_exit_code_device)5)
#define QMCKL_INVALID_ARG_6_DEVICE ((qmckl_exit_code_device)6)
#define QMCKL_INVALID_ARG_7_DEVICE ((qmckl_exit_code_device)7)
#define QMCKL_INVALID_ARG_8_DEVICE ((qmckl_exit_code_device)8)
#define QMCKL_INVALID_ARG_9_DEVICE ((qmckl_exit_code_device)9)
#define QMCKL_INVALID_ARG_10_DEVICE ((qmckl_exit_code_device)10)
#define QMCKL_INVALID_ARG_11_DEVICE ((qmckl_exit_code_device)11)
#define QMCKL_INVALID_ARG_12_DEVICE ((qmckl_exit_code_device)12)
#define QMCKL_INVALID_ARG_13_DEVICE ((qmckl_exit_code_device)13)
#define QMCKL_INVALID_ARG_14_DEVICE ((qmckl_exit_code_device)14)
#define QMCKL_INVALID_ARG_15_DEVICE ((qmckl_exit_code_device)15)
#define QMCKL_INVALID_ARG_16_DEVICE ((qmckl_exit_code_device)16)
#define QMCKL_INVALID_ARG_17_DEVICE ((qmckl_exit_code_device)17)
#define QMCKL_INVALID_ARG_18_DEVICE ((qmckl_exit_code_device)18)
#define QMCKL_INVALID_ARG_19_DEVICE ((qmckl_exit_code_device)19)
#define QMCKL_INVALID_ARG_20_DEVICE ((qmckl_exit_code_device)20)
#define QMCKL_FAILURE_DEVICE ((qmckl_exit_code_device)101)
#define QMCKL_ERRNO_DEVICE ((qmckl_exit_code_device)102)
#define QMCKL_INVALID_CONTEXT_DEVICE ((qmckl_exit_code_device)103)
#define QMCKL_ALLOCATION_FAILED_DEVICE ((qmckl_exit_code_device)104)
#define QMCKL_DEALLOCATION_FAILED_DEVICE ((qmckl_exit_code_device)105)
#define QMCKL_NOT_PROVIDED_DEVICE ((qmckl_exit_code_device)106)
#define QMCKL_OUT_OF_BOUNDS_DEVICE ((qmckl_exit_code_device)107)
#define QMCKL_ALREADY_SET_DEVICE ((qmckl_exit_code_device)108)
#define QMCKL_INVALID_EXIT_CODE_DEVICE ((qmckl_exit_code_device)109)

#define QMCKL_MAX_FUN_LEN_DEVICE 256
#define QMCKL_MAX_MSG_LEN_DEVICE 1024

/* Host allocation record (reference: include/qmckl_types.hpp:100-103). */
typedef struct qmckl_memory_info_struct {
  size_t size;
  void* pointer;
} qmckl_memory_info_struct_device;

/* Containers, Fortran order: element (i, j) of a matrix is data[i + j*size[0]]
 * (reference: include/qmckl_types.hpp:78-96). */
typedef struct qmckl_vector_device {
  double* data;
  int64_t size;
} qmckl_vector_device;
typedef struct qmckl_matrix_device {
  double* data;
  int64_t size[2];
} qmckl_matrix_device;
#define QMCKL_TENSOR_ORDER_MAX_DEVICE 16
typedef struct qmckl_tensor_device {
  double* data;
  int64_t order;
  int64_t size[QMCKL_TENSOR_ORDER_MAX_DEVICE];
} qmckl_tensor_device;

/* ---- Context (reference: src/qmckl_context.cpp) ---- */
/* replaces qmckl_context_create_device(sycl::queue), src/qmckl_context.cpp:187-288 */
qmckl_context_device qmckl_context_create_device(int32_t device_id);
/* same, but work is issued on the caller's cudaStream_t (passed as void*) */
qmckl_context_device qmckl_context_create_with_stream_device(int32_t device_id, void* cuda_stream);
/* src/qmckl_context.cpp:294-345: frees every registered allocation, invalidates the tag */
qmckl_exit_code_device qmckl_context_destroy_device(const qmckl_context_device context);
/* src/qmckl_context.cpp:64-79: the context itself if valid, else QMCKL_NULL_CONTEXT_DEVICE */
qmckl_context_device qmckl_context_check_device(const qmckl_context_device context);
/* src/qmckl_context.cpp:47-62: date += 1, point.date = date (invalidates every cached array) */
qmckl_exit_code_device qmckl_context_touch_device(const qmckl_context_device context);
/* src/qmckl_context.cpp:81-110 (recursive lock) */
void qmckl_lock_device(qmckl_context_device context);
void qmckl_unlock_device(qmckl_context_device context);

/* ---- Errors (reference: src/qmckl_basic_functions.cpp) ---- */
/* src/qmckl_basic_functions.cpp:12-40 */
qmckl_exit_code_device qmckl_set_error_device(qmckl_context_device context, const qmckl_exit_code_device exit_code,
                                              const char* function_name, const char* message);
/* src/qmckl_basic_functions.cpp:51-78: records the error and returns exit_code */
qmckl_exit_code_device qmckl_failwith_device(qmckl_context_device context, const qmckl_exit_code_device exit_code,
                                             const char* function, const char* message);
/* src/qmckl_basic_functions.cpp:42-48 (the reference's switch is empty; this one names each code) */
const char* qmckl_string_of_error_device(const qmckl_exit_code_device error);
/* Reads ctx->error (include/qmckl_types.hpp:59-65); function/message buffers may be NULL. */
qmckl_exit_code_device qmckl_get_error_device(qmckl_context_device context, qmckl_exit_code_device* exit_code,
                                              char* function, int64_t function_size, char* message,
                                              int64_t message_size);

/* ---- Memory (reference: src/qmckl_memory.cpp) ---- */
/* src/qmckl_memory.cpp:15-65 */
void* qmckl_malloc_host(qmckl_context_device context, const qmckl_memory_info_struct_device info);
/* src/qmckl_memory.cpp:70-125: device allocation recorded in the context (zero-filled) */
void* qmckl_malloc_device(qmckl_context_device context, size_t size);
/* src/qmckl_memory.cpp:127-171 */
qmckl_exit_code_device qmckl_free_host(qmckl_context_device context, void* const ptr);
/* src/qmckl_memory.cpp:173-220: QMCKL_FAILURE_DEVICE if the pointer is not registered */
qmckl_exit_code_device qmckl_free_device(qmckl_context_device context, void* const ptr);
/* src/qmckl_memory.cpp:226-361: synchronous copies on the context's stream */
qmckl_exit_code_device qmckl_memcpy_H2D(qmckl_context_device context, void* const dest, void* const src, size_t size);
qmckl_exit_code_device qmckl_memcpy_D2H(qmckl_context_device context, void* const dest, void* const src, size_t size);
qmckl_exit_code_device qmckl_memcpy_D2D(qmckl_context_device context, void* const dest, void* const src, size_t size);

/* ---- Containers (reference: src/qmckl_blas.cpp:14-306) ---- */
qmckl_vector_device qmckl_vector_alloc_device(qmckl_context_device context, const int64_t size);
qmckl_exit_code_device qmckl_vector_free_device(qmckl_context_device context, qmckl_vector_device* vector);
qmckl_exit_code_device qmckl_vector_of_double_device(const qmckl_context_device context, const double* target,
                                                     const int64_t size_max, qmckl_vector_device* vector_out);
qmckl_matrix_device qmckl_matrix_alloc_device(qmckl_context_device context, const int64_t size1, const int64_t size2);
qmckl_exit_code_device qmckl_matrix_free_device(qmckl_context_device context, qmckl_matrix_device* matrix);
qmckl_exit_code_device qmckl_matrix_of_double_device(const qmckl_context_device context, const double* target,
                                                     const int64_t size_max, qmckl_matrix_device* matrix_out);
qmckl_exit_code_device qmckl_transpose_device(qmckl_context_device context, const qmckl_matrix_device A,
                                              qmckl_matrix_device At);
qmckl_tensor_device qmckl_tensor_alloc_device(qmckl_context_device context, const int64_t order, const int64_t* size);
qmckl_exit_code_device qmckl_tensor_free_device(qmckl_context_device context, qmckl_tensor_device* tensor);

/* ---- Points (reference: src/qmckl_point.cpp) ---- */
/* src/qmckl_point.cpp:68-135: 'N' = coord[num][3], 'T' = coord[3][num]; touches the context */
qmckl_exit_code_device qmckl_set_point_device(qmckl_context_device context, char transp, int64_t num, double* coord,
                                              int64_t size_max);
/* src/qmckl_point.cpp:5-66 */
qmckl_exit_code_device qmckl_get_point_device(const qmckl_context_device context, const char transp,
                                              double* const coord, const int64_t size_max);

/* ---- Nucleus (reference: src/qmckl_nucleus.cpp:359-663) ---- */
bool qmckl_nucleus_provided_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_get_nucleus_num_device(qmckl_context_device context, int64_t* num);
/* src/qmckl_nucleus.cpp:510-540: QMCKL_ALREADY_SET_DEVICE on a second call */
qmckl_exit_code_device qmckl_set_nucleus_num_device(qmckl_context_device context, int64_t num);
/* src/qmckl_nucleus.cpp:614-663 */
qmckl_exit_code_device qmckl_set_nucleus_charge_device(qmckl_context_device context, double* charge,
                                                       int64_t size_max);
/* src/qmckl_nucleus.cpp:543-610: 'N' = coord[num][3], 'T' = coord[3][num] */
qmckl_exit_code_device qmckl_set_nucleus_coord_device(qmckl_context_device context, char transp, double* coord,
                                                      int64_t size_max);
qmckl_exit_code_device qmckl_get_nucleus_coord_device(const qmckl_context_device context, const char transp,
                                                      double* const coord, const int64_t size_max);
qmckl_exit_code_device qmckl_get_nucleus_charge_device(const qmckl_context_device context, double* const charge,
                                                       const int64_t size_max);

/* ---- Electrons (reference: src/qmckl_electron.cpp:8-190) ---- */
bool qmckl_electron_provided_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_set_electron_num_device(qmckl_context_device context, int64_t up_num, int64_t down_num);
/* src/qmckl_electron.cpp:50-90: swaps the walker point sets, then set_point(walk_num*elec_num) */
qmckl_exit_code_device qmckl_set_electron_coord_device(qmckl_context_device context, char transp, int64_t walk_num,
                                                       double* coord, int64_t size_max);
qmckl_exit_code_device qmckl_get_electron_num_device(const qmckl_context_device context, int64_t* const num);
qmckl_exit_code_device qmckl_get_electron_coord_device(const qmckl_context_device context, const char transp,
                                                       double* const coord, const int64_t size_max);

/* ---- AO basis (reference: src/qmckl_ao.cpp, src/qmckl_ao_sycl.cpp) ---- */
bool qmckl_ao_basis_provided_device(qmckl_context_device context); /* src/qmckl_ao.cpp:28-40 */
/* Setters, src/qmckl_ao.cpp:402-1236. Each clears one bit of the 14-bit mask; the setter
 * that clears the last bit runs the finalize step (src/qmckl_ao_sycl.cpp:1067-1236). */
qmckl_exit_code_device qmckl_set_ao_basis_type_device(qmckl_context_device context, char basis_type);
qmckl_exit_code_device qmckl_set_ao_basis_shell_num_device(qmckl_context_device context, int64_t shell_num);
qmckl_exit_code_device qmckl_set_ao_basis_prim_num_device(qmckl_context_device context, int64_t prim_num);
qmckl_exit_code_device qmckl_set_ao_basis_ao_num_device(qmckl_context_device context, int64_t ao_num);
qmckl_exit_code_device qmckl_set_ao_basis_nucleus_index_device(qmckl_context_device context, int64_t* nucleus_index,
                                                               int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_nucleus_shell_num_device(qmckl_context_device context,
                                                                   int64_t* nucleus_shell_num, int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_shell_ang_mom_device(qmckl_context_device context, int32_t* shell_ang_mom,
                                                               int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_shell_prim_num_device(qmckl_context_device context,
                                                                int64_t* shell_prim_num, int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_shell_prim_index_device(qmckl_context_device context,
                                                                  int64_t* shell_prim_index, int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_shell_factor_device(qmckl_context_device context, double* shell_factor,
                                                              int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_exponent_device(qmckl_context_device context, double* exponent,
                                                          int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_coefficient_device(qmckl_context_device context, double* coefficient,
                                                             int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_prim_factor_device(qmckl_context_device context, double* prim_factor,
                                                             int64_t size_max);
qmckl_exit_code_device qmckl_set_ao_basis_ao_factor_device(qmckl_context_device context, double* ao_factor,
                                                           int64_t size_max);
/* Getters, src/qmckl_ao.cpp:1238-1765 */
qmckl_exit_code_device qmckl_get_ao_basis_type_device(qmckl_context_device context, char* const basis_type);
qmckl_exit_code_device qmckl_get_ao_basis_shell_num_device(qmckl_context_device context, int64_t* const shell_num);
qmckl_exit_code_device qmckl_get_ao_basis_prim_num_device(qmckl_context_device context, int64_t* prim_num);
qmckl_exit_code_device qmckl_get_ao_basis_ao_num_device(qmckl_context_device context, int64_t* ao_num);
qmckl_exit_code_device qmckl_get_ao_basis_nucleus_shell_num_device(qmckl_context_device context,
                                                                   int64_t* nucleus_shell_num, int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_nucleus_index_device(qmckl_context_device context, int64_t* nucleus_index,
                                                               int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_shell_ang_mom_device(qmckl_context_device context, int32_t* shell_ang_mom,
                                                               int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_shell_factor_device(qmckl_context_device context, double* shell_factor,
                                                              int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_shell_prim_num_device(qmckl_context_device context,
                                                                int64_t* shell_prim_num, int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_shell_prim_index_device(qmckl_context_device context,
                                                                  int64_t* shell_prim_index, int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_exponent_device(qmckl_context_device context, double* exponent,
                                                          int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_coefficient_device(qmckl_context_device context, double* coefficient,
                                                             int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_prim_factor_device(qmckl_context_device context, double* prim_factor,
                                                             int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_ao_factor_device(qmckl_context_device context, double* ao_factor,
                                                           int64_t size_max);
/* Derived tables of the finalize step, src/qmckl_ao_sycl.cpp:1087-1231 */
qmckl_exit_code_device qmckl_get_ao_basis_nucleus_range_device(qmckl_context_device context, double* nucleus_range,
                                                               int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_nucleus_max_ang_mom_device(qmckl_context_device context,
                                                                     int32_t* nucleus_max_ang_mom, int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_coefficient_normalized_device(qmckl_context_device context,
                                                                        double* coefficient_normalized,
                                                                        int64_t size_max);
/* The finalize steps, run by the last setter of each basis; callable directly as in the
 * reference (include/qmckl_gpu.hpp:651,654,796). The AO finalize ends with the per-nucleus
 * exponent tables, as the reference's does (src/qmckl_ao_sycl.cpp:1233). */
qmckl_exit_code_device qmckl_finalize_ao_basis_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_finalize_mo_basis_device(qmckl_context_device context);
/* Per-nucleus exponent tables, src/qmckl_ao_sycl.cpp:855-1065 (the reference keeps them in
 * ctx->ao_basis.{prim_num_per_nucleus, expo_per_nucleus, coef_per_nucleus}, include/
 * qmckl_gpu.hpp:294-296; the getters below stand in for reading that struct): each nucleus'
 * primitives sorted by exponent, equal exponents merged with their coefficients summed per
 * shell. prim_num_per_nucleus [nucl_num] = entries per nucleus; expo_per_nucleus
 * [nucl_num][prim_max]; coef_per_nucleus [nucl_num][shell_max][prim_max], zero where unused;
 * prim_max = the largest primitive count of a nucleus, shell_max = the largest shell count. */
qmckl_exit_code_device qmckl_finalize_ao_basis_hpc_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_get_ao_basis_hpc_dims_device(qmckl_context_device context, int64_t* prim_max,
                                                          int64_t* shell_max);
qmckl_exit_code_device qmckl_get_ao_basis_prim_num_per_nucleus_device(qmckl_context_device context,
                                                                      int32_t* prim_num_per_nucleus, int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_expo_per_nucleus_device(qmckl_context_device context,
                                                                  double* expo_per_nucleus, int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_coef_per_nucleus_device(qmckl_context_device context,
                                                                  double* coef_per_nucleus, int64_t size_max);
/* Provides (lazy, date-stamped), src/qmckl_ao.cpp:47-199, src/qmckl_ao_sycl.cpp:748-849 */
qmckl_exit_code_device qmckl_provide_ao_basis_shell_vgl_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_provide_ao_basis_ao_vgl_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_provide_ao_basis_ao_value_device(qmckl_context_device context);
/* Results, src/qmckl_ao.cpp:207-396 */
qmckl_exit_code_device qmckl_get_ao_basis_shell_vgl_device(qmckl_context_device context, double* const shell_vgl,
                                                           const int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_ao_vgl_device(qmckl_context_device context, double* const ao_vgl,
                                                        const int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_ao_vgl_inplace_device(qmckl_context_device context, double* const ao_vgl,
                                                                const int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_ao_value_device(qmckl_context_device context, double* const ao_value,
                                                          const int64_t size_max);
qmckl_exit_code_device qmckl_get_ao_basis_ao_value_inplace_device(qmckl_context_device context,
                                                                  double* const ao_value, const int64_t size_max);

/* ---- MO basis (reference: src/qmckl_mo.cpp, src/qmckl_mo_sycl.cpp) ---- */
bool qmckl_mo_basis_provided_device(qmckl_context_device context); /* src/qmckl_mo.cpp:10-23 */
qmckl_exit_code_device qmckl_get_mo_basis_mo_num_device(qmckl_context_device context, int64_t* mo_num);
/* src/qmckl_mo.cpp:487-524 and :527-583: QMCKL_ALREADY_SET_DEVICE on a second call.
 * coefficient is [mo_num][ao_num]. */
qmckl_exit_code_device qmckl_set_mo_basis_mo_num_device(qmckl_context_device context, int64_t mo_num);
qmckl_exit_code_device qmckl_set_mo_basis_coefficient_device(qmckl_context_device context, double* coefficient);
/* src/qmckl_mo.cpp:31-106: keep[] is a HOST array of mo_num flags */
bool qmckl_mo_basis_select_mo_device(qmckl_context_device context, int32_t* keep, int64_t size_max);
qmckl_exit_code_device qmckl_provide_mo_basis_mo_vgl_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_provide_mo_basis_mo_value_device(qmckl_context_device context);
/* src/qmckl_mo.cpp:294-453 */
qmckl_exit_code_device qmckl_get_mo_basis_mo_vgl_device(qmckl_context_device context, double* const mo_vgl,
                                                        const int64_t size_max);
qmckl_exit_code_device qmckl_get_mo_basis_mo_vgl_inplace_device(qmckl_context_device context, double* const mo_vgl,
                                                                const int64_t size_max);
qmckl_exit_code_device qmckl_get_mo_basis_mo_value_device(qmckl_context_device context, double* const mo_value,
                                                          const int64_t size_max);
qmckl_exit_code_device qmckl_get_mo_basis_mo_value_inplace_device(qmckl_context_device context,
                                                                  double* const mo_value, const int64_t size_max);

/* ======================================================================================
 * GB300 extensions (no counterpart in the reference; the reference behaviour is the
 * default of each).
 * ====================================================================================== */

/* MO contraction precision. FP64 (default, the drop-in) or a split-BF16 product on the
 * tcgen05 tensor cores (each operand split into three BF16 terms, six cross products, FP32
 * accumulation with per-block two-sum folding). The displacements, r2 and the screening
 * decisions are FP64 in both modes; in the split-BF16 mode the AO operand carries 24
 * significant bits, so its primitives and radial sums run in FP32 pair arithmetic (about 44
 * bits, within 2e-10 relative of the exact primitive values) and its AO components are
 * assembled in FP32, while the reference's zero-value skip keeps its FP64 decisions. A basis
 * with a coefficient beyond 2^+-64 or an exponent beyond 2^+-60 takes the FP64 radials in that
 * mode too. The AO getters always return the FP64 AOs. Changing the mode touches the context. */
#define QMCKL_PRECISION_FP64_DEVICE 0
#define QMCKL_PRECISION_SPLIT_BF16_DEVICE 1
qmckl_exit_code_device qmckl_set_precision_mode_device(qmckl_context_device context, int32_t mode);
qmckl_exit_code_device qmckl_get_precision_mode_device(qmckl_context_device context, int32_t* mode);

/* Shared exponentials of the fused AO kernels. Contracted bases repeat exponents among the
 * shells of a nucleus (CHBrClF: 297 primitives, 133 distinct exponents per nucleus); with
 * sharing on, the kernels evaluate each distinct exponential once per point and nucleus and
 * the shells' primitives multiply it by their coefficients. AUTO (default) shares for the
 * FP64 AO outputs when the distinct exponents carry at most half of the primitives' active
 * volume (sum of a^-1.5; generally contracted bases), and not for the split-BF16 planes; ON
 * shares for both; at most 64 distinct exponents per nucleus are supported (off beyond). The
 * FP64 results are bit-identical either way; in the split-BF16 mode the radials are rounded
 * differently (well inside the mode's tolerance). The get function reports whether the current
 * basis shares in the current precision mode (needs a finalized AO basis). */
#define QMCKL_SHARED_EXP_AUTO_DEVICE (-1)
#define QMCKL_SHARED_EXP_OFF_DEVICE 0
#define QMCKL_SHARED_EXP_ON_DEVICE 1
qmckl_exit_code_device qmckl_set_ao_shared_exponentials_device(qmckl_context_device context, int32_t mode);
qmckl_exit_code_device qmckl_get_ao_shared_exponentials_device(qmckl_context_device context, int32_t* active);

/* Asynchronous mode: when on, calls return after enqueueing their work on the
 * context's stream (no host wait). Off by default (the reference waits on every call). */
qmckl_exit_code_device qmckl_set_async_device(qmckl_context_device context, int32_t async);
/* The cudaStream_t the context issues its work on (as void*). */
void* qmckl_get_stream_device(qmckl_context_device context);
/* Waits for all work issued by the context. */
qmckl_exit_code_device qmckl_synchronize_device(qmckl_context_device context);

/* Kernel timing: when enabled, every kernel the context launches is bracketed by CUDA
 * events on its stream. qmckl_get_kernel_stats_device returns, for kernel slot `which`,
 * its name, launch count and total milliseconds (completed work only). */
qmckl_exit_code_device qmckl_set_profiling_device(qmckl_context_device context, int32_t enable);
qmckl_exit_code_device qmckl_reset_kernel_stats_device(qmckl_context_device context);
int32_t qmckl_get_kernel_stats_device(qmckl_context_device context, int32_t which, char* name, int64_t name_size,
                                      int64_t* launches, double* total_ms);
/* Total number of kernels the context has launched since creation or the last reset. */
int64_t qmckl_get_launch_count_device(qmckl_context_device context);

/* Device-side timing of the work issued on the context's stream: start records a CUDA
 * event on the stream; stop records a second one, waits for it and returns the elapsed
 * milliseconds. */
qmckl_exit_code_device qmckl_timer_start_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_timer_stop_device(qmckl_context_device context, double* elapsed_ms);

/* Page-locks (or releases) a caller's host buffer so that transfers to and from it run
 * at full link speed and kernels may read it directly. */
qmckl_exit_code_device qmckl_host_register_device(qmckl_context_device context, void* ptr, size_t size);
qmckl_exit_code_device qmckl_host_unregister_device(qmckl_context_device context, void* ptr);

/* Measures the FP64 tensor-pipe (DMMA) throughput of the context's GPU in TFLOP/s with a
 * register-resident mma loop over every SM (a roofline denominator for the FP64 form). */
qmckl_exit_code_device qmckl_measure_fp64_peak_device(qmckl_context_device context, double* tflops);

/* Validation of the exponential the fused AO kernel evaluates (a table-driven method for
 * arguments in the screened range): for device arrays x[n] with 0 <= x[i] <= 27.7, writes
 * out[2i] = the kernel's e^-x[i] and out[2i+1] = CUDA's exp(-x[i]). Needs a finalized AO
 * basis (QMCKL_NOT_PROVIDED_DEVICE otherwise). */
qmckl_exit_code_device qmckl_exp_check_device(qmckl_context_device context, const double* x, int64_t n, double* out);

/* Validation of the primitive values the split-BF16 form's AO kernel computes: for a device
 * array r2[n] of squared distances, writes out[i][k] = coefficient_normalized[k] *
 * e^(-exponent[k] r2[i]) as that kernel evaluates it, or 0 where the primitive is screened
 * (exponent[k] r2[i] > 27.631021115928547), for every primitive k < prim_num (out: device,
 * n * prim_num doubles). Needs a finalized AO basis (QMCKL_NOT_PROVIDED_DEVICE otherwise). */
qmckl_exit_code_device qmckl_prim_value_check_device(qmckl_context_device context, const double* r2, int64_t n,
                                                     double* out, int64_t size_max);

/* Split-BF16 MO contraction that allocates nothing (no counterpart in the reference).
 *
 *   out[r][m] = sum_k ao[r][k] * coefficient[m][k]      (r < rows, m < mo_num)
 *
 * with the same split-BF16 tensor-core product as QMCKL_PRECISION_SPLIT_BF16_DEVICE. It is
 * meant for callers that must not have device memory allocated behind their back: codes
 * whose own pool allocator owns the GPU's memory, hosts that load this library as a plug-in
 * and forbid it to allocate, and loops where a cudaMalloc/cudaFree would synchronise the
 * device. The caller passes every input and output (device pointers: ao [rows][ao_num] FP64,
 * coefficient [mo_num][ao_num] FP64 in the reference's layout, out [rows][mo_num] FP64); the
 * scratch space (BF16 operand planes) is a 28 MiB device array compiled into the library,
 * which every GPU that loads the library keeps until the process exits. No cudaMalloc,
 * cudaFree or other allocating routine is called.
 *
 * Limits set by that array: 1 <= ao_num <= 2048 (else QMCKL_INVALID_ARG_3_DEVICE) and
 * 1 <= mo_num <= 1024 (else QMCKL_INVALID_ARG_5_DEVICE); rows is unbounded (processed in
 * chunks). With vgl_mask = 1, rows are ao_vgl rows (5 per point: value, d/dx, d/dy, d/dz,
 * Laplacian; rows % 5 == 0 else QMCKL_INVALID_ARG_2_DEVICE) and an AO whose value is exactly
 * zero is dropped from that point's four derivative rows too, as the reference's MO kernel
 * does; with vgl_mask = 0 every row is used as is (ao_value rows). NULL pointers give
 * QMCKL_INVALID_ARG_1/4/7_DEVICE. Work is issued on cuda_stream (a cudaStream_t; NULL for the
 * legacy default stream) and the call waits for it; a pipeline stall in the kernel returns
 * QMCKL_FAILURE_DEVICE.
 *
 * The first call on a device resolves the array's device address for that device (with that
 * device current); make that first call before any stream capture. Every call waits for
 * cuda_stream before it returns (it reads the kernel's error word on the host). All calls share
 * the one array, so calls whose work overlaps on the GPU (different streams, or concurrent host
 * threads) race on it: serialise them. */
qmckl_exit_code_device qmckl_mo_contract_split_bf16_noalloc_device(const double* ao, int64_t rows, int64_t ao_num,
                                                                   const double* coefficient, int64_t mo_num,
                                                                   int32_t vgl_mask, double* out, void* cuda_stream);

/* ---- Electron-nucleus and electron-electron distances ---------------------------------------
 * src/qmckl_electron.cpp:192-552 of the reference (include/qmckl_electron.hpp:30-41,
 * include/qmckl_gpu.hpp:1043-1046). C[i + j*ldc] = |A_i - B_j| for i < m, j < n, where point i of A
 * is (A[0 + i*lda], A[1 + i*lda], A[2 + i*lda]) for transa 'N' and (A[i], A[i + lda], A[i + 2*lda])
 * for 'T' (same for B with ldb); device pointers. The reference's kernel takes square roots of whole
 * columns from every work-item (src/qmckl_electron.cpp:504-546); this one computes each entry once:
 * sqrt((x*x + y*y) + z*z) rounded like the reference's host arithmetic. Argument checks as the
 * reference's (bad trans: ARG_1; m, n <= 0: ARG_4/5; lda, ldb, ldc too small: ARG_7/9/11), with lda
 * checked against transa and ldb against transb. */
qmckl_exit_code_device qmckl_distance_device(const qmckl_context_device context, const char transa, const char transb,
                                             const int64_t m, const int64_t n, const double* A, const int64_t lda,
                                             const double* B, const int64_t ldb, double* const C, const int64_t ldc);
/* en_distance[point][nucl] from coord [3][point_num] and nucl_coord [3][nucl_num]. */
qmckl_exit_code_device qmckl_compute_en_distance_device(const qmckl_context_device context, const int64_t point_num,
                                                        const int64_t nucl_num, const double* elec_coord,
                                                        const double* nucl_coord, double* const en_distance);
/* ee_distance[walker][j][i] for the elec_num electrons of each of the walk_num walkers; coord is the
 * points array [3][walk_num * elec_num]. */
qmckl_exit_code_device qmckl_compute_ee_distance_device(const qmckl_context_device context, const int64_t elec_num,
                                                        const int64_t walk_num, const double* coord,
                                                        double* const ee_distance);
/* Date-cached providers (recomputed when the points changed). */
qmckl_exit_code_device qmckl_provide_en_distance_device(qmckl_context_device context);
qmckl_exit_code_device qmckl_provide_ee_distance_device(qmckl_context_device context);
/* Getters (no counterpart in the reference, whose cached arrays are read only by its Jastrow code):
 * copy the cached en_distance [point_num][nucl_num] / ee_distance [walk_num][elec_num][elec_num] to
 * `distance` (device or host); size_max too small gives QMCKL_INVALID_ARG_3_DEVICE. */
qmckl_exit_code_device qmckl_get_electron_en_distance_device(qmckl_context_device context, double* distance,
                                                             int64_t size_max);
qmckl_exit_code_device qmckl_get_electron_ee_distance_device(qmckl_context_device context, double* distance,
                                                             int64_t size_max);

/* ---- Batched form: many molecules of uneven size evaluated together ----------------------
 *
 * A batch groups member contexts (each set up with the usual calls: nucleus, AO basis, MO
 * basis, points) on one GPU. qmckl_batch_provide_mo_vgl_device computes the MO vgl of every
 * member whose points changed since its last evaluation, with one persistent kernel per stage
 * covering all members (point ordering, fused AO kernel, MO contraction), the stages captured
 * once as a CUDA graph and replayed on later calls. Results land in the members' own caches:
 * qmckl_get_mo_basis_mo_vgl_device(member, ...) then returns them without recomputation (and,
 * in FP64 mode, qmckl_get_ao_basis_ao_vgl_device too). The batch's precision mode applies to
 * the results of all its members. Errors are recorded in the first member's error slot.
 * Destroy a batch before its members. No counterpart in the reference, whose API evaluates
 * one context per call. */
typedef int64_t qmckl_batch_device;
#define QMCKL_NULL_BATCH_DEVICE ((qmckl_batch_device)0)
/* members: member_num distinct valid contexts on the same device; QMCKL_NULL_BATCH_DEVICE on
 * invalid arguments. */
qmckl_batch_device qmckl_batch_create_device(const qmckl_context_device* members, int64_t member_num);
qmckl_exit_code_device qmckl_batch_destroy_device(qmckl_batch_device batch);
qmckl_exit_code_device qmckl_batch_set_precision_mode_device(qmckl_batch_device batch, int32_t mode);
/* enable = 0 issues the stages as ordinary launches (per-kernel profiling of the first member
 * applies then); 1 (default) replays a captured CUDA graph. */
qmckl_exit_code_device qmckl_batch_set_graph_device(qmckl_batch_device batch, int32_t enable);
/* async = 1: provide returns once the work is enqueued on the first member's stream; call
 * qmckl_batch_synchronize_device before reading member results. */
qmckl_exit_code_device qmckl_batch_set_async_device(qmckl_batch_device batch, int32_t async);
qmckl_exit_code_device qmckl_batch_synchronize_device(qmckl_batch_device batch);
qmckl_exit_code_device qmckl_batch_provide_mo_vgl_device(qmckl_batch_device batch);
/* Touches every member (the next provide recomputes all of them). */
qmckl_exit_code_device qmckl_batch_touch_device(qmckl_batch_device batch);
/* Launch parameters, chosen by the built-in autotuner on the first provide of each batch shape
 * (timed candidates; results cached per shape in the process and, when the environment
 * variable QMCKL_GB300_TUNE_CACHE names a file, in that file):
 *   params[0] nucleus-chunk level of the AO kernel's warp tasks (0 = whole molecule, v ~ 2^v chunks)
 *   params[1] FP64 contraction CTA tile: 0 = 64x64, 1 = 128x64, 2 = 64x128
 *   params[2] split-BF16 contraction: widest column tile (16..160, multiple of 16)
 * set pins the parameters (n = 3; no autotuning afterwards); get reads them (-1 = not chosen yet);
 * autotune re-times the candidates now (members must be ready to provide). */
qmckl_exit_code_device qmckl_batch_set_tuning_device(qmckl_batch_device batch, const int32_t* params, int64_t n);
qmckl_exit_code_device qmckl_batch_get_tuning_device(qmckl_batch_device batch, int32_t* params, int64_t n);
qmckl_exit_code_device qmckl_batch_autotune_device(qmckl_batch_device batch);
/* Kernels launched by one provide (all stages). */
int64_t qmckl_batch_get_launch_count_device(qmckl_batch_device batch);

/* ---- Adjoint form: vector-Jacobian products (no counterpart in the reference) -------------
 *
 * For the scalar L = sum_{p,l,m} w[p][l][m] * mo_vgl[p][l][m] of the current points,
 * qmckl_vjp_mo_vgl_device writes
 *   d_coefficient [mo_num][ao_num]  dL/dC, in the layout of qmckl_set_mo_basis_coefficient_device
 *   d_exponent    [prim_num]        dL/d(primitive exponent), the user's primitive order
 *   d_coord       [point_num][3]    dL/d(point coordinates), the 'N' layout of qmckl_set_point_device
 * (any of them may be NULL: not computed). w is [point_num][5][mo_num] (the mo_vgl layout).
 * Computed in FP64 whatever the precision mode, with the shell radials recomputed (nothing is
 * stored between forward and adjoint). The MO kernel's zero-value skip is a constant mask: an AO
 * whose value is exactly zero at a point passes no gradient there; screening decisions are
 * constants. Pointers may be device or host memory. Results are deterministic (fixed-order
 * reductions). Sizes too small give QMCKL_INVALID_ARG_3/5/7/9_DEVICE, a NULL w
 * QMCKL_INVALID_ARG_2_DEVICE.
 *
 * qmckl_vjp_ao_vgl_device is the same for L = sum ao_vgl_bar[p][l][k] * ao_vgl[p][l][k]
 * (ao_vgl_bar [point_num][5][ao_num]; no mask): exponent and coordinate gradients. */
qmckl_exit_code_device qmckl_vjp_mo_vgl_device(qmckl_context_device context, const double* w, int64_t w_size,
                                               double* d_coefficient, int64_t d_coefficient_size, double* d_exponent,
                                               int64_t d_exponent_size, double* d_coord, int64_t d_coord_size);
qmckl_exit_code_device qmckl_vjp_ao_vgl_device(qmckl_context_device context, const double* ao_vgl_bar,
                                               int64_t ao_vgl_bar_size, double* d_exponent, int64_t d_exponent_size,
                                               double* d_coord, int64_t d_coord_size);

/* Test hook for allocation failure handling: the n-th device allocation from now on
 * (n >= 1) fails as if cudaMalloc had failed; n = 0 disables the hook. */
qmckl_exit_code_device qmckl_set_allocation_failure_device(qmckl_context_device context, int64_t n);

/* Test hook for the device-side failure path of the split-BF16 contraction (no counterpart in the
 * reference, whose only failure handling is error codes, src/qmckl_basic_functions.cpp:51): every
 * mbarrier wait of that kernel gives up after wait_cycles clock cycles (0 restores the default,
 * about one second), and with withhold_loads = 1 its producer issues no operand loads, so the first
 * wait of its consumers is one that nothing completes. On expiry the kernel records an error word,
 * releases its tensor memory and exits; the call returns QMCKL_FAILURE_DEVICE and the context
 * stays usable. Bad wait_cycles (< 0): QMCKL_INVALID_ARG_2_DEVICE; withhold_loads not 0 or 1:
 * QMCKL_INVALID_ARG_3_DEVICE. */
qmckl_exit_code_device qmckl_set_split_wait_test_device(qmckl_context_device context, int64_t wait_cycles,
                                                        int32_t withhold_loads);

/* Debug build with bounds checks (no counterpart in the reference). The library built with
 * -DQMCKL_BOUNDS_CHECK (python -m qmckl_sycl_gb300.build --bounds: _lib/libqmckl_gpu_bounds.so)
 * tests the element index of the kernels' global stores against the extent of the array they
 * write; an out-of-range store is skipped and the first one recorded. This returns 1 and fills
 * site (the store site: 1 AO rows, 2 AO planes, 3 shell_vgl, 4 point order, 5 split-BF16 output,
 * 6 split planes, 7 FP64 contraction output, 8 split-K sums, 9 distances, 10 transposes and
 * copies, 11 adjoint), index and extent (elements) when a store was out of range on the current
 * device, 0 when none was, -1 for the normal build (no checks) and -2 on a CUDA error; reset = 1
 * clears the records. It waits for all work on the current device first. Any pointer may be
 * NULL. */
int32_t qmckl_bounds_check_status_device(int32_t reset, int64_t* site, int64_t* index, int64_t* extent);
/* Self-test of that recording: a one-thread kernel evaluates the check for element `index` of an
 * array of `extent` elements (site 10) and stores nothing. Returns 0 when it ran, -1 for the normal
 * build, -2 on a CUDA error. */
int32_t qmckl_bounds_check_selftest_device(int64_t index, int64_t extent);

/* ---- TREXIO reader (reference: src/qmckl_trexio.cpp, include/qmckl_trexio.hpp) ----
 * Fills a context from a TREXIO file through the setters above. libtrexio is bound at run time
 * (dlopen of $QMCKL_TREXIO_LIBRARY, else libtrexio.so, else libtrexio.so.2), so this library links
 * and loads without it; where it cannot be loaded these calls return QMCKL_FAILURE_DEVICE (open:
 * NULL) with the loader's message. trexio_t is libtrexio's opaque file handle. The shells of one
 * nucleus and the primitives of one shell must be contiguous in the file (else QMCKL_FAILURE_DEVICE,
 * "Irrelevant data in TREXIO file"; the reference accepts such files and mis-assigns them). */
typedef struct trexio_s trexio_t;
/* src/qmckl_trexio.cpp:937-958: opens file_name read-only with the text back end, else HDF5; NULL
 * and *rc = QMCKL_FAILURE_DEVICE when neither opens. Close the handle with libtrexio's trexio_close. */
trexio_t* qmckl_trexio_open_X_device(char* file_name, qmckl_exit_code_device* rc);
/* src/qmckl_trexio.cpp:7-41: electron.up_num and dn_num -> qmckl_set_electron_num_device */
qmckl_exit_code_device qmckl_trexio_read_electron_X_device(qmckl_context_device context, trexio_t* file);
/* src/qmckl_trexio.cpp:43-141: nucleus.num, charge and coord ([nucleus][3], set with 'N') */
qmckl_exit_code_device qmckl_trexio_read_nucleus_X_device(qmckl_context_device context, trexio_t* file);
/* src/qmckl_trexio.cpp:143-866: the basis (Gaussian only: "Invalid basis type" otherwise) and
 * ao.num/normalization; the nucleus of each shell and the shell of each primitive become each
 * nucleus's first shell and shell count and each shell's first primitive and primitive count.
 * Needs the nucleus number set. */
qmckl_exit_code_device qmckl_trexio_read_ao_X_device(qmckl_context_device context, trexio_t* file);
/* src/qmckl_trexio.cpp:868-935: mo.num and mo.coefficient ([mo][ao], read size-checked as
 * ao_num * mo_num values). Needs ao_num set. */
qmckl_exit_code_device qmckl_trexio_read_mo_X_device(qmckl_context_device context, trexio_t* file);
/* src/qmckl_trexio.cpp:960-1021: all four, in that order, from the file named by the first
 * size_max characters of file_name. A file that opens with neither back end:
 * QMCKL_INVALID_ARG_2_DEVICE; a failing group: QMCKL_FAILURE_DEVICE ("Error reading electron",
 * "... nucleus", "... AOs", "... MOs"). NULL context: QMCKL_INVALID_CONTEXT_DEVICE (the reference
 * returns 0). */
qmckl_exit_code_device qmckl_trexio_read_device(qmckl_context_device context, char* file_name, int64_t size_max);

/* Library build information: "sm_103a" plus the git-independent build flags. */
const char* qmckl_gb300_build_info(void);

#ifdef __cplusplus
}
#endif

#endif /* QMCKL_GPU_H */
