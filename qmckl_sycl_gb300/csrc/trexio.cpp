// TREXIO reader: fills a context from a TREXIO file through the context's own setters
// (reference: src/qmckl_trexio.cpp, include/qmckl_trexio.hpp of qmckl_sycl).
//
// libtrexio is bound at run time with dlopen ($QMCKL_TREXIO_LIBRARY, else libtrexio.so, else
// libtrexio.so.2), so the library builds and loads where libtrexio is absent; the calls then fail
// with QMCKL_FAILURE_DEVICE and the loader's message. Every array is read into host memory with
// TREXIO's size-checked ("safe") reads and handed to the setters, which copy host memory like
// device memory, so nothing is staged on the device here.
//
// The conversions follow the reference: TREXIO keeps the nucleus of every shell and the shell of
// every primitive; the context keeps, per nucleus, its first shell and shell count and, per shell,
// its first primitive and primitive count (src/qmckl_trexio.cpp:229-420 and :460-640). Differences,
// each deliberate:
// - the members of one owner (the shells of a nucleus, the primitives of a shell) must be
//   contiguous, or the file is refused as "Irrelevant data in TREXIO file"; the reference accepts
//   such a file and builds a basis whose (first, count) pairs cover other owners' members;
// - an owner without members gets first = 0 (the reference leaves the entry uninitialised);
// - the MO coefficients are read with the size-checked read of ao_num * mo_num values (the
//   reference's unchecked read, :910, writes whatever the file holds into a buffer of that size);
// - a NULL context gives QMCKL_INVALID_CONTEXT_DEVICE (the reference returns `false`, i.e. 0,
//   :962-965) and a NULL file handle QMCKL_INVALID_ARG_2_DEVICE (the reference asserts).
#include <dlfcn.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "internal.hpp"

using namespace qg;

namespace {

// TREXIO's C API as the reference calls it: exit codes are int32 with 0 for success, back ends
// int32 (0 HDF5, 1 text), files opened with mode 'r'.
using trexio_exit_code = int32_t;
constexpr trexio_exit_code kTrexioSuccess = 0;
constexpr int32_t kBackEndHdf5 = 0;
constexpr int32_t kBackEndText = 1;

using NumFn = trexio_exit_code (*)(trexio_t*, int64_t*);
using F64Fn = trexio_exit_code (*)(trexio_t*, double*, int64_t);
using I64Fn = trexio_exit_code (*)(trexio_t*, int64_t*, int64_t);
using I32Fn = trexio_exit_code (*)(trexio_t*, int32_t*, int64_t);

struct TrexioApi {
  trexio_t* (*open)(const char*, char, int32_t, trexio_exit_code*);
  trexio_exit_code (*close)(trexio_t*);
  const char* (*string_of_error)(trexio_exit_code);
  trexio_exit_code (*basis_type)(trexio_t*, char*, int32_t);
  NumFn up_num, dn_num, nucleus_num, shell_num, prim_num, ao_num, mo_num;
  F64Fn nucleus_charge, nucleus_coord, shell_factor, exponent, coefficient, prim_factor, ao_normalization,
      mo_coefficient;
  I64Fn nucleus_index, shell_index;
  I32Fn shell_ang_mom;
};

struct Loaded {
  std::string name;  // what was passed to dlopen
  TrexioApi api;
};

// Resolves TrexioApi from one shared object; false (and *why) when it or a symbol is missing.
bool resolve(const char* so, TrexioApi* api, std::string* why) {
  void* h = dlopen(so, RTLD_NOW | RTLD_GLOBAL);
  if (!h) {
    const char* e = dlerror();
    *why = e ? e : so;
    return false;
  }
  struct Sym {
    const char* name;
    void** slot;
  } syms[] = {
      {"trexio_open", reinterpret_cast<void**>(&api->open)},
      {"trexio_close", reinterpret_cast<void**>(&api->close)},
      {"trexio_string_of_error", reinterpret_cast<void**>(&api->string_of_error)},
      {"trexio_read_basis_type", reinterpret_cast<void**>(&api->basis_type)},
      {"trexio_read_electron_up_num_64", reinterpret_cast<void**>(&api->up_num)},
      {"trexio_read_electron_dn_num_64", reinterpret_cast<void**>(&api->dn_num)},
      {"trexio_read_nucleus_num_64", reinterpret_cast<void**>(&api->nucleus_num)},
      {"trexio_read_basis_shell_num_64", reinterpret_cast<void**>(&api->shell_num)},
      {"trexio_read_basis_prim_num_64", reinterpret_cast<void**>(&api->prim_num)},
      {"trexio_read_ao_num_64", reinterpret_cast<void**>(&api->ao_num)},
      {"trexio_read_mo_num_64", reinterpret_cast<void**>(&api->mo_num)},
      {"trexio_read_safe_nucleus_charge_64", reinterpret_cast<void**>(&api->nucleus_charge)},
      {"trexio_read_safe_nucleus_coord_64", reinterpret_cast<void**>(&api->nucleus_coord)},
      {"trexio_read_safe_basis_shell_factor_64", reinterpret_cast<void**>(&api->shell_factor)},
      {"trexio_read_safe_basis_exponent_64", reinterpret_cast<void**>(&api->exponent)},
      {"trexio_read_safe_basis_coefficient_64", reinterpret_cast<void**>(&api->coefficient)},
      {"trexio_read_safe_basis_prim_factor_64", reinterpret_cast<void**>(&api->prim_factor)},
      {"trexio_read_safe_ao_normalization_64", reinterpret_cast<void**>(&api->ao_normalization)},
      {"trexio_read_safe_mo_coefficient_64", reinterpret_cast<void**>(&api->mo_coefficient)},
      {"trexio_read_safe_basis_nucleus_index_64", reinterpret_cast<void**>(&api->nucleus_index)},
      {"trexio_read_safe_basis_shell_index_64", reinterpret_cast<void**>(&api->shell_index)},
      {"trexio_read_safe_basis_shell_ang_mom_32", reinterpret_cast<void**>(&api->shell_ang_mom)},
  };
  for (const Sym& s : syms) {
    *s.slot = dlsym(h, s.name);
    if (!*s.slot) {
      *why = std::string(so) + " has no " + s.name;
      dlclose(h);
      return false;
    }
  }
  return true;  // the handle stays open: file handles it returns may outlive this call
}

// The bound API, or nullptr with *why. A successful binding is kept per library name (handles
// are never closed); a failed one is retried on the next call, so QMCKL_TREXIO_LIBRARY may be set
// after a first attempt.
const TrexioApi* trexio_api(std::string* why) {
  static std::mutex mutex;
  static std::vector<std::unique_ptr<Loaded>> loaded;
  std::lock_guard<std::mutex> lock(mutex);
  const char* env = std::getenv("QMCKL_TREXIO_LIBRARY");
  std::vector<std::string> names;
  if (env && *env)
    names.push_back(env);
  else
    names = {"libtrexio.so", "libtrexio.so.2"};
  for (const std::string& n : names)
    for (const auto& l : loaded)
      if (l->name == n) return &l->api;
  std::string last;
  for (const std::string& n : names) {
    auto l = std::make_unique<Loaded>();
    l->name = n;
    if (resolve(n.c_str(), &l->api, &last)) {
      loaded.push_back(std::move(l));
      return &loaded.back()->api;
    }
  }
  *why = "libtrexio could not be loaded: " + last;
  return nullptr;
}

// Valid context and bound API, or an error recorded under fn.
qmckl_exit_code_device prologue(qmckl_context_device context, trexio_t* file, const char* fn,
                                const TrexioApi** api) {
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!file) return fail(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL file handle");
  std::string why;
  *api = trexio_api(&why);
  if (!*api) return fail(context, QMCKL_FAILURE_DEVICE, fn, why.c_str());
  return QMCKL_SUCCESS_DEVICE;
}

qmckl_exit_code_device io_fail(qmckl_context_device context, const TrexioApi* api, const char* what,
                               trexio_exit_code rcio) {
  return fail(context, QMCKL_FAILURE_DEVICE, what, api->string_of_error(rcio));
}

// A zero-filled host array from calloc: an allocation that fails (a file that declares absurd
// sizes) leaves it empty and returns false instead of throwing across the C ABI.
template <class T>
struct Array {
  T* p = nullptr;
  Array() = default;
  Array(const Array&) = delete;
  Array& operator=(const Array&) = delete;
  ~Array() { free(p); }
  bool resize(int64_t n) {
    free(p);
    p = nullptr;
    if (n < 0 || (uint64_t)n > (uint64_t)(PTRDIFF_MAX / sizeof(T))) return false;
    p = static_cast<T*>(calloc(n > 0 ? (size_t)n : 1, sizeof(T)));
    return p != nullptr;
  }
  T* data() { return p; }
  T& operator[](int64_t i) { return p[i]; }
  const T& operator[](int64_t i) const { return p[i]; }
};

// Inverts a member -> owner map (TREXIO's basis.nucleus_index per shell, basis.shell_index per
// primitive) into each owner's first member and member count. Fails when an owner is out of
// [0, owner_num) or its members are not contiguous.
bool group_members(const Array<int64_t>& owner, int64_t member_num, int64_t owner_num, Array<int64_t>* first,
                   Array<int64_t>* count) {
  for (int64_t k = 0; k < owner_num; ++k) (*first)[k] = (*count)[k] = 0;
  for (int64_t i = 0; i < member_num; ++i) {
    const int64_t k = owner[i];
    if (k < 0 || k >= owner_num) return false;
    if ((*count)[k] == 0) {
      (*first)[k] = i;
    } else if (owner[i - 1] != k) {
      return false;  // k's members resume after another owner's
    }
    (*count)[k] += 1;
  }
  return true;
}

}  // namespace

extern "C" {

// src/qmckl_trexio.cpp:7-41
qmckl_exit_code_device qmckl_trexio_read_electron_X_device(qmckl_context_device context, trexio_t* file) {
  QG_NVTX_RANGE("qmckl_trexio_read_electron_X_device");
  const TrexioApi* api = nullptr;
  qmckl_exit_code_device rc = prologue(context, file, "qmckl_trexio_read_electron_X_device", &api);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  int64_t up = 0, dn = 0;
  trexio_exit_code rcio = api->up_num(file, &up);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_electron_up_num", rcio);
  rcio = api->dn_num(file, &dn);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_electron_dn_num", rcio);
  return qmckl_set_electron_num_device(context, up, dn);
}

// src/qmckl_trexio.cpp:43-141
qmckl_exit_code_device qmckl_trexio_read_nucleus_X_device(qmckl_context_device context, trexio_t* file) {
  QG_NVTX_RANGE("qmckl_trexio_read_nucleus_X_device");
  const TrexioApi* api = nullptr;
  qmckl_exit_code_device rc = prologue(context, file, "qmckl_trexio_read_nucleus_X_device", &api);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  int64_t n = 0;
  trexio_exit_code rcio = api->nucleus_num(file, &n);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_nucleus_num", rcio);
  rc = qmckl_set_nucleus_num_device(context, n);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  Array<double> charge, coord;
  if (n > INT64_MAX / 3 || !charge.resize(n) || !coord.resize(3 * n))
    return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_trexio_read_nucleus_X_device", nullptr);
  rcio = api->nucleus_charge(file, charge.data(), n);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_nucleus_charge", rcio);
  rc = qmckl_set_nucleus_charge_device(context, charge.data(), n);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rcio = api->nucleus_coord(file, coord.data(), 3 * n);  // TREXIO's [nucleus][3]
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_nucleus_coord", rcio);
  return qmckl_set_nucleus_coord_device(context, 'N', coord.data(), 3 * n);
}

// src/qmckl_trexio.cpp:143-866
qmckl_exit_code_device qmckl_trexio_read_ao_X_device(qmckl_context_device context, trexio_t* file) {
  QG_NVTX_RANGE("qmckl_trexio_read_ao_X_device");
  const TrexioApi* api = nullptr;
  qmckl_exit_code_device rc = prologue(context, file, "qmckl_trexio_read_ao_X_device", &api);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  int64_t nucl_num = 0;
  rc = qmckl_get_nucleus_num_device(context, &nucl_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  char type[1024];  // the reference's MAX_STR_LEN
  trexio_exit_code rcio = api->basis_type(file, type, (int32_t)sizeof type);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_basis_type", rcio);
  if (type[0] != 'G') return fail(context, QMCKL_FAILURE_DEVICE, "trexio_read_basis_type", "Invalid basis type");
  rc = qmckl_set_ao_basis_type_device(context, 'G');
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  int64_t shell_num = 0, prim_num = 0, ao_num = 0;
  rcio = api->shell_num(file, &shell_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_basis_shell_num", rcio);
  rc = qmckl_set_ao_basis_shell_num_device(context, shell_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rcio = api->prim_num(file, &prim_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_basis_prim_num", rcio);
  rc = qmckl_set_ao_basis_prim_num_device(context, prim_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rcio = api->ao_num(file, &ao_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_ao_num", rcio);
  rc = qmckl_set_ao_basis_ao_num_device(context, ao_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  // shells per nucleus from the nucleus of each shell (:229-420)
  const char* fn = "qmckl_trexio_read_ao_X_device";
  Array<int64_t> owner, first, count;
  Array<int32_t> ang_mom;
  Array<double> values;
  if (!owner.resize(shell_num) || !first.resize(nucl_num) || !count.resize(nucl_num))
    return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  rcio = api->nucleus_index(file, owner.data(), shell_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_basis_nucleus_index", rcio);
  if (!group_members(owner, shell_num, nucl_num, &first, &count))
    return fail(context, QMCKL_FAILURE_DEVICE, "trexio_read_basis_nucleus_index", "Irrelevant data in TREXIO file");
  rc = qmckl_set_ao_basis_nucleus_index_device(context, first.data(), nucl_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rc = qmckl_set_ao_basis_nucleus_shell_num_device(context, count.data(), nucl_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  if (!ang_mom.resize(shell_num)) return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  rcio = api->shell_ang_mom(file, ang_mom.data(), shell_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_basis_shell_ang_mom", rcio);
  rc = qmckl_set_ao_basis_shell_ang_mom_device(context, ang_mom.data(), shell_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  // primitives per shell from the shell of each primitive (:460-640)
  if (!owner.resize(prim_num) || !first.resize(shell_num) || !count.resize(shell_num))
    return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
  rcio = api->shell_index(file, owner.data(), prim_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_basis_shell_prim_num", rcio);
  if (!group_members(owner, prim_num, shell_num, &first, &count))
    return fail(context, QMCKL_FAILURE_DEVICE, "trexio_read_basis_shell_prim_num", "Irrelevant data in TREXIO file");
  rc = qmckl_set_ao_basis_shell_prim_num_device(context, count.data(), shell_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  rc = qmckl_set_ao_basis_shell_prim_index_device(context, first.data(), shell_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;

  struct Dset {
    F64Fn read;
    int64_t num;
    qmckl_exit_code_device (*set)(qmckl_context_device, double*, int64_t);
    const char* what;
  } dsets[] = {
      {api->shell_factor, shell_num, qmckl_set_ao_basis_shell_factor_device, "trexio_read_basis_shell_factor"},
      {api->exponent, prim_num, qmckl_set_ao_basis_exponent_device, "trexio_read_basis_exponent"},
      {api->coefficient, prim_num, qmckl_set_ao_basis_coefficient_device, "trexio_read_basis_coefficient"},
      {api->prim_factor, prim_num, qmckl_set_ao_basis_prim_factor_device, "trexio_read_basis_prim_factor"},
      {api->ao_normalization, ao_num, qmckl_set_ao_basis_ao_factor_device, "trexio_read_ao_normalization"},
  };
  for (const Dset& d : dsets) {
    if (!values.resize(d.num)) return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, fn, nullptr);
    rcio = d.read(file, values.data(), d.num);
    if (rcio != kTrexioSuccess) return io_fail(context, api, d.what, rcio);
    rc = d.set(context, values.data(), d.num);
    if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  }
  return QMCKL_SUCCESS_DEVICE;
}

// src/qmckl_trexio.cpp:868-935
qmckl_exit_code_device qmckl_trexio_read_mo_X_device(qmckl_context_device context, trexio_t* file) {
  QG_NVTX_RANGE("qmckl_trexio_read_mo_X_device");
  const TrexioApi* api = nullptr;
  qmckl_exit_code_device rc = prologue(context, file, "qmckl_trexio_read_mo_X_device", &api);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  int64_t ao_num = 0, mo_num = 0;
  rc = qmckl_get_ao_basis_ao_num_device(context, &ao_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  trexio_exit_code rcio = api->mo_num(file, &mo_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_mo_num", rcio);
  rc = qmckl_set_mo_basis_mo_num_device(context, mo_num);
  if (rc != QMCKL_SUCCESS_DEVICE) return rc;
  Array<double> coef;  // TREXIO's [mo][ao]
  if (mo_num > INT64_MAX / ao_num || !coef.resize(ao_num * mo_num))
    return fail(context, QMCKL_ALLOCATION_FAILED_DEVICE, "qmckl_trexio_read_mo_X_device", nullptr);
  rcio = api->mo_coefficient(file, coef.data(), ao_num * mo_num);
  if (rcio != kTrexioSuccess) return io_fail(context, api, "trexio_read_mo_coefficient", rcio);
  return qmckl_set_mo_basis_coefficient_device(context, coef.data());
}

// src/qmckl_trexio.cpp:937-958: the text back end first, then HDF5.
trexio_t* qmckl_trexio_open_X_device(char* file_name, qmckl_exit_code_device* rc) {
  qmckl_exit_code_device dummy;
  if (!rc) rc = &dummy;
  *rc = QMCKL_SUCCESS_DEVICE;
  std::string why;
  const TrexioApi* api = trexio_api(&why);
  if (!api || !file_name) {
    *rc = QMCKL_FAILURE_DEVICE;
    return nullptr;
  }
  for (int32_t back_end : {kBackEndText, kBackEndHdf5}) {
    trexio_exit_code rcio = kTrexioSuccess;
    trexio_t* f = api->open(file_name, 'r', back_end, &rcio);
    if (f) return f;
  }
  *rc = QMCKL_FAILURE_DEVICE;
  return nullptr;
}

// src/qmckl_trexio.cpp:960-1021: electrons, nuclei, basis and AOs, MOs, in that order; file_name
// is read up to size_max characters.
qmckl_exit_code_device qmckl_trexio_read_device(qmckl_context_device context, char* file_name, int64_t size_max) {
  QG_NVTX_RANGE("qmckl_trexio_read_device");
  const char* fn = "qmckl_trexio_read_device";
  if (qmckl_context_check_device(context) == QMCKL_NULL_CONTEXT_DEVICE) return QMCKL_INVALID_CONTEXT_DEVICE;
  if (!file_name) return fail(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "NULL file name");
  if (size_max < 0) return fail(context, QMCKL_INVALID_ARG_3_DEVICE, fn, "size_max < 0");
  std::string why;
  const TrexioApi* api = trexio_api(&why);
  if (!api) return fail(context, QMCKL_FAILURE_DEVICE, fn, why.c_str());
  std::string name(file_name, strnlen(file_name, (size_t)size_max));
  qmckl_exit_code_device rc = QMCKL_SUCCESS_DEVICE;
  trexio_t* file = qmckl_trexio_open_X_device(&name[0], &rc);
  if (!file) return fail(context, QMCKL_INVALID_ARG_2_DEVICE, fn, "the file opens with neither back end");
  struct Step {
    qmckl_exit_code_device (*read)(qmckl_context_device, trexio_t*);
    const char* fn;
    const char* msg;
  } steps[] = {
      {qmckl_trexio_read_electron_X_device, fn, "Error reading electron"},
      {qmckl_trexio_read_nucleus_X_device, fn, "Error reading nucleus"},
      {qmckl_trexio_read_ao_X_device, fn, "Error reading AOs"},
      // the reference records this one under "qmckl_trexio_omp_read" (:1011-1016); kept for the
      // error record's sake
      {qmckl_trexio_read_mo_X_device, "qmckl_trexio_omp_read", "Error reading MOs"},
  };
  for (const Step& s : steps) {
    if (s.read(context, file) != QMCKL_SUCCESS_DEVICE) {
      api->close(file);
      return fail(context, QMCKL_FAILURE_DEVICE, s.fn, s.msg);
    }
  }
  api->close(file);
  return QMCKL_SUCCESS_DEVICE;
}

}  // extern "C"
