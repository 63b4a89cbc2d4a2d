// Split-BF16 MO contraction on the tcgen05 tensor cores (precision form).
#include "internal.hpp"

namespace qg {

qmckl_exit_code_device provide_mo_split(Ctx* ctx, qmckl_context_device c, double* dst, bool value_only) {
  (void)ctx;
  (void)dst;
  (void)value_only;
  return fail(c, QMCKL_FAILURE_DEVICE, "qmckl_provide_mo_basis_mo_vgl_device", "split-BF16 form not available");
}

}  // namespace qg
