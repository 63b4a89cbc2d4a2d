"""Source compatibility with callers of the reference's SYCL interface: the queue-based context
idiom compiles and links against the C ABI through include/qmckl_gpu_sycl_compat.hpp, and so do
the reference's own test programs (tests/test_qmckl_{ao,mo}.cpp of qmckl_sycl, unmodified; built
by oracle/ref_tests_compile.sh where the reference checkout is present). Compile and link only:
running needs a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "qmckl_sycl_gb300", "_lib")

def _reference_dir():
    from oracle import oracle

    return oracle.reference_dir()

IDIOM = r'''
#include "qmckl_gpu_sycl_compat.hpp"
using namespace sycl;
int main() {
  queue q;
  try {
    q = queue(gpu_selector_v);
    std::cout << q.get_device().get_info<info::device::name>() << "\n";
  } catch (const sycl::exception&) {
    q = queue();
  }
  qmckl_context_device context = qmckl_context_create_device(q);
  double* d = (double*)qmckl_malloc_device(context, 8 * sizeof(double));
  double h[8] = {0};
  qmckl_memcpy_H2D(context, d, h, sizeof h);
  qmckl_exit_code_device rc = qmckl_set_nucleus_num_device(context, 1);
  qmckl_free_device(context, d);
  qmckl_context_destroy_device(context);
  return rc == QMCKL_SUCCESS_DEVICE ? 0 : 1;
}
'''


def _lib():
    from qmckl_sycl_gb300 import build

    build.build()
    return LIB_DIR


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_queue_idiom_compiles_and_links(tmp_path):
    lib = _lib()
    src = tmp_path / "idiom.cpp"
    src.write_text(IDIOM)
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-o", str(tmp_path / "idiom"), "-L", lib, "-lqmckl_gpu", "-Wl,-rpath," + lib],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_test_programs_compile_against_the_c_abi():
    ref = _reference_dir()
    if ref is None or not os.path.isdir(os.path.join(ref, "tests")):
        pytest.skip("reference checkout absent (QMCKL_REFERENCE_DIR)")
    _lib()
    r = subprocess.run(["sh", os.path.join(ROOT, "oracle", "ref_tests_compile.sh"), ref],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    for t in ("test_qmckl_ao", "test_qmckl_mo"):
        assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "compat", t))
