/* C++ compatibility layer for callers written against the reference's SYCL interface
 * (qmckl_sycl, include/qmckl_gpu.hpp).
 *
 * The reference creates its context from a sycl::queue (src/qmckl_context.cpp:187); this
 * library takes a CUDA device ordinal (include/qmckl_gpu.h). Code that builds a queue with
 * the usual selectors and passes it to qmckl_context_create_device compiles unchanged against
 * this header in place of the reference's qmckl_gpu.hpp: it declares just enough of the sycl
 * namespace for that idiom (a queue, the gpu/accelerator selectors, device names, the
 * exception type), and an overload of qmckl_context_create_device that maps any queue to
 * CUDA device 0 (or to the ordinal in QMCKL_GB300_DEVICE). Every other qmckl_*_device
 * function is the C ABI of qmckl_gpu.h, with the reference's names and argument lists.
 *
 * No SYCL runtime is involved: the queue carries no work; kernels run on the context's CUDA
 * stream. The standard headers the reference's header brings in are included as well, since
 * its callers rely on them.
 */
#pragma once

#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <iostream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "qmckl_gpu.h"

// Callers that bring their own SYCL headers (a SYCL compiler's, or any other implementation of
// sycl::queue) define QMCKL_COMPAT_EXTERNAL_SYCL (SYCL compilers define SYCL_LANGUAGE_VERSION);
// then only the context overload below is added.
#if !defined(SYCL_LANGUAGE_VERSION) && !defined(QMCKL_COMPAT_EXTERNAL_SYCL)
namespace sycl {

class exception : public std::exception {
 public:
  const char* what() const noexcept override { return "sycl::exception"; }
};

namespace info {
namespace device {
struct name {};
}  // namespace device
}  // namespace info

class device {
 public:
  template <class Param>
  std::string get_info() const {
    return "CUDA device (qmckl GB300 library)";
  }
};

struct gpu_selector_t {};
struct accelerator_selector_t {};
struct default_selector_t {};
inline constexpr gpu_selector_t gpu_selector_v{};
inline constexpr accelerator_selector_t accelerator_selector_v{};
inline constexpr default_selector_t default_selector_v{};

class queue {
 public:
  queue() = default;
  explicit queue(gpu_selector_t) {}
  explicit queue(accelerator_selector_t) {}
  explicit queue(default_selector_t) {}
  device get_device() const { return device{}; }
  void wait() const {}
};

}  // namespace sycl
#endif

// The device a queue-created context uses: QMCKL_GB300_DEVICE if set, else 0.
inline int32_t qmckl_compat_device_ordinal() {
  const char* v = std::getenv("QMCKL_GB300_DEVICE");
  return v ? (int32_t)std::atoi(v) : 0;
}

// The reference's context constructor (src/qmckl_context.cpp:187-288), on a CUDA device.
inline qmckl_context_device qmckl_context_create_device(const sycl::queue&) {
  return qmckl_context_create_device(qmckl_compat_device_ordinal());
}
