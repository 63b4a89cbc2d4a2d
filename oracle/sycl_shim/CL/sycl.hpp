// Host-only stand-in for the small subset of SYCL 2020 that the reference library
// (qmckl_sycl, src/*.cpp) uses, so that its unmodified sources compile with g++ and
// run on the CPU. Test infrastructure only: it exists so that the oracle in this
// directory can be checked against the reference's own code path.
//
// Semantics chosen to match a device run of the reference:
//  * malloc_device returns zeroed memory (calloc), which is what a fresh allocation
//    looks like in the reference's tests; the reference never zeroes by itself.
//  * parallel_for bodies write disjoint slots in every kernel the hot path uses
//    (per point, per (point, shell), per (point, AO)), so running them on several
//    host threads gives the same bits as running them serially. OpenMP is used
//    when the translation unit is compiled with -fopenmp.
//  * buffers alias their host pointer, so host accessors see kernel writes directly.
#pragma once

#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <iostream>
#include <pthread.h>
#include <string>

namespace sycl {

class exception : public std::exception {
 public:
  const char* what() const noexcept override { return "sycl shim exception"; }
};

template <int D> struct range;
template <> struct range<1> {
  size_t n[1];
  explicit range(size_t a) : n{a} {}
  size_t size() const { return n[0]; }
};
template <> struct range<2> {
  size_t n[2];
  range(size_t a, size_t b) : n{a, b} {}
  size_t size() const { return n[0] * n[1]; }
};

template <int D> struct id;
template <> struct id<1> {
  size_t v;
  id(size_t a = 0) : v(a) {}
  operator size_t() const { return v; }
  size_t operator[](int) const { return v; }
};
template <> struct id<2> {
  size_t v[2];
  id(size_t a, size_t b) : v{a, b} {}
  size_t operator[](int i) const { return v[i]; }
};

namespace detail {
template <class F> void run1(size_t n, F f) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (long long i = 0; i < (long long)n; ++i) f(id<1>((size_t)i));
}
template <class F> void run2(size_t n0, size_t n1, F f) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (long long i = 0; i < (long long)n0; ++i)
    for (size_t j = 0; j < n1; ++j) f(id<2>((size_t)i, j));
}
}  // namespace detail

struct event {
  void wait() {}
};

namespace info {
namespace device {
struct name {};
}  // namespace device
}  // namespace info

struct device {
  template <class T> std::string get_info() const { return "host (sycl shim)"; }
};

struct gpu_selector_t {};
struct accelerator_selector_t {};
inline constexpr gpu_selector_t gpu_selector_v{};
inline constexpr accelerator_selector_t accelerator_selector_v{};

namespace access {
enum class mode { read, write, read_write, discard_write };
}
struct write_only_t {};
struct read_only_t {};
struct read_write_t {};
inline constexpr write_only_t write_only{};
inline constexpr read_only_t read_only{};
inline constexpr read_write_t read_write{};

class handler {
 public:
  template <class Name = void, class F> void parallel_for(range<1> r, F f) { detail::run1(r.n[0], f); }
  template <class Name = void, class F> void parallel_for(range<2> r, F f) { detail::run2(r.n[0], r.n[1], f); }
  template <class Name = void, class F> void parallel_for(size_t n, F f) { detail::run1(n, f); }
  template <class Name = void, class F> void single_task(F f) { f(); }
};

template <class T, int D = 1> class accessor {
 public:
  T* p;
  explicit accessor(T* q) : p(q) {}
  template <class B, class Tag> accessor(B& b, handler&, Tag) : p(b.data()) {}
  T& operator[](size_t i) const { return p[i]; }
};

template <class T, int D = 1> class buffer {
 public:
  buffer(T* host, range<1>) : p_(host) {}
  T* data() { return p_; }
  template <access::mode M> accessor<T, D> get_access(handler&) { return accessor<T, D>(p_); }
  accessor<T, D> get_host_access() { return accessor<T, D>(p_); }

 private:
  T* p_;
};

template <class T, int D, class Tag> accessor(buffer<T, D>&, handler&, Tag) -> accessor<T, D>;

class queue {
 public:
  queue() {}
  explicit queue(const gpu_selector_t&) { throw exception(); }
  explicit queue(const accelerator_selector_t&) { throw exception(); }
  device get_device() const { return device(); }
  template <class F> event submit(F f) {
    handler h;
    f(h);
    return event();
  }
  template <class Name = void, class F> event parallel_for(range<1> r, F f) { detail::run1(r.n[0], f); return event(); }
  template <class Name = void, class F> event parallel_for(range<2> r, F f) { detail::run2(r.n[0], r.n[1], f); return event(); }
  template <class Name = void, class F> event parallel_for(size_t n, F f) { detail::run1(n, f); return event(); }
  template <class F> event single_task(F f) { f(); return event(); }
  event memcpy(void* dst, const void* src, size_t n) {
    if (n) std::memmove(dst, src, n);
    return event();
  }
  void wait() {}
};

inline void* malloc_device(size_t n, const queue&) { return std::calloc(n ? n : 1, 1); }
template <class T> T* malloc_device(size_t count, const queue&) { return static_cast<T*>(std::calloc(count ? count : 1, sizeof(T))); }
inline void free(void* p, const queue&) { std::free(p); }

}  // namespace sycl

namespace cl {
namespace sycl = ::sycl;
}
