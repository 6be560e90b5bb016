// Host-only stand-ins for the SYCL types named in the reference's scorer
// classes: the 1-D accessor of src/TreeScorer.hpp, the 2-D accessor and
// the vec<T, N> of cpu_scoring_benchmark/CPUTreeScorer.hpp.  Test
// infrastructure for oracle/_ref only.
#pragma once
#include <cstddef>
namespace cl::sycl {
namespace access {
enum class mode { read, write, read_write, discard_write };
enum class target { device, host_buffer };
} // namespace access
template <class T, int D, access::mode M, access::target Tg> struct accessor {
  const T *ptr;
  const T &operator[](std::size_t i) const { return ptr[i]; }
};
// Two dimensions: [row][column] over a row-major block of `cols` columns.
template <class T, access::mode M, access::target Tg>
struct accessor<T, 2, M, Tg> {
  const T *ptr;
  std::size_t cols;
  const T *operator[](std::size_t i) const { return ptr + i * cols; }
};
// Element-wise N-vector with the operators the scorer uses.
template <class T, int N> struct vec {
  T v[N];
  vec() : v{} {}
  vec(T x) {
    for (int i = 0; i < N; i++) v[i] = x;
  }
  T &operator[](int i) { return v[i]; }
  const T &operator[](int i) const { return v[i]; }
  vec operator&(const vec &o) const {
    vec r;
    for (int i = 0; i < N; i++) r.v[i] = v[i] & o.v[i];
    return r;
  }
  vec operator~() const {
    vec r;
    for (int i = 0; i < N; i++) r.v[i] = ~v[i];
    return r;
  }
  vec operator*(T x) const {
    vec r;
    for (int i = 0; i < N; i++) r.v[i] = v[i] * x;
    return r;
  }
  vec &operator+=(const vec &o) {
    for (int i = 0; i < N; i++) v[i] += o.v[i];
    return *this;
  }
};
} // namespace cl::sycl
