// Host-only stand-in for the SYCL accessor type named in the reference's
// TreeScorer signature.  Test infrastructure for oracle/_ref only.
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
} // namespace cl::sycl
