/*
 * Stand-in for the few Thrust facilities the reference uses (device_vector
 * storage, raw_pointer_cast, sort of floats at mainPUMP.cu:303, reduce of
 * ints at collisionProbability.cu:28) when the reference is built for the
 * CPU oracle.  Sorting and integer summation have one exact result, so the
 * reference's outputs do not depend on which implementation produced them.
 * Storage is host memory, value-initialised like thrust::device_vector.
 *
 * Test infrastructure only.
 */
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdlib>

namespace thrust {
template <class T>
class device_vector {
 public:
  explicit device_vector(size_t n) : p_(static_cast<T *>(std::calloc(n ? n : 1, sizeof(T)))), n_(n) {}
  ~device_vector() { std::free(p_); }
  device_vector(const device_vector &) = delete;
  device_vector &operator=(const device_vector &) = delete;
  T *data() { return p_; }
  T *begin() { return p_; }
  T *end() { return p_ + n_; }
  T &operator[](size_t i) { return p_[i]; }
  size_t size() const { return n_; }

 private:
  T *p_;
  size_t n_;
};
template <class T> using host_vector = device_vector<T>;
template <class T> inline T *raw_pointer_cast(T *p) { return p; }
template <class T> inline void sort(T *b, T *e) { std::sort(b, e); }
template <class T> inline T reduce(T *b, T *e) {
  T s = T();
  for (; b != e; ++b) s += *b;
  return s;
}
}  // namespace thrust
