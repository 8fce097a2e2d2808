// Element-wise arithmetic on std::vector and small vector helpers, with the
// same names and semantics as the minim library's utils/vec.h (global
// operators, namespace vec), so user potentials written against minim build
// unchanged.
#ifndef MINIM_GB300_VEC_H
#define MINIM_GB300_VEC_H

#include <algorithm>
#include <cmath>
#include <numeric>
#include <type_traits>
#include <vector>

using std::vector;

namespace minim_detail {
template <typename T> struct is_vec : std::false_type {};
template <typename T> struct is_vec<std::vector<T>> : std::true_type {};
template <typename A, typename B, typename F>
auto zip(const vector<A>& a, const vector<B>& b, F f) {
  vector<decltype(f(a[0], b[0]))> r(a.size());
  for (size_t i = 0; i < a.size(); i++) r[i] = f(a[i], b[i]);
  return r;
}
template <typename A, typename F>
auto each(const vector<A>& a, F f) {
  vector<decltype(f(a[0]))> r(a.size());
  for (size_t i = 0; i < a.size(); i++) r[i] = f(a[i]);
  return r;
}
}  // namespace minim_detail

#define MINIM_VEC_BINOP(OP)                                                                      \
  template <typename T, typename U, typename = std::enable_if_t<!minim_detail::is_vec<T>::value>> \
  auto operator OP(T a, const vector<U>& b) {                                                    \
    return minim_detail::each(b, [a](const U& y) { return a OP y; });                            \
  }                                                                                              \
  template <typename T, typename U, typename = std::enable_if_t<!minim_detail::is_vec<U>::value>> \
  auto operator OP(const vector<T>& a, U b) {                                                    \
    return minim_detail::each(a, [b](const T& x) { return x OP b; });                            \
  }                                                                                              \
  template <typename T, typename U>                                                              \
  auto operator OP(const vector<T>& a, const vector<U>& b) {                                     \
    return minim_detail::zip(a, b, [](const T& x, const U& y) { return x OP y; });               \
  }                                                                                              \
  template <typename T, typename U, typename = std::enable_if_t<!minim_detail::is_vec<U>::value>> \
  vector<T>& operator OP##=(vector<T>& a, U b) {                                                 \
    for (auto& x : a) x = x OP b;                                                                \
    return a;                                                                                    \
  }                                                                                              \
  template <typename T, typename U>                                                              \
  vector<T>& operator OP##=(vector<T>& a, const vector<U>& b) {                                  \
    for (size_t i = 0; i < a.size(); i++) a[i] = a[i] OP b[i];                                   \
    return a;                                                                                    \
  }
MINIM_VEC_BINOP(+)
MINIM_VEC_BINOP(-)
MINIM_VEC_BINOP(*)
MINIM_VEC_BINOP(/)
#undef MINIM_VEC_BINOP

template <typename T>
auto operator-(const vector<T>& a) {
  return minim_detail::each(a, [](const T& x) { return -x; });
}

namespace vec {
template <typename T, typename U>
double dotProduct(const vector<T>& a, const vector<U>& b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}
template <typename T, typename U>
auto crossProduct(const vector<T>& a, const vector<U>& b) {
  return vector<decltype(a[0] * b[0])>{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                                       a[0] * b[1] - a[1] * b[0]};
}
template <typename T> T sum(const vector<T>& a) { return std::accumulate(a.begin(), a.end(), T(0)); }
template <typename T> T product(const vector<T>& a) {
  return std::accumulate(a.begin(), a.end(), T(1), std::multiplies<T>());
}
template <typename T> double norm(const vector<T>& a) { return std::sqrt(dotProduct(a, a)); }
template <typename T> double rms(const vector<T>& a) { return std::sqrt(dotProduct(a, a) / a.size()); }
template <typename T> vector<T> abs(const vector<T>& a) {
  return minim_detail::each(a, [](const T& x) { return x < 0 ? -x : x; });
}
template <typename T> vector<T> sqrt(const vector<T>& a) {
  return minim_detail::each(a, [](const T& x) { return (T)std::sqrt(x); });
}
template <typename T, typename U> vector<T> pow(const vector<T>& a, U n) {
  return minim_detail::each(a, [n](const T& x) { return (T)std::pow(x, n); });
}
template <typename T> bool any(const vector<T>& a) {
  return std::any_of(a.begin(), a.end(), [](const T& x) { return (bool)x; });
}
template <typename T> bool all(const vector<T>& a) {
  return std::all_of(a.begin(), a.end(), [](const T& x) { return (bool)x; });
}
template <typename T> bool isIn(const vector<T>& v, T value) {
  return std::find(v.begin(), v.end(), value) != v.end();
}
template <typename T> vector<T> slice(const vector<T>& in, const vector<int>& index) {
  vector<T> r(index.size());
  for (size_t i = 0; i < index.size(); i++) r[i] = in[index[i]];
  return r;
}
inline vector<int> iota(int n, int start = 0) {
  vector<int> r(n);
  std::iota(r.begin(), r.end(), start);
  return r;
}
}  // namespace vec

#endif
