// print(...): space-separated values and a newline on rank 0 (the only rank).
#ifndef MINIM_GB300_PRINT_H
#define MINIM_GB300_PRINT_H

#include <iostream>
#include <vector>

namespace minim {
inline void print() { std::cout << std::endl; }
template <typename T>
inline void print_one(const T& v) { std::cout << v; }
template <typename T>
inline void print_one(const std::vector<T>& v) {
  for (size_t i = 0; i < v.size(); i++) std::cout << (i ? " " : "") << v[i];
}
template <typename T, typename... Args>
void print(const T& first, const Args&... args) {
  print_one(first);
  ((std::cout << " ", print_one(args)), ...);
  std::cout << std::endl;
}
template <typename... Args>
void printAll(const Args&... args) { print(args...); }
}  // namespace minim

#endif
