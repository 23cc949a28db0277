// Utilities of the reference's detail::util namespace
// (include/SkelCL/detail/Util.h:60-98, src/Util.cpp:149-235): the program
// hash (SHA-1, computed by libskelcl_cuda.so), the OpenCL spelling of a C++
// type, and integer helpers.
#ifndef SKELCL_UTIL_H_
#define SKELCL_UTIL_H_

#include <cxxabi.h>

#include <cmath>
#include <cstdlib>
#include <string>
#include <typeinfo>

#include "Runtime.h"

namespace skelcl {
namespace detail {

// Name of T as the device code spells it: the demangled type name without
// namespaces ("float", "unsigned int", "float4", a typedef'd struct's name),
// as detail::util::typeToString does in the reference.
template <typename T>
std::string typeName() {
  int status = 0;
  char* d = abi::__cxa_demangle(typeid(T).name(), nullptr, nullptr, &status);
  std::string name = (status == 0 && d) ? d : typeid(T).name();
  std::free(d);
  auto ns = name.rfind(':');
  if (ns != std::string::npos) name.erase(0, ns + 1);
  return name;
}

namespace util {

inline std::string hash(const std::string& text) {
  char out[41] = {0};
  checkStatus(scl_sha1_hex(text.data(), text.size(), out), "scl_sha1_hex");
  return std::string(out);
}

template <typename T>
std::string typeToString() {
  return typeName<T>();
}

inline std::string envVarValue(const std::string& v) {
  const char* e = std::getenv(v.c_str());
  return e ? std::string(e) : std::string();
}

inline size_t devideAndRoundUp(size_t i, size_t j) { return i / j + (i % j != 0); }

inline size_t devideAndAlign(size_t i, size_t j, size_t a) {
  size_t x = devideAndRoundUp(i, j);
  size_t r = x % a;
  return r ? x + (a - r) : x;
}

inline size_t ceilToMultipleOf(size_t i, size_t j) {
  if (i == 0) return j;
  size_t r = i % j;
  return r ? i + (j - r) : i;
}

inline bool isPowerOfTwo(size_t n) { return (n & (n - 1)) == 0; }

inline int floorPow2(int n) {
  int p = 1;
  while (p * 2 <= n) p *= 2;
  return p;
}

inline int ceilPow2(int n) {
  int p = 1;
  while (p < n) p *= 2;
  return p;
}

}  // namespace util
}  // namespace detail
}  // namespace skelcl

#endif  // SKELCL_UTIL_H_
