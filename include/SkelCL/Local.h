// __local memory for a user function parameter `__local T* p`
// (include/SkelCL/Local.h, src/Local.cpp:44-57 of the reference).
#ifndef SKELCL_LOCAL_H_
#define SKELCL_LOCAL_H_

#include <cstddef>

namespace skelcl {

class Local {
public:
  explicit Local(size_t sizeInBytes) : _sizeInBytes(sizeInBytes) {}
  size_t getSizeInBytes() const { return _sizeInBytes; }

private:
  size_t _sizeInBytes;
};

inline Local local(size_t sizeInBytes) { return Local(sizeInBytes); }

}  // namespace skelcl

#endif  // SKELCL_LOCAL_H_
