// Glue between the header templates and libskelcl_cuda.so: status checking
// with the reference's failure behaviour (LOG_ERROR + exit, or throw with
// THROW_ON_FAILURE; libraries/pvsutil/include/pvsutil/Logger.h:108-114), and
// a runtime generation counter so that device buffers from before a
// terminate()/init() pair are never freed into the new context.
#ifndef SKELCL_RUNTIME_H_
#define SKELCL_RUNTIME_H_

#include <cstddef>
#include <string>

#include <pvsutil/Logger.h>

#include "../../skelcl_cuda.h"

namespace skelcl {
namespace detail {

inline unsigned long& runtimeGeneration() {
  static unsigned long g = 0;
  return g;
}

inline void checkStatus(int status, const char* what) {
  if (status == SCL_OK) return;
  std::string msg = std::string(what) + " failed (status " + std::to_string(status) +
                    "): " + scl_last_error_string();
  ABORT_WITH_ERROR(msg);
}

inline void ensureInitialized() {
  if (!scl_is_initialized()) {
    ABORT_WITH_ERROR("SkelCL is not initialised: call skelcl::init() first");
  }
}

// RAII device allocation owned by a container.
class DeviceBuffer {
public:
  typedef size_t size_type;
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t bytes) : _bytes(bytes) {
    ensureInitialized();
    checkStatus(scl_alloc(bytes, &_ptr), "scl_alloc");
    _gen = runtimeGeneration();
  }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() {
    if (_ptr && _gen == runtimeGeneration() && scl_is_initialized()) scl_free(_ptr);
  }
  void* get() const { return _ptr; }
  size_t bytes() const { return _bytes; }
  bool valid() const { return _ptr && _gen == runtimeGeneration() && scl_is_initialized(); }

private:
  void* _ptr = nullptr;
  size_t _bytes = 0;
  unsigned long _gen = 0;
};

}  // namespace detail
}  // namespace skelcl

#endif  // SKELCL_RUNTIME_H_
