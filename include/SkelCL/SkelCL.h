// skelcl::init / terminate and device selection
// (include/SkelCL/SkelCL.h:144-207 of the reference).  All selections run on
// one GB300 through libskelcl_cuda.so.
#ifndef SKELCL_H_
#define SKELCL_H_

#include <cstddef>

#include "detail/Device.h"
#include "detail/Macros.h"
#include "detail/Runtime.h"
#include "detail/Types.h"
#include "detail/skelclDll.h"

namespace skelcl {

typedef detail::Device::Type device_type;

inline detail::DeviceProperties allDevices() { return detail::DeviceProperties::allDevices(); }
inline detail::DeviceProperties nDevices(size_t n) { return detail::DeviceProperties::nDevices(n); }
inline detail::PlatformID platform(size_t pID) { return detail::PlatformID(pID); }
inline detail::DeviceID device(size_t dID) { return detail::DeviceID(dID); }

namespace detail {
inline void initOn(int cudaDevice) {
  if (scl_is_initialized()) scl_terminate();
  checkStatus(scl_init(cudaDevice), "skelcl::init");
  ++runtimeGeneration();
  globalDeviceList.clear();
  globalDeviceList.push_back(std::make_shared<Device>(cudaDevice, 0));
}
}  // namespace detail

inline void init(detail::DeviceProperties properties = allDevices()) {
  (void)properties;
  detail::initOn(0);
}

inline void init(detail::PlatformID pID, detail::DeviceID dID) {
  (void)pID;
  detail::initOn((int)dID.id());
}

inline void terminate() {
  if (!scl_is_initialized()) return;
  scl_sync();
  detail::globalDeviceList.clear();
  scl_terminate();
  ++detail::runtimeGeneration();
}

}  // namespace skelcl

#endif  // SKELCL_H_
