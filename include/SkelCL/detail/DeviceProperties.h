// Compatibility header: the device classes live in detail/Device.h.
#ifndef SKELCL_DETAIL_DeviceProperties_H_
#define SKELCL_DETAIL_DeviceProperties_H_
#include "Device.h"
#endif
