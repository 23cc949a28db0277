// The one GB300 the runtime drives, presented with the reference's Device
// interface (include/SkelCL/detail/Device.h:69-360): id, type, name,
// work-group limits, double support.
#ifndef SKELCL_DEVICE_H_
#define SKELCL_DEVICE_H_

#include <cctype>
#include <istream>
#include <string>
#include <cstddef>
#include <memory>
#include <string>
#include <vector>

#include "Runtime.h"

namespace skelcl {
namespace detail {

class Device {
public:
  typedef size_t id_type;
  enum Type { DEFAULT = 1, CPU = 2, GPU = 4, ACCELERATOR = 8, ALL = 0xFFFFFFFF, ANY = ALL };

  Device(int cudaDevice, id_type id) : _cuda(cudaDevice), _id(id) {
    char name[256] = {0};
    int sms = 0;
    size_t mem = 0;
    checkStatus(scl_device_info(&sms, &mem, name, sizeof(name)), "scl_device_info");
    _name = name;
    _sms = sms;
    _mem = mem;
  }
  id_type id() const { return _id; }
  int cudaDevice() const { return _cuda; }
  std::string name() const { return _name; }
  std::string vendorName() const { return "NVIDIA Corporation"; }
  Type type() const { return GPU; }
  bool isType(Type t) const { return t == GPU || t == ALL || t == DEFAULT; }
  size_t maxWorkGroupSize() const { return 1024; }
  size_t maxWorkGroups() const { return 0x7fffffff; }
  unsigned int maxComputeUnits() const { return (unsigned int)_sms; }
  unsigned long globalMemSize() const { return (unsigned long)_mem; }
  unsigned long localMemSize() const { return 227ul * 1024; }
  bool supportsDouble() const { return true; }
  void wait() const { checkStatus(scl_sync(), "scl_sync"); }

private:
  int _cuda;
  id_type _id;
  std::string _name;
  int _sms = 0;
  size_t _mem = 0;
};

class DeviceList {
public:
  typedef std::shared_ptr<Device> value_type;
  typedef std::vector<std::shared_ptr<Device>>::iterator iterator;
  typedef std::vector<std::shared_ptr<Device>>::const_iterator const_iterator;
  iterator begin() { return _devices.begin(); }
  iterator end() { return _devices.end(); }
  const_iterator begin() const { return _devices.begin(); }
  const_iterator end() const { return _devices.end(); }
  size_t size() const { return _devices.size(); }
  bool empty() const { return _devices.empty(); }
  std::shared_ptr<Device>& front() { return _devices.front(); }
  const std::shared_ptr<Device>& front() const { return _devices.front(); }
  std::shared_ptr<Device>& operator[](size_t i) { return _devices[i]; }
  const std::shared_ptr<Device>& operator[](size_t i) const { return _devices[i]; }
  void clear() { _devices.clear(); }
  void push_back(std::shared_ptr<Device> d) { _devices.push_back(std::move(d)); }

private:
  std::vector<std::shared_ptr<Device>> _devices;
};

// One device at most: every skeleton runs on the GPU that init() selected.
inline DeviceList globalDeviceList;

class DeviceID {
public:
  explicit DeviceID(size_t id) : _id(id) {}
  size_t id() const { return _id; }

private:
  size_t _id;
};

class PlatformID {
public:
  explicit PlatformID(size_t id) : _id(id) {}
  size_t id() const { return _id; }

private:
  size_t _id;
};

// Device selection (include/SkelCL/detail/DeviceProperties.h:56-68).  Any
// count or type selects the single GB300; nDevices(n) with n > 1 still runs
// on one device.
class DeviceProperties {
public:
  static DeviceProperties nDevices(size_t n) {
    DeviceProperties p;
    p._count = n;
    p._takeAll = false;
    return p;
  }
  static DeviceProperties allDevices() {
    DeviceProperties p;
    p._takeAll = true;
    return p;
  }
  DeviceProperties& deviceType(Device::Type t) {
    _type = t;
    return *this;
  }
  Device::Type deviceType() const { return _type; }
  size_t count() const { return _count; }
  bool takeAll() const { return _takeAll; }

private:
  DeviceProperties() = default;
  Device::Type _type = Device::ALL;
  bool _takeAll = true;
  size_t _count = 0;
};

inline std::ostream& operator<<(std::ostream& os, Device::Type t) {
  switch (t) {
    case Device::CPU: return os << "CPU";
    case Device::GPU: return os << "GPU";
    case Device::ACCELERATOR: return os << "ACCELERATOR";
    case Device::DEFAULT: return os << "DEFAULT";
    default: return os << "ANY";
  }
}

// Reads ANY, ALL, CPU, GPU, ACCELERATOR or DEFAULT (command-line arguments of
// type device_type); anything else sets the stream's fail bit.
inline std::istream& operator>>(std::istream& is, Device::Type& t) {
  std::string w;
  is >> w;
  for (char& c : w) c = (char)std::toupper((unsigned char)c);
  if (w == "ANY" || w == "ALL") t = Device::ANY;
  else if (w == "CPU") t = Device::CPU;
  else if (w == "GPU") t = Device::GPU;
  else if (w == "ACCELERATOR") t = Device::ACCELERATOR;
  else if (w == "DEFAULT") t = Device::DEFAULT;
  else is.setstate(std::ios::failbit);
  return is;
}

}  // namespace detail
}  // namespace skelcl

#endif  // SKELCL_DEVICE_H_
