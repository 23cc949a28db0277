// skelcl::Vector<T>: a host std::vector<T> mirrored lazily on the GB300
// (include/SkelCL/Vector.h, include/SkelCL/detail/VectorDef.h:67-691 of the
// reference).
//
// Coherence follows the reference: data moves only when needed.  Element
// access (operator[], at, front, back, iterators) first brings the host copy
// up to date; a skeleton call uploads inputs whose device copy is stale and
// marks its outputs device-modified.  Like the reference, writing through the
// non-const accessors does not mark the device copy stale: call
// dataOnHostModified() after changing a vector that already lives on the
// device.  Device memory is one allocation per vector (one GPU).
#ifndef SKELCL_VECTOR_H_
#define SKELCL_VECTOR_H_

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include <pvsutil/Assert.h>
#include <pvsutil/Logger.h>

#include "Distributions.h"
#include "detail/Device.h"
#include "detail/Runtime.h"

namespace skelcl {

namespace detail {

// Completion handle of an upload / download (detail::Event of the
// reference); transfers complete synchronously here, so wait() is cheap.
class Event {
public:
  void wait() const {}
};

// Per-device sizes of a container (one device: the whole size).
class Sizes {
public:
  Sizes() = default;
  void push_back(size_t s) { _sizes.push_back(s); }
  unsigned int operator[](size_t i) const { return static_cast<unsigned int>(_sizes[i]); }

private:
  std::vector<size_t> _sizes;
};

}  // namespace detail

template <typename T>
class Vector {
public:
  typedef std::vector<T> host_buffer_type;
  typedef typename host_buffer_type::value_type value_type;
  typedef typename host_buffer_type::pointer pointer;
  typedef typename host_buffer_type::const_pointer const_pointer;
  typedef typename host_buffer_type::reference reference;
  typedef typename host_buffer_type::const_reference const_reference;
  typedef typename host_buffer_type::iterator iterator;
  typedef typename host_buffer_type::const_iterator const_iterator;
  typedef typename host_buffer_type::size_type size_type;
  typedef typename host_buffer_type::difference_type difference_type;
  typedef typename host_buffer_type::allocator_type allocator_type;

  Vector() : _distribution(new detail::Distribution<Vector<T>>()) {}

  explicit Vector(const size_type size, const value_type& value = value_type(),
                  const detail::Distribution<Vector<T>>& distribution =
                      detail::Distribution<Vector<T>>())
      : _size(size),
        _distribution(distribution.clone()),
        _deviceUpToDate(false),
        _host(size, value) {}

  template <class InputIterator>
  Vector(InputIterator first, InputIterator last)
      : _distribution(new detail::Distribution<Vector<T>>()), _deviceUpToDate(false),
        _host(first, last) {
    _size = _host.size();
  }

  template <class InputIterator>
  Vector(InputIterator first, InputIterator last,
         const detail::Distribution<Vector<T>>& distribution)
      : _distribution(distribution.clone()), _deviceUpToDate(false), _host(first, last) {
    _size = _host.size();
  }

  Vector(const Vector<T>& rhs)
      : _size(rhs._size), _distribution(rhs._distribution->clone()), _deviceUpToDate(false) {
    rhs.copyDataToHost();
    _host = rhs._host;
  }

  Vector(Vector<T>&& rhs) noexcept
      : _size(rhs._size),
        _distribution(std::move(rhs._distribution)),
        _hostUpToDate(rhs._hostUpToDate),
        _deviceUpToDate(rhs._deviceUpToDate),
        _host(std::move(rhs._host)),
        _device(std::move(rhs._device)) {
    rhs._size = 0;
    rhs._distribution.reset(new detail::Distribution<Vector<T>>());
    rhs._hostUpToDate = true;
    rhs._deviceUpToDate = true;
  }

  Vector<T>& operator=(const Vector<T>& rhs) {
    if (this == &rhs) return *this;
    rhs.copyDataToHost();
    _size = rhs._size;
    _host = rhs._host;
    _distribution = rhs._distribution->clone();
    _hostUpToDate = true;
    _deviceUpToDate = false;
    _device.reset();
    return *this;
  }

  Vector<T>& operator=(Vector<T>&& rhs) noexcept {
    if (this == &rhs) return *this;
    _size = rhs._size;
    _distribution = std::move(rhs._distribution);
    _hostUpToDate = rhs._hostUpToDate;
    _deviceUpToDate = rhs._deviceUpToDate;
    _host = std::move(rhs._host);
    _device = std::move(rhs._device);
    rhs._size = 0;
    rhs._distribution.reset(new detail::Distribution<Vector<T>>());
    rhs._hostUpToDate = true;
    rhs._deviceUpToDate = true;
    return *this;
  }

  ~Vector() = default;

  // ---- iterators and element access (bring the host copy up to date) ----------
  iterator begin() { copyDataToHost(); return _host.begin(); }
  const_iterator begin() const { copyDataToHost(); return _host.begin(); }
  iterator end() { copyDataToHost(); return _host.end(); }
  const_iterator end() const { copyDataToHost(); return _host.end(); }

  size_type size() const { return _size; }
  detail::Sizes sizes() const {
    detail::Sizes s;
    s.push_back(_size);
    return s;
  }
  size_type max_size() const { return _host.max_size(); }
  void resize(size_type count, T value = T()) {
    copyDataToHost();
    _host.resize(count, value);
    _size = count;
    _deviceUpToDate = false;
    _device.reset();
  }
  size_type capacity() const { return std::max(_host.capacity(), _size); }
  bool empty() const { return _size == 0; }
  void reserve(size_type n) { _host.reserve(n); }

  reference operator[](size_type pos) { copyDataToHost(); return _host[pos]; }
  const_reference operator[](size_type pos) const { copyDataToHost(); return _host[pos]; }
  reference at(size_type pos) { copyDataToHost(); return _host.at(pos); }
  const_reference at(size_type pos) const { copyDataToHost(); return _host.at(pos); }
  reference front() { copyDataToHost(); return _host.front(); }
  const_reference front() const { copyDataToHost(); return _host.front(); }
  reference back() { copyDataToHost(); return _host.back(); }
  const_reference back() const { copyDataToHost(); return _host.back(); }

  // ---- modifiers (the host copy becomes the only valid one) --------------------
  template <class InputIterator>
  void assign(InputIterator first, InputIterator last) {
    _host.assign(first, last);
    hostResized();
  }
  void assign(size_type count, const T& value = T()) {
    _host.assign(count, value);
    hostResized();
  }
  void push_back(const T& value) {
    copyDataToHost();
    _host.push_back(value);
    hostResized();
  }
  void pop_back() {
    copyDataToHost();
    _host.pop_back();
    hostResized();
  }
  iterator insert(iterator pos, const T& value) {
    auto it = _host.insert(pos, value);
    hostResized();
    return it;
  }
  iterator insert(iterator pos, size_type count, const T& value) {
    auto it = _host.insert(pos, count, value);
    hostResized();
    return it;
  }
  template <class InputIterator>
  void insert(iterator pos, InputIterator first, InputIterator last) {
    _host.insert(pos, first, last);
    hostResized();
  }
  iterator erase(iterator pos) {
    auto it = _host.erase(pos);
    hostResized();
    return it;
  }
  iterator erase(iterator first, iterator last) {
    auto it = _host.erase(first, last);
    hostResized();
    return it;
  }
  void swap(Vector<T>& rhs) {
    std::swap(_size, rhs._size);
    std::swap(_distribution, rhs._distribution);
    std::swap(_hostUpToDate, rhs._hostUpToDate);
    std::swap(_deviceUpToDate, rhs._deviceUpToDate);
    _host.swap(rhs._host);
    std::swap(_device, rhs._device);
  }
  void clear() {
    _host.clear();
    hostResized();
  }

  // ---- distributions (one device) ------------------------------------------------
  detail::Distribution<Vector<T>>& distribution() const { return *_distribution; }
  template <typename U>
  void setDistribution(const detail::Distribution<Vector<U>>& d) const {
    _distribution = detail::cloneAndConvert<Vector<T>>(d);
  }
  template <typename U>
  void setDistribution(const std::unique_ptr<detail::Distribution<Vector<U>>>& d) const {
    _distribution = detail::cloneAndConvert<Vector<T>>(*d);
  }
  void setDistribution(std::unique_ptr<detail::Distribution<Vector<T>>>&& d) const {
    _distribution = std::move(d);
  }

  // ---- host/device coherence -------------------------------------------------------
  void createDeviceBuffers() const {
    if (!_device || !_device->valid() || _device->bytes() < bytes()) forceCreateDeviceBuffers();
  }
  void forceCreateDeviceBuffers() const {
    _device.reset(new detail::DeviceBuffer(bytes() ? bytes() : sizeof(T)));
  }
  detail::Event startUpload() const {
    copyDataToDevices();
    return detail::Event();
  }
  void copyDataToDevices() const {
    const bool fresh = !_device || !_device->valid() || _device->bytes() < bytes();
    if (fresh) {
      copyDataToHost();
      forceCreateDeviceBuffers();
      _deviceUpToDate = false;
    }
    if (!_deviceUpToDate) {
      if (bytes()) detail::checkStatus(scl_h2d(_device->get(), _host.data(), bytes()), "upload");
      _deviceUpToDate = true;
    }
  }
  detail::Event startDownload() const {
    copyDataToHost();
    return detail::Event();
  }
  void copyDataToHost() const {
    if (_hostUpToDate) return;
    if (!_device || !_device->valid()) {  // device copy lost (terminate): keep host
      _hostUpToDate = true;
      return;
    }
    _host.resize(_size);
    if (bytes()) detail::checkStatus(scl_d2h(_host.data(), _device->get(), bytes()), "download");
    _hostUpToDate = true;
  }
  void dataOnDeviceModified() const {
    _hostUpToDate = false;
    _deviceUpToDate = true;
  }
  void dataOnHostModified() const {
    _hostUpToDate = true;
    _deviceUpToDate = false;
  }
  bool hostIsUpToDate() const { return _hostUpToDate; }
  bool devicesAreUpToDate() const { return _deviceUpToDate; }

  const detail::DeviceBuffer& deviceBuffer(const detail::Device&) const {
    createDeviceBuffers();
    return *_device;
  }
  host_buffer_type& hostBuffer() const { return _host; }
  static std::string deviceFunctions() { return std::string(); }

  // Device address of the (up to date) data: uploads if needed.
  T* devicePtr() const {
    copyDataToDevices();
    return static_cast<T*>(_device->get());
  }
  // Device address for writing; the caller marks the data device-modified.
  T* deviceOutputPtr() const {
    createDeviceBuffers();
    if (!_hostUpToDate) _deviceUpToDate = true;
    return static_cast<T*>(_device->get());
  }

private:
  size_t bytes() const { return _size * sizeof(T); }
  void hostResized() {
    _size = _host.size();
    _hostUpToDate = true;
    _deviceUpToDate = false;
    _device.reset();
  }

  size_type _size = 0;
  mutable std::unique_ptr<detail::Distribution<Vector<T>>> _distribution;
  mutable bool _hostUpToDate = true;
  mutable bool _deviceUpToDate = true;
  mutable host_buffer_type _host;
  mutable std::shared_ptr<detail::DeviceBuffer> _device;
};

}  // namespace skelcl

#endif  // SKELCL_VECTOR_H_
