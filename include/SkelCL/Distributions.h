// Distributions (include/SkelCL/Distributions.h:64-401 of the reference).
// With one GPU every distribution places the whole container on that device;
// the classes keep the reference's API and validity semantics so that code
// choosing distributions compiles and runs unchanged.
#ifndef SKELCL_DISTRIBUTIONS_H_
#define SKELCL_DISTRIBUTIONS_H_

#include <functional>
#include <memory>

#include "detail/Device.h"
#include "detail/Padding.h"

namespace skelcl {
namespace detail {

template <typename C>
class Distribution {
public:
  Distribution() = default;
  virtual ~Distribution() = default;
  virtual bool isValid() const { return false; }
  virtual bool isSingle() const { return false; }
  virtual bool isBlock() const { return false; }
  virtual bool isCopy() const { return false; }
  virtual bool isOL() const { return false; }
  virtual std::unique_ptr<Distribution<C>> clone() const {
    return std::unique_ptr<Distribution<C>>(new Distribution<C>(*this));
  }
  const DeviceList& devices() const { return globalDeviceList; }
  // The i-th device the container lives on (always the one GPU).
  std::shared_ptr<Device> device(size_t i) const {
    return i < globalDeviceList.size() ? globalDeviceList[i] : std::shared_ptr<Device>();
  }
  bool operator==(const Distribution<C>& rhs) const { return kind() == rhs.kind(); }
  bool operator!=(const Distribution<C>& rhs) const { return !(*this == rhs); }
  virtual int kind() const { return 0; }
};

template <typename C>
class SingleDistribution : public Distribution<C> {
public:
  SingleDistribution() = default;
  explicit SingleDistribution(const std::shared_ptr<Device>&) {}
  template <typename U>
  SingleDistribution(const SingleDistribution<U>&) {}
  bool isValid() const override { return true; }
  bool isSingle() const override { return true; }
  int kind() const override { return 1; }
  std::unique_ptr<Distribution<C>> clone() const override {
    return std::unique_ptr<Distribution<C>>(new SingleDistribution<C>(*this));
  }
};

template <typename C>
class BlockDistribution : public Distribution<C> {
public:
  BlockDistribution() = default;
  template <typename U>
  BlockDistribution(const BlockDistribution<U>&) {}
  bool isValid() const override { return true; }
  bool isBlock() const override { return true; }
  int kind() const override { return 2; }
  std::unique_ptr<Distribution<C>> clone() const override {
    return std::unique_ptr<Distribution<C>>(new BlockDistribution<C>(*this));
  }
};

template <typename C>
class CopyDistribution : public Distribution<C> {
public:
  typedef typename C::value_type T;
  CopyDistribution() = default;
  CopyDistribution(const DeviceList&, std::function<T(const T&, const T&)> combine = nullptr)
      : _combine(combine) {}
  template <typename U>
  CopyDistribution(const CopyDistribution<U>&) {}
  bool isValid() const override { return true; }
  bool isCopy() const override { return true; }
  int kind() const override { return 3; }
  std::unique_ptr<Distribution<C>> clone() const override {
    return std::unique_ptr<Distribution<C>>(new CopyDistribution<C>(*this));
  }
  std::function<T(const T&, const T&)> combineFunc() const { return _combine; }

private:
  std::function<T(const T&, const T&)> _combine;
};

template <typename C>
class OLDistribution : public Distribution<C> {
public:
  OLDistribution() = default;
  OLDistribution(unsigned int range, Padding padding) : _range(range), _padding(padding) {}
  template <typename U>
  OLDistribution(const OLDistribution<U>& o) : _range(o.overlapRange()), _padding(o.padding()) {}
  bool isValid() const override { return true; }
  bool isOL() const override { return true; }
  int kind() const override { return 4; }
  std::unique_ptr<Distribution<C>> clone() const override {
    return std::unique_ptr<Distribution<C>>(new OLDistribution<C>(*this));
  }
  unsigned int overlapRange() const { return _range; }
  Padding padding() const { return _padding; }

private:
  unsigned int _range = 0;
  Padding _padding = Padding::NEAREST;
};

// Clone a distribution onto a container of another element type.
template <typename OutC, typename InC>
std::unique_ptr<Distribution<OutC>> cloneAndConvert(const Distribution<InC>& d) {
  if (auto* s = dynamic_cast<const SingleDistribution<InC>*>(&d))
    return std::unique_ptr<Distribution<OutC>>(new SingleDistribution<OutC>(*s));
  if (auto* b = dynamic_cast<const BlockDistribution<InC>*>(&d))
    return std::unique_ptr<Distribution<OutC>>(new BlockDistribution<OutC>(*b));
  if (auto* c = dynamic_cast<const CopyDistribution<InC>*>(&d))
    return std::unique_ptr<Distribution<OutC>>(new CopyDistribution<OutC>(*c));
  if (auto* o = dynamic_cast<const OLDistribution<InC>*>(&d))
    return std::unique_ptr<Distribution<OutC>>(new OLDistribution<OutC>(*o));
  return std::unique_ptr<Distribution<OutC>>(new Distribution<OutC>());
}

}  // namespace detail

namespace distribution {

template <typename T>
struct identity {
  typedef T type;
};

template <template <typename> class C, typename T>
std::unique_ptr<detail::Distribution<C<T>>> Block(const C<T>&) {
  return std::unique_ptr<detail::Distribution<C<T>>>(new detail::BlockDistribution<C<T>>());
}
template <template <typename> class C, typename T>
void setBlock(const C<T>& c) {
  c.setDistribution(Block(c));
}
template <template <typename> class C, typename T>
std::unique_ptr<detail::Distribution<C<T>>> OL(const C<T>&) {
  return std::unique_ptr<detail::Distribution<C<T>>>(new detail::OLDistribution<C<T>>());
}
template <template <typename> class C, typename T>
void setOL(const C<T>& c) {
  c.setDistribution(OL(c));
}
template <template <typename> class C, typename T>
std::unique_ptr<detail::Distribution<C<T>>> Copy(
    const C<T>&, typename identity<std::function<T(const T&, const T&)>>::type combine = nullptr) {
  return std::unique_ptr<detail::Distribution<C<T>>>(
      new detail::CopyDistribution<C<T>>(detail::globalDeviceList, combine));
}
template <template <typename> class C, typename T>
void setCopy(const C<T>& c, std::function<T(const T&, const T&)> combine = nullptr) {
  c.setDistribution(Copy(c, combine));
}
template <template <typename> class C, typename T>
std::unique_ptr<detail::Distribution<C<T>>> Single(const C<T>&) {
  return std::unique_ptr<detail::Distribution<C<T>>>(new detail::SingleDistribution<C<T>>());
}
template <template <typename> class C, typename T>
std::unique_ptr<detail::Distribution<C<T>>> Single(const C<T>&,
                                                   const std::shared_ptr<detail::Device>& d) {
  return std::unique_ptr<detail::Distribution<C<T>>>(new detail::SingleDistribution<C<T>>(d));
}
template <template <typename> class C, typename T>
void setSingle(const C<T>& c) {
  c.setDistribution(Single(c));
}
template <template <typename> class C, typename T>
void setSingle(const C<T>& c, const std::shared_ptr<detail::Device>& d) {
  c.setDistribution(Single(c, d));
}

}  // namespace distribution
}  // namespace skelcl

#endif  // SKELCL_DISTRIBUTIONS_H_
