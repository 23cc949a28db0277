// Vector<Index>: the virtual index space 0..n-1 (include/SkelCL/IndexVector.h
// of the reference).  Nothing is stored or uploaded; Map over it passes each
// index to the user function.
#ifndef SKELCL_INDEX_VECTOR_H_
#define SKELCL_INDEX_VECTOR_H_

#include <memory>

#include "Distributions.h"
#include "Index.h"
#include "Vector.h"

namespace skelcl {

template <>
class Vector<Index> {
public:
  typedef Index value_type;
  typedef size_t size_type;

  Vector(const size_type size) : _size(size), _distribution(new detail::Distribution<Vector<Index>>()) {}
  Vector(const Vector<Index>& rhs) : _size(rhs._size), _distribution(rhs._distribution->clone()) {}
  ~Vector() = default;

  size_type size() const { return _size; }
  detail::Sizes sizes() const {
    detail::Sizes s;
    s.push_back(_size);
    return s;
  }
  value_type operator[](size_type n) const { return Index(n); }
  value_type at(size_type n) const { return Index(n); }
  value_type front() const { return Index(0); }
  value_type back() const { return Index(_size ? _size - 1 : 0); }

  detail::Distribution<Vector<Index>>& distribution() const { return *_distribution; }
  template <typename U>
  void setDistribution(const detail::Distribution<Vector<U>>& d) const {
    _distribution = detail::cloneAndConvert<Vector<Index>>(d);
  }
  template <typename U>
  void setDistribution(const std::unique_ptr<detail::Distribution<Vector<U>>>& d) const {
    _distribution = detail::cloneAndConvert<Vector<Index>>(*d);
  }
  void setDistribution(std::unique_ptr<detail::Distribution<Vector<Index>>>&& d) const {
    _distribution = std::move(d);
  }
  static std::string deviceFunctions() { return std::string(); }
  void dataOnDeviceModified() const {}
  void dataOnHostModified() const {}

private:
  Vector() = delete;
  Vector<Index>& operator=(const Vector<Index>&) = delete;
  size_type _size;
  mutable std::unique_ptr<detail::Distribution<Vector<Index>>> _distribution;
};

typedef const Vector<Index> IndexVector;

}  // namespace skelcl

#endif  // SKELCL_INDEX_VECTOR_H_
