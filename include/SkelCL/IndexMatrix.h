// Matrix<IndexPoint>: the virtual 2D index space (include/SkelCL/IndexMatrix.h
// of the reference).  IndexPoint(row, column); nothing is stored or uploaded.
#ifndef SKELCL_INDEX_MATRIX_H_
#define SKELCL_INDEX_MATRIX_H_

#include <memory>

#include "Distributions.h"
#include "Index.h"
#include "Matrix.h"

namespace skelcl {

template <>
class Matrix<IndexPoint> {
public:
  typedef IndexPoint value_type;
  typedef MatrixSize size_type;

  Matrix(const size_type size)
      : _size(size), _distribution(new detail::Distribution<Matrix<IndexPoint>>()) {}
  Matrix(const Matrix<IndexPoint>& rhs)
      : _size(rhs._size), _distribution(rhs._distribution->clone()) {}
  ~Matrix() = default;

  size_type size() const { return _size; }
  typename size_type::size_type rowCount() const { return _size.rowCount(); }
  typename size_type::size_type columnCount() const { return _size.columnCount(); }
  value_type operator[](size_t n) const {
    return IndexPoint(Index(n / _size.columnCount()), Index(n % _size.columnCount()));
  }
  value_type at(size_t n) const { return (*this)[n]; }
  value_type front() const { return IndexPoint(Index(0), Index(0)); }
  value_type back() const {
    return IndexPoint(Index(_size.rowCount() - 1), Index(_size.columnCount() - 1));
  }

  detail::Distribution<Matrix<IndexPoint>>& distribution() const { return *_distribution; }
  template <typename U>
  void setDistribution(const detail::Distribution<Matrix<U>>& d) const {
    _distribution = detail::cloneAndConvert<Matrix<IndexPoint>>(d);
  }
  template <typename U>
  void setDistribution(const std::unique_ptr<detail::Distribution<Matrix<U>>>& d) const {
    _distribution = detail::cloneAndConvert<Matrix<IndexPoint>>(*d);
  }
  void setDistribution(std::unique_ptr<detail::Distribution<Matrix<IndexPoint>>>&& d) const {
    _distribution = std::move(d);
  }
  static std::string deviceFunctions() { return std::string(); }
  void dataOnDeviceModified() const {}
  void dataOnHostModified() const {}

private:
  Matrix() = delete;
  Matrix<IndexPoint>& operator=(const Matrix<IndexPoint>&) = delete;
  size_type _size;
  mutable std::unique_ptr<detail::Distribution<Matrix<IndexPoint>>> _distribution;
};

typedef const Matrix<IndexPoint> IndexMatrix;

}  // namespace skelcl

#endif  // SKELCL_INDEX_MATRIX_H_
