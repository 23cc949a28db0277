// skelcl::Matrix<T>: a row-major matrix in a host std::vector<T>, mirrored
// lazily on the GB300 (include/SkelCL/Matrix.h:69-445,
// include/SkelCL/detail/MatrixDef.h:72-867 of the reference).  Same
// coherence rules as Vector; m[row][col] and m({row, col}) address elements.
// As an extra skeleton argument a Matrix<T> arrives in the user function as
// T_matrix_t (data pointer + column count) read with get(m, row, col).
#ifndef SKELCL_MATRIX_H_
#define SKELCL_MATRIX_H_

#include <initializer_list>
#include <memory>
#include <string>
#include <vector>

#include <pvsutil/Assert.h>

#include "Distributions.h"
#include "Source.h"
#include "Vector.h"
#include "detail/Runtime.h"
#include "detail/Util.h"

namespace skelcl {

class MatrixSize {
public:
  typedef size_t size_type;
  MatrixSize(size_type rowCount, size_type columnCount) : _rows(rowCount), _cols(columnCount) {}
  size_type elemCount() const { return _rows * _cols; }
  size_type rowCount() const { return _rows; }
  size_type columnCount() const { return _cols; }
  bool operator==(const MatrixSize& r) const { return _rows == r._rows && _cols == r._cols; }
  bool operator!=(const MatrixSize& r) const { return !(*this == r); }
  bool operator<(const MatrixSize& r) const { return elemCount() < r.elemCount(); }
  bool operator>(const MatrixSize& r) const { return elemCount() > r.elemCount(); }
  bool operator<=(const MatrixSize& r) const { return elemCount() <= r.elemCount(); }
  bool operator>=(const MatrixSize& r) const { return elemCount() >= r.elemCount(); }

private:
  size_type _rows;
  size_type _cols;
};

inline std::ostream& operator<<(std::ostream& os, const MatrixSize& s) {
  return os << s.rowCount() << "x" << s.columnCount();
}

namespace detail {
// T_matrix_t for element types the device prelude does not predefine; the
// guard macro makes repeated registrations harmless (MatrixDef.h:834-867).
template <typename T>
std::string matrixDeviceFunctions(const std::string& type) {
  std::string t = type;
  for (char& c : t)
    if (c == ' ') c = '_';
  return "#ifndef " + t + "_MATRIX_T\ntypedef struct {\n  " + type + "* data;\n"
         "  unsigned int col_count;\n} " + t + "_matrix_t;\n#define " + t + "_MATRIX_T\n#endif\n";
}
}  // namespace detail

template <typename T>
class Matrix {
public:
  typedef std::vector<T> host_buffer_type;
  typedef typename host_buffer_type::value_type value_type;
  typedef typename host_buffer_type::pointer pointer;
  typedef typename host_buffer_type::const_pointer const_pointer;
  typedef typename host_buffer_type::reference reference;
  typedef typename host_buffer_type::const_reference const_reference;
  typedef typename host_buffer_type::iterator iterator;
  typedef typename host_buffer_type::const_iterator const_iterator;
  typedef MatrixSize size_type;
  typedef typename host_buffer_type::difference_type difference_type;
  typedef typename host_buffer_type::allocator_type allocator_type;

  struct coordinate {
    typedef size_type::size_type index_type;
    index_type rowIndex;
    index_type columnIndex;
  };

  Matrix() : _size(0, 0), _distribution(new detail::Distribution<Matrix<T>>()) { registerType(); }

  Matrix(const size_type size, const value_type& value = value_type(),
         const detail::Distribution<Matrix<T>>& distribution = detail::Distribution<Matrix<T>>())
      : _size(size), _distribution(distribution.clone()), _deviceUpToDate(false),
        _host(size.elemCount(), value) {
    registerType();
  }

  // rows = ceil(vector.size() / columnCount); the last row is padded with T()
  // (MatrixDef.h:108-130)
  Matrix(const std::vector<T>& vector, const typename size_type::size_type columnCount,
         const detail::Distribution<Matrix<T>>& distribution = detail::Distribution<Matrix<T>>())
      : _size(0, 0), _distribution(distribution.clone()), _deviceUpToDate(false), _host(vector) {
    registerType();
    ASSERT(columnCount > 0);
    size_t rows = vector.size() / columnCount + (vector.size() % columnCount ? 1 : 0);
    _size = size_type(rows, columnCount);
    _host.resize(_size.elemCount());
  }

  Matrix(const std::vector<T>& vector, const size_type size,
         const detail::Distribution<Matrix<T>>& distribution = detail::Distribution<Matrix<T>>())
      : _size(size), _distribution(distribution.clone()), _deviceUpToDate(false), _host(vector) {
    registerType();
    _host.resize(_size.elemCount());
  }

  static Matrix<T> from2DVector(const std::vector<std::vector<T>>& m,
                                const detail::Distribution<Matrix<T>>& distribution =
                                    detail::Distribution<Matrix<T>>()) {
    std::vector<T> flat;
    size_t cols = m.empty() ? 0 : m.front().size();
    for (auto& row : m) {
      ASSERT(row.size() == cols);
      flat.insert(flat.end(), row.begin(), row.end());
    }
    return Matrix<T>(flat, size_type(m.size(), cols), distribution);
  }

  template <class InputIterator>
  Matrix(InputIterator first, InputIterator last, const typename size_type::size_type columnCount,
         const detail::Distribution<Matrix<T>>& distribution = detail::Distribution<Matrix<T>>())
      : Matrix(std::vector<T>(first, last), columnCount, distribution) {}

  template <class InputIterator>
  Matrix(InputIterator first, InputIterator last, const size_type size,
         const detail::Distribution<Matrix<T>>& distribution = detail::Distribution<Matrix<T>>())
      : Matrix(std::vector<T>(first, last), size, distribution) {}

  Matrix(Matrix<T>&& rhs) noexcept
      : _size(rhs._size),
        _distribution(std::move(rhs._distribution)),
        _hostUpToDate(rhs._hostUpToDate),
        _deviceUpToDate(rhs._deviceUpToDate),
        _host(std::move(rhs._host)),
        _device(std::move(rhs._device)) {
    rhs._size = size_type(0, 0);
    rhs._distribution.reset(new detail::Distribution<Matrix<T>>());
    rhs._hostUpToDate = rhs._deviceUpToDate = true;
  }
  Matrix<T>& operator=(Matrix<T>&& rhs) noexcept {
    if (this == &rhs) return *this;
    _size = rhs._size;
    _distribution = std::move(rhs._distribution);
    _hostUpToDate = rhs._hostUpToDate;
    _deviceUpToDate = rhs._deviceUpToDate;
    _host = std::move(rhs._host);
    _device = std::move(rhs._device);
    rhs._size = size_type(0, 0);
    rhs._distribution.reset(new detail::Distribution<Matrix<T>>());
    rhs._hostUpToDate = rhs._deviceUpToDate = true;
    return *this;
  }
  ~Matrix() = default;

  // ---- element access ---------------------------------------------------------------
  iterator begin() { copyDataToHost(); return _host.begin(); }
  const_iterator begin() const { copyDataToHost(); return _host.begin(); }
  iterator end() { copyDataToHost(); return _host.end(); }
  const_iterator end() const { copyDataToHost(); return _host.end(); }
  iterator row_begin(typename coordinate::index_type r) { return begin() + r * _size.columnCount(); }
  const_iterator row_begin(typename coordinate::index_type r) const {
    return begin() + r * _size.columnCount();
  }
  iterator row_end(typename coordinate::index_type r) { return row_begin(r) + _size.columnCount(); }
  const_iterator row_end(typename coordinate::index_type r) const {
    return row_begin(r) + _size.columnCount();
  }
  iterator operator[](typename coordinate::index_type r) { return row_begin(r); }
  const_iterator operator[](typename coordinate::index_type r) const { return row_begin(r); }

  size_type size() const { return _size; }
  typename size_type::size_type rowCount() const { return _size.rowCount(); }
  typename size_type::size_type columnCount() const { return _size.columnCount(); }
  typename size_type::size_type max_size() const { return _host.max_size(); }
  void resize(const size_type& size, T c = T()) {
    copyDataToHost();
    std::vector<T> nh(size.elemCount(), c);
    for (size_t r = 0; r < std::min(size.rowCount(), _size.rowCount()); ++r)
      for (size_t col = 0; col < std::min(size.columnCount(), _size.columnCount()); ++col)
        nh[r * size.columnCount() + col] = _host[r * _size.columnCount() + col];
    _host.swap(nh);
    _size = size;
    hostChanged();
  }
  typename size_type::size_type capacity() const { return _host.capacity(); }
  bool empty() const { return _size.elemCount() == 0; }
  void reserve(typename size_type::size_type n) { _host.reserve(n); }

  reference operator()(coordinate c) {
    copyDataToHost();
    return _host[c.rowIndex * _size.columnCount() + c.columnIndex];
  }
  const_reference operator()(coordinate c) const {
    copyDataToHost();
    return _host[c.rowIndex * _size.columnCount() + c.columnIndex];
  }
  reference at(coordinate c) {
    ASSERT(c.rowIndex < rowCount() && c.columnIndex < columnCount());
    return (*this)(c);
  }
  const_reference at(coordinate c) const {
    ASSERT(c.rowIndex < rowCount() && c.columnIndex < columnCount());
    return (*this)(c);
  }
  reference front() { copyDataToHost(); return _host.front(); }
  const_reference front() const { copyDataToHost(); return _host.front(); }
  reference back() { copyDataToHost(); return _host.back(); }
  const_reference back() const { copyDataToHost(); return _host.back(); }

  // ---- modifiers -------------------------------------------------------------------------
  template <class InputIterator>
  void assign(InputIterator first, InputIterator last) {
    copyDataToHost();
    std::copy(first, last, _host.begin());
    hostChanged();
  }
  void assign(size_type size, const T& v) {
    _host.assign(size.elemCount(), v);
    _size = size;
    hostChanged();
  }
  template <class InputIterator>
  void push_back_row(InputIterator first, InputIterator last) {
    copyDataToHost();
    std::vector<T> row(first, last);
    if (_size.columnCount() == 0) _size = size_type(0, row.size());
    ASSERT(row.size() == _size.columnCount());
    _host.insert(_host.end(), row.begin(), row.end());
    _size = size_type(_size.rowCount() + 1, _size.columnCount());
    hostChanged();
  }
  void push_back_row(std::initializer_list<T> list) { push_back_row(list.begin(), list.end()); }
  void pop_back_row() {
    copyDataToHost();
    if (_size.rowCount() == 0) return;
    _host.resize(_host.size() - _size.columnCount());
    _size = size_type(_size.rowCount() - 1, _size.columnCount());
    hostChanged();
  }
  template <class InputIterator>
  void insert_row(typename coordinate::index_type rowIndex, InputIterator first, InputIterator last) {
    copyDataToHost();
    std::vector<T> row(first, last);
    ASSERT(row.size() == _size.columnCount());
    _host.insert(_host.begin() + rowIndex * _size.columnCount(), row.begin(), row.end());
    _size = size_type(_size.rowCount() + 1, _size.columnCount());
    hostChanged();
  }
  void insert_row(typename coordinate::index_type rowIndex, std::initializer_list<T> list) {
    insert_row(rowIndex, list.begin(), list.end());
  }
  iterator erase_row(typename coordinate::index_type rowIndex) {
    copyDataToHost();
    auto it = _host.erase(_host.begin() + rowIndex * _size.columnCount(),
                          _host.begin() + (rowIndex + 1) * _size.columnCount());
    _size = size_type(_size.rowCount() - 1, _size.columnCount());
    hostChanged();
    return it;
  }
  void clear() {
    _host.clear();
    _size = size_type(0, 0);
    hostChanged();
  }

  // ---- distributions (one device) ----------------------------------------------------------
  detail::Distribution<Matrix<T>>& distribution() const { return *_distribution; }
  template <typename U>
  void setDistribution(const detail::Distribution<Matrix<U>>& d) const {
    _distribution = detail::cloneAndConvert<Matrix<T>>(d);
  }
  template <typename U>
  void setDistribution(const std::unique_ptr<detail::Distribution<Matrix<U>>>& d) const {
    _distribution = detail::cloneAndConvert<Matrix<T>>(*d);
  }
  void setDistribution(std::unique_ptr<detail::Distribution<Matrix<T>>>&& d) const {
    _distribution = std::move(d);
  }

  // ---- host/device coherence -------------------------------------------------------------------
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
    if (!_device || !_device->valid()) {
      _hostUpToDate = true;
      return;
    }
    _host.resize(_size.elemCount());
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
  static std::string deviceFunctions() {
    return detail::matrixDeviceFunctions<T>(detail::typeName<T>());
  }

  T* devicePtr() const {
    copyDataToDevices();
    return static_cast<T*>(_device->get());
  }
  T* deviceOutputPtr() const {
    createDeviceBuffers();
    return static_cast<T*>(_device->get());
  }

private:
  // T_matrix_t of this element type joins the common definitions once
  // (the reference registers it from a static member, MatrixDef.h:72-76).
  static void registerType() {
    static const bool done = [] {
      detail::CommonDefinitions::append(deviceFunctions(),
                                        detail::CommonDefinitions::GENERATED_DEFINITION);
      return true;
    }();
    (void)done;
  }
  Matrix(const Matrix<T>&) = delete;
  Matrix<T>& operator=(const Matrix<T>&) = delete;
  size_t bytes() const { return _size.elemCount() * sizeof(T); }
  void hostChanged() {
    _hostUpToDate = true;
    _deviceUpToDate = false;
    _device.reset();
  }

  MatrixSize _size;
  mutable std::unique_ptr<detail::Distribution<Matrix<T>>> _distribution;
  mutable bool _hostUpToDate = true;
  mutable bool _deviceUpToDate = true;
  mutable host_buffer_type _host;
  mutable std::shared_ptr<detail::DeviceBuffer> _device;
};

}  // namespace skelcl

#endif  // SKELCL_MATRIX_H_
