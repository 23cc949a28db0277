// Index and IndexPoint (include/SkelCL/Index.h:54-140 of the reference).
// On the device an Index is a size_t and an IndexPoint a struct {x, y} with
// x = column and y = row.
#ifndef SKELCL_INDEX_H_
#define SKELCL_INDEX_H_

#include <cstddef>
#include <ostream>
#include <utility>

namespace skelcl {

class Index {
public:
  typedef size_t index_type;
  Index() : _index(0) {}
  Index(const index_type index) : _index(index) {}
  bool operator==(const Index& rhs) const { return _index == rhs._index; }
  bool operator!=(const Index& rhs) const { return _index != rhs._index; }
  operator index_type() const { return _index; }
  index_type get() const { return _index; }

private:
  index_type _index;
};

class IndexPoint {
public:
  typedef std::pair<Index, Index> indexPoint_type;
  IndexPoint() : _p(Index(0), Index(0)) {}
  IndexPoint(const indexPoint_type& p) : _p(p) {}
  IndexPoint(const IndexPoint& rhs) = default;
  IndexPoint(const Index& row, const Index& column) : _p(row, column) {}
  IndexPoint(IndexPoint&& rhs) = default;
  IndexPoint& operator=(IndexPoint&& rhs) = default;
  IndexPoint& operator=(const IndexPoint& rhs) = default;
  bool operator==(const IndexPoint& rhs) const { return _p == rhs._p; }
  bool operator!=(const IndexPoint& rhs) const { return _p != rhs._p; }
  operator indexPoint_type() const { return _p; }
  indexPoint_type get() const { return _p; }
  const Index& rowID() const { return _p.first; }
  const Index& y() const { return _p.first; }
  const Index& columnID() const { return _p.second; }
  const Index& x() const { return _p.second; }

private:
  indexPoint_type _p;
};

inline std::ostream& operator<<(std::ostream& os, const IndexPoint& p) {
  return os << "(" << p.rowID().get() << ", " << p.columnID().get() << ")";
}

}  // namespace skelcl

#endif  // SKELCL_INDEX_H_
