// Segments: many vectors of uneven length stored back to back in one
// Vector<T> (no counterpart in the reference).  Scan::segmented and
// Reduce::segmented process all of them with one launch each; Map and Zip
// need nothing special (they are element-wise).
#ifndef SKELCL_SEGMENTS_H_
#define SKELCL_SEGMENTS_H_

#include <cstdint>
#include <vector>

#include <pvsutil/Assert.h>

#include "Vector.h"

namespace skelcl {

class Segments {
public:
  Segments() = default;
  // From the lengths of the vectors, in storage order.
  explicit Segments(const std::vector<size_t>& lengths) {
    std::vector<uint64_t> off(lengths.size() + 1, 0);
    for (size_t i = 0; i < lengths.size(); ++i) off[i + 1] = off[i] + lengths[i];
    _offsets = Vector<uint64_t>(off.begin(), off.end());
  }
  // From offsets: vector s is [offsets[s], offsets[s+1]); non-decreasing.
  static Segments fromOffsets(const std::vector<uint64_t>& offsets) {
    ASSERT_MESSAGE(!offsets.empty(), "Segments: at least one offset");
    Segments s;
    s._offsets = Vector<uint64_t>(offsets.begin(), offsets.end());
    return s;
  }
  size_t count() const { return _offsets.size() ? _offsets.size() - 1 : 0; }
  // total number of elements (the last offset)
  size_t total() const { return _offsets.size() ? (size_t)_offsets.back() : 0; }
  const uint64_t* devicePtr() const { return _offsets.devicePtr(); }

private:
  Vector<uint64_t> _offsets;
};

}  // namespace skelcl

#endif  // SKELCL_SEGMENTS_H_
