// Segments: many vectors of uneven length stored back to back in one
// Vector<T> (no counterpart in the reference).  Scan::segmented and
// Reduce::segmented process all of them with one launch each; Map and Zip
// need nothing special (they are element-wise).
#ifndef SKELCL_SEGMENTS_H_
#define SKELCL_SEGMENTS_H_

#include <cstdint>
#include <memory>
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
  // The segment plan of these offsets (scl_segplan_create), made on first
  // use and shared by copies: with it a segmented Scan or Reduce is one
  // launch and the offsets pre-pass runs once, not on every call.  The
  // offsets never change after construction, so the plan stays valid.
  uint32_t plan() const {
    if (!_plan && count()) {
      uint32_t id = 0;
      if (scl_segplan_create(devicePtr(), count(), total(), &id) == SCL_OK && id)
        _plan = std::shared_ptr<uint32_t>(new uint32_t(id), [](uint32_t* p) {
          scl_segplan_release(*p);
          delete p;
        });
    }
    return _plan ? *_plan : 0u;
  }

private:
  Vector<uint64_t> _offsets;
  mutable std::shared_ptr<uint32_t> _plan;
};

}  // namespace skelcl

#endif  // SKELCL_SEGMENTS_H_
