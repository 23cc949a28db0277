// Scan<T(T)> (include/SkelCL/Scan.h:80-197, detail/ScanDef.h:70-327 of the
// reference): the EXCLUSIVE prefix scan seeded with the identity `id`
// (default "0").  Extensions beyond the reference, off by default:
// setInclusive(true) gives the inclusive scan (= exclusive scan combined with
// the input), setReverse(true) scans from the last element towards the first
// (the adjoint of a forward sum-scan).  Extra arguments reach the user
// function (the reference declares them but never sets them, ScanDef.h:206).
#ifndef SKELCL_SCAN_H_
#define SKELCL_SCAN_H_

#include <string>

#include "Out.h"
#include "Segments.h"
#include "Source.h"
#include "Vector.h"
#include "detail/Skeleton.h"

namespace skelcl {

template <typename> class Scan;

template <typename T>
class Scan<T(T)> : public detail::Skeleton {
public:
  Scan(const Source& source, const std::string& id = std::string("0"),
       const std::string& funcName = std::string("func"))
      : _source(source), _func(funcName), _id(id) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_SCAN;
    s.source = _source;
    s.func = funcName;
    s.identity = id;
    s.types = {detail::typeName<T>()};
    _program = s.build();
  }

  template <typename... Args>
  Vector<T> operator()(const Vector<T>& input, Args&&... args) const {
    Vector<T> output;
    (*this)(out(output), input, std::forward<Args>(args)...);
    return output;
  }

  template <typename... Args>
  Vector<T>& operator()(Out<Vector<T>> output, const Vector<T>& input, Args&&... args) const {
    Vector<T>& o = output.container();
    if ((const void*)&o != (const void*)&input) detail::resizeLike(o, input);
    if (input.size() == 0) return o;
    void* bufs[2];
    bufs[0] = input.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[1] = o.deviceOutputPtr();
    scl_shape sh = detail::makeShape(input.size());
    sh.flags = (_inclusive ? SCL_SHAPE_INCLUSIVE : 0u) | (_reverse ? SCL_SHAPE_REVERSE : 0u);
    scl_tuning t = tuning();
    launched(scl_launch_scan(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Scan");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

  // One scan per vector of `segments` (vectors stored back to back in
  // `input`), all in one launch.
  template <typename... Args>
  Vector<T>& segmented(Out<Vector<T>> output, const Vector<T>& input, const Segments& segments,
                       Args&&... args) const {
    Vector<T>& o = output.container();
    ASSERT_MESSAGE(segments.total() <= input.size(), "Scan::segmented: segments beyond the input");
    if ((const void*)&o != (const void*)&input) detail::resizeLike(o, input);
    if (input.size() == 0 || segments.count() == 0) return o;
    void* bufs[2];
    bufs[0] = input.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[1] = o.deviceOutputPtr();
    scl_shape sh = detail::makeShape(input.size());
    sh.flags = (_inclusive ? SCL_SHAPE_INCLUSIVE : 0u) | (_reverse ? SCL_SHAPE_REVERSE : 0u);
    sh.seg_offsets = segments.devicePtr();
    sh.n_segments = segments.count();
    sh.seg_plan = segments.plan();
    scl_tuning t = tuning();
    launched(scl_launch_scan(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Scan");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }
  template <typename... Args>
  Vector<T> segmented(const Vector<T>& input, const Segments& segments, Args&&... args) const {
    Vector<T> output;
    segmented(out(output), input, segments, std::forward<Args>(args)...);
    return output;
  }

  Scan& setInclusive(bool inclusive) {
    _inclusive = inclusive;
    return *this;
  }
  Scan& setReverse(bool reverse) {
    _reverse = reverse;
    return *this;
  }
  bool inclusive() const { return _inclusive; }
  bool reverse() const { return _reverse; }
  std::string source() const { return _source; }
  std::string func() const { return _func; }
  std::string id() const { return _id; }

private:
  std::string _source, _func, _id;
  bool _inclusive = false, _reverse = false;
  detail::Program _program;
};

}  // namespace skelcl

#endif  // SKELCL_SCAN_H_
