// Fused skeleton pairs (no counterpart in the reference): built from two
// skeleton objects, as AllPairs is built from a Reduce and a Zip, and run as
// one kernel that never writes the intermediate vector.
//
//   skelcl::ZipReduce<float(float, float)> dot(sum, mult);   // Reduce(Zip(x, y))
//   skelcl::Vector<float> d = dot(x, y);                      // one element
//   skelcl::ScanMap<int(int)> sm(scan, mod);                  // Map(Scan(x))
//   skelcl::Vector<int> r = sm(x);
//
// Results equal the unfused pair's (for float folds up to the reassociation
// a Reduce or Scan allows anyway).  Extra arguments: the first skeleton's,
// then the second's.
#ifndef SKELCL_FUSED_H_
#define SKELCL_FUSED_H_

#include <string>

#include <pvsutil/Assert.h>

#include "Map.h"
#include "Out.h"
#include "Reduce.h"
#include "Scan.h"
#include "Vector.h"
#include "Zip.h"
#include "detail/Skeleton.h"

namespace skelcl {

template <typename> class ZipReduce;

template <typename T, typename Tl, typename Tr>
class ZipReduce<T(Tl, Tr)> : public detail::Skeleton {
public:
  ZipReduce(const Reduce<T(T)>& reduce, const Zip<T(Tl, Tr)>& zip) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_ZIP_REDUCE;
    s.source = reduce.source();
    s.func = reduce.func();
    s.source2 = zip.source();
    s.func2 = zip.func();
    s.identity = reduce.id();
    s.types = {detail::typeName<Tl>(), detail::typeName<Tr>(), detail::typeName<T>()};
    _program = s.build();
  }

  template <typename... Args>
  Vector<T> operator()(const Vector<Tl>& left, const Vector<Tr>& right, Args&&... args) const {
    Vector<T> output;
    (*this)(out(output), left, right, std::forward<Args>(args)...);
    return output;
  }

  template <typename... Args>
  Vector<T>& operator()(Out<Vector<T>> output, const Vector<Tl>& left, const Vector<Tr>& right,
                        Args&&... args) const {
    ASSERT_MESSAGE(left.size() <= right.size(), "ZipReduce: the right operand is shorter");
    Vector<T>& o = output.container();
    if (o.size() < 1) o.resize(1);
    void* bufs[3];
    bufs[0] = left.size() ? (void*)left.devicePtr() : nullptr;
    bufs[1] = left.size() ? (void*)right.devicePtr() : nullptr;
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[2] = o.deviceOutputPtr();
    if (!bufs[0]) bufs[0] = bufs[1] = bufs[2];  // empty input: nothing is read
    scl_shape sh = detail::makeShape(left.size());
    scl_tuning t = tuning();
    launched(scl_launch_reduce(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "ZipReduce");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

private:
  detail::Program _program;
};

template <typename> class ScanMap;

template <typename Tout, typename T>
class ScanMap<Tout(T)> : public detail::Skeleton {
public:
  // The scan's inclusive / reverse settings at construction are kept.
  ScanMap(const Scan<T(T)>& scan, const Map<Tout(T)>& map)
      : _inclusive(scan.inclusive()), _reverse(scan.reverse()) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_SCAN_MAP;
    s.source = scan.source();
    s.func = scan.func();
    s.source2 = map.source();
    s.func2 = map.func();
    s.identity = scan.id();
    s.types = {detail::typeName<T>(), detail::typeName<Tout>()};
    _program = s.build();
  }

  template <typename... Args>
  Vector<Tout> operator()(const Vector<T>& input, Args&&... args) const {
    Vector<Tout> output;
    (*this)(out(output), input, std::forward<Args>(args)...);
    return output;
  }

  template <typename... Args>
  Vector<Tout>& operator()(Out<Vector<Tout>> output, const Vector<T>& input, Args&&... args) const {
    Vector<Tout>& o = output.container();
    ASSERT((const void*)&o != (const void*)&input || sizeof(Tout) == sizeof(T));
    if ((const void*)&o != (const void*)&input) detail::resizeLike(o, input.size());
    if (input.size() == 0) return o;
    void* bufs[2];
    bufs[0] = input.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[1] = o.deviceOutputPtr();
    scl_shape sh = detail::makeShape(input.size());
    sh.flags = (_inclusive ? SCL_SHAPE_INCLUSIVE : 0u) | (_reverse ? SCL_SHAPE_REVERSE : 0u);
    scl_tuning t = tuning();
    launched(scl_launch_scan(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "ScanMap");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

private:
  bool _inclusive, _reverse;
  detail::Program _program;
};

}  // namespace skelcl

#endif  // SKELCL_FUSED_H_
