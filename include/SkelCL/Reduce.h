// Reduce<T(T)> (include/SkelCL/Reduce.h:95-224, detail/ReduceDef.h:79-293 of
// the reference): folds a Vector with a user binary function into a Vector of
// one element.  As in the reference the identity string is kept (source(),
// func(), id() feed AllPairs) but does not seed the fold; for an empty input
// the result is the identity.
#ifndef SKELCL_REDUCE_H_
#define SKELCL_REDUCE_H_

#include <string>

#include "Out.h"
#include "Segments.h"
#include "Source.h"
#include "Vector.h"
#include "detail/Skeleton.h"

namespace skelcl {

template <typename> class Reduce;

template <typename T>
class Reduce<T(T)> : public detail::Skeleton {
public:
  Reduce(const Source& source, const std::string& id = std::string("0"),
         const std::string& funcName = std::string("func"))
      : _source(source), _func(funcName), _id(id) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_REDUCE;
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
    void* bufs[2];
    bufs[0] = input.size() ? (void*)input.devicePtr() : nullptr;
    if ((const void*)&o != (const void*)&input && o.size() < 1) o.resize(1);
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[1] = o.deviceOutputPtr();
    if (!bufs[0]) bufs[0] = bufs[1];  // empty input: nothing is read
    scl_shape sh = detail::makeShape(input.size());
    scl_tuning t = tuning();
    launched(scl_launch_reduce(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Reduce");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

  // One result per vector of `segments` (vectors stored back to back in
  // `input`), all in one launch; an empty vector yields the identity.
  template <typename... Args>
  Vector<T>& segmented(Out<Vector<T>> output, const Vector<T>& input, const Segments& segments,
                       Args&&... args) const {
    Vector<T>& o = output.container();
    ASSERT_MESSAGE(segments.total() <= input.size(), "Reduce::segmented: segments beyond the input");
    ASSERT((const void*)&o != (const void*)&input);
    if (o.size() < segments.count()) o.resize(segments.count());
    if (segments.count() == 0) return o;
    void* bufs[2];
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[1] = o.deviceOutputPtr();
    bufs[0] = input.size() ? (void*)input.devicePtr() : bufs[1];
    scl_shape sh = detail::makeShape(input.size());
    sh.seg_offsets = segments.devicePtr();
    sh.n_segments = segments.count();
    sh.seg_plan = segments.plan();
    scl_tuning t = tuning();
    launched(scl_launch_reduce(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Reduce");
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

  std::string source() const { return _source; }
  std::string func() const { return _func; }
  std::string id() const { return _id; }

private:
  std::string _source, _func, _id;
  detail::Program _program;
};

}  // namespace skelcl

#endif  // SKELCL_REDUCE_H_
