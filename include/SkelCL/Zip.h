// Zip skeletons (include/SkelCL/Zip.h:96-350, detail/ZipDef.h:70-442 of the
// reference): out[i] = f(left[i], right[i], extra...), and the void form.
#ifndef SKELCL_ZIP_H_
#define SKELCL_ZIP_H_

#include <string>

#include <pvsutil/Assert.h>

#include "Matrix.h"
#include "Out.h"
#include "Source.h"
#include "Vector.h"
#include "detail/Skeleton.h"

namespace skelcl {

template <typename> class Zip;

template <typename Tleft, typename Tright, typename Tout>
class Zip<Tout(Tleft, Tright)> : public detail::Skeleton {
public:
  Zip(const Source& source, const std::string& funcName = std::string("func"))
      : _source(source), _func(funcName) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_ZIP;
    s.source = _source;
    s.func = funcName;
    s.types = {detail::typeName<Tleft>(), detail::typeName<Tright>(), detail::typeName<Tout>()};
    _program = s.build();
  }

  template <template <typename> class C, typename... Args>
  C<Tout> operator()(const C<Tleft>& left, const C<Tright>& right, Args&&... args) const {
    C<Tout> output;
    (*this)(out(output), left, right, std::forward<Args>(args)...);
    return output;
  }

  template <template <typename> class C, typename... Args>
  C<Tout>& operator()(Out<C<Tout>> output, const C<Tleft>& left, const C<Tright>& right,
                      Args&&... args) const {
    ASSERT(detail::elementCount(left) <= detail::elementCount(right));  // ZipDef.h:101
    C<Tout>& o = output.container();
    if ((const void*)&o != (const void*)&left && (const void*)&o != (const void*)&right)
      detail::resizeLike(o, left);
    void* bufs[3];
    bufs[0] = left.devicePtr();
    bufs[1] = right.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[2] = o.deviceOutputPtr();
    scl_shape sh = detail::makeShape(detail::elementCount(left));
    scl_tuning t = tuning();
    launched(scl_launch_zip(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Zip");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

  std::string source() const { return _source; }
  std::string func() const { return _func; }

private:
  std::string _source, _func;
  detail::Program _program;
};

template <typename Tleft, typename Tright>
class Zip<void(Tleft, Tright)> : public detail::Skeleton {
public:
  Zip(const Source& source, const std::string& funcName = std::string("func"))
      : _source(source), _func(funcName) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_ZIP_VOID;
    s.source = _source;
    s.func = funcName;
    s.types = {detail::typeName<Tleft>(), detail::typeName<Tright>()};
    _program = s.build();
  }

  template <template <typename> class C, typename... Args>
  void operator()(const C<Tleft>& left, const C<Tright>& right, Args&&... args) const {
    ASSERT(detail::elementCount(left) <= detail::elementCount(right));
    void* bufs[2];
    bufs[0] = left.devicePtr();
    bufs[1] = right.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    scl_shape sh = detail::makeShape(detail::elementCount(left));
    scl_tuning t = tuning();
    launched(scl_launch_zip(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Zip");
    detail::markModified(args...);
  }

  std::string source() const { return _source; }
  std::string func() const { return _func; }

private:
  std::string _source, _func;
  detail::Program _program;
};

}  // namespace skelcl

#endif  // SKELCL_ZIP_H_
