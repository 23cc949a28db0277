// Map skeletons (include/SkelCL/Map.h:129-640, detail/MapDef.h:75-752 and
// src/Map.cpp of the reference), all six specialisations:
//   Map<Tout(Tin)>, Map<void(Tin)>            over Vector / Matrix
//   Map<Tout(Index)>, Map<void(Index)>        over IndexVector
//   Map<Tout(IndexPoint)>, Map<void(IndexPoint)> over IndexMatrix
// The user function (OpenCL C source) is spliced into the sm_103a Map
// template and compiled with NVRTC when the skeleton is constructed.
#ifndef SKELCL_MAP_H_
#define SKELCL_MAP_H_

#include <string>

#include "Index.h"
#include "IndexMatrix.h"
#include "IndexVector.h"
#include "Matrix.h"
#include "Out.h"
#include "Source.h"
#include "Vector.h"
#include "detail/Skeleton.h"

namespace skelcl {

template <typename> class Map;

template <typename Tin, typename Tout>
class Map<Tout(Tin)> : public detail::Skeleton {
public:
  Map(const Source& source, const std::string& funcName = std::string("func"))
      : _source(source), _func(funcName) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_MAP;
    s.source = _source;
    s.func = funcName;
    s.types = {detail::typeName<Tin>(), detail::typeName<Tout>()};
    _program = s.build();
  }

  template <template <typename> class C, typename... Args>
  C<Tout> operator()(const C<Tin>& input, Args&&... args) const {
    C<Tout> output;
    (*this)(out(output), input, std::forward<Args>(args)...);
    return output;
  }

  template <template <typename> class C, typename... Args>
  C<Tout>& operator()(Out<C<Tout>> output, const C<Tin>& input, Args&&... args) const {
    C<Tout>& o = output.container();
    if ((const void*)&o != (const void*)&input) detail::resizeLike(o, input);
    void* bufs[2];
    bufs[0] = input.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[1] = o.deviceOutputPtr();
    scl_shape sh = detail::makeShape(detail::elementCount(input));
    scl_tuning t = tuning();
    launched(scl_launch_map(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Map");
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

template <typename Tin>
class Map<void(Tin)> : public detail::Skeleton {
public:
  Map(const Source& source, const std::string& funcName = std::string("func")) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_MAP_VOID;
    s.source = source;
    s.func = funcName;
    s.types = {detail::typeName<Tin>()};
    _program = s.build();
  }

  template <template <typename> class C, typename... Args>
  void operator()(const C<Tin>& input, Args&&... args) const {
    void* bufs[1];
    bufs[0] = input.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    scl_shape sh = detail::makeShape(detail::elementCount(input));
    scl_tuning t = tuning();
    launched(scl_launch_map(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Map");
    detail::markModified(args...);
  }

private:
  detail::Program _program;
};

template <typename Tout>
class Map<Tout(Index)> : public detail::Skeleton {
public:
  Map(const Source& source, const std::string& funcName = std::string("func")) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_MAP_INDEX;
    s.source = source;
    s.func = funcName;
    s.types = {detail::typeName<Tout>()};
    _program = s.build();
  }

  template <typename... Args>
  Vector<Tout> operator()(const Vector<Index>& input, Args&&... args) const {
    Vector<Tout> output;
    (*this)(out(output), input, std::forward<Args>(args)...);
    return output;
  }

  template <typename... Args>
  Vector<Tout>& operator()(Out<Vector<Tout>> output, const Vector<Index>& input,
                           Args&&... args) const {
    Vector<Tout>& o = output.container();
    if (o.size() < input.size()) o.resize(input.size());
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    void* bufs[1] = {o.deviceOutputPtr()};
    scl_shape sh = detail::makeShape(input.size());
    scl_tuning t = tuning();
    launched(scl_launch_map(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Map");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

private:
  detail::Program _program;
};

template <>
class Map<void(Index)> : public detail::Skeleton {
public:
  Map(const Source& source, const std::string& funcName = std::string("func")) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_MAP_INDEX_VOID;
    s.source = source;
    s.func = funcName;
    _program = s.build();
  }

  template <typename... Args>
  void operator()(const Vector<Index>& input, Args&&... args) const {
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    scl_shape sh = detail::makeShape(input.size());
    scl_tuning t = tuning();
    launched(scl_launch_map(_program.get(), &sh, nullptr, blob.data(), blob.size(), &t), "Map");
    detail::markModified(args...);
  }

private:
  detail::Program _program;
};

template <typename Tout>
class Map<Tout(IndexPoint)> : public detail::Skeleton {
public:
  Map(const Source& source, const std::string& funcName = std::string("func")) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_MAP_POINT;
    s.source = source;
    s.func = funcName;
    s.types = {detail::typeName<Tout>()};
    _program = s.build();
  }

  template <typename... Args>
  Matrix<Tout> operator()(const Matrix<IndexPoint>& input, Args&&... args) const {
    Matrix<Tout> output;
    (*this)(out(output), input, std::forward<Args>(args)...);
    return output;
  }

  template <typename... Args>
  Matrix<Tout>& operator()(Out<Matrix<Tout>> output, const Matrix<IndexPoint>& input,
                           Args&&... args) const {
    Matrix<Tout>& o = output.container();
    if (o.size() != input.size()) o.resize(input.size());
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    void* bufs[1] = {o.deviceOutputPtr()};
    scl_shape sh = detail::makeShape(0);
    sh.rows = input.rowCount();
    sh.cols = input.columnCount();
    scl_tuning t = tuning();
    launched(scl_launch_map(_program.get(), &sh, bufs, blob.data(), blob.size(), &t), "Map");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

private:
  detail::Program _program;
};

template <>
class Map<void(IndexPoint)> : public detail::Skeleton {
public:
  Map(const Source& source, const std::string& funcName = std::string("func")) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_MAP_POINT_VOID;
    s.source = source;
    s.func = funcName;
    _program = s.build();
  }

  template <typename... Args>
  void operator()(const Matrix<IndexPoint>& input, Args&&... args) const {
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    scl_shape sh = detail::makeShape(0);
    sh.rows = input.rowCount();
    sh.cols = input.columnCount();
    scl_tuning t = tuning();
    launched(scl_launch_map(_program.get(), &sh, nullptr, blob.data(), blob.size(), &t), "Map");
    detail::markModified(args...);
  }

private:
  detail::Program _program;
};

}  // namespace skelcl

#endif  // SKELCL_MAP_H_
