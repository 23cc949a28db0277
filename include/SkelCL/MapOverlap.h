// MapOverlap<Tout(Tin)> (include/SkelCL/MapOverlap.h:103-188,
// detail/MapOverlapDef.h:71-279 of the reference): a 2D stencil over a
// Matrix.  The user function receives an input_matrix_t view and reads
// neighbours with getData(view, dx, dy), dx along columns and dy along rows,
// |dx|, |dy| <= overlap range.  Padding NEAREST clamps to the edge, NEUTRAL
// reads the neutral element outside the matrix.
#ifndef SKELCL_MAPOVERLAP_H_
#define SKELCL_MAPOVERLAP_H_

#include <string>

#include <pvsutil/Assert.h>

#include "Matrix.h"
#include "Out.h"
#include "Source.h"
#include "detail/Padding.h"
#include "detail/Skeleton.h"

namespace skelcl {

template <typename> class MapOverlap;

template <typename Tin, typename Tout>
class MapOverlap<Tout(Tin)> : public detail::Skeleton {
public:
  MapOverlap(const Source& source, unsigned overlap_range = 1,
             detail::Padding padding = detail::Padding::NEAREST, Tin neutral_element = Tin(),
             const std::string& func = std::string("func"))
      : _source(source), _func(func), _range(overlap_range), _padding(padding) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_MAPOVERLAP;
    s.source = _source;
    s.func = func;
    s.overlapRange = (int)overlap_range;
    s.padding = padding == detail::Padding::NEUTRAL ? SCL_PAD_NEUTRAL : SCL_PAD_NEAREST;
    s.neutral = detail::sourceLiteral(neutral_element);
    s.types = {detail::typeName<Tin>(), detail::typeName<Tout>()};
    _program = s.build();
  }

  template <typename... Args>
  Matrix<Tout> operator()(const Matrix<Tin>& in, Args&&... args) const {
    Matrix<Tout> output;
    (*this)(out(output), in, std::forward<Args>(args)...);
    return output;
  }

  template <typename... Args>
  Matrix<Tout>& operator()(Out<Matrix<Tout>> output, const Matrix<Tin>& in, Args&&... args) const {
    ASSERT(in.rowCount() > 0 && in.columnCount() > 0);
    Matrix<Tout>& o = output.container();
    ASSERT((const void*)&o != (const void*)&in);  // the stencil reads neighbours: no in-place form
    if (o.size() != in.size()) o.resize(in.size());
    void* bufs[2];
    bufs[0] = in.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[1] = o.deviceOutputPtr();
    scl_shape sh = detail::makeShape(0);
    sh.rows = in.rowCount();
    sh.cols = in.columnCount();
    scl_tuning t = tuning();
    launched(scl_launch_mapoverlap(_program.get(), &sh, bufs, blob.data(), blob.size(), &t),
             "MapOverlap");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

  unsigned overlapRange() const { return _range; }
  detail::Padding padding() const { return _padding; }
  std::string source() const { return _source; }
  std::string func() const { return _func; }

private:
  std::string _source, _func;
  unsigned _range;
  detail::Padding _padding;
  detail::Program _program;
};

}  // namespace skelcl

#endif  // SKELCL_MAPOVERLAP_H_
