// AllPairs<Tout(Tl,Tr)> (include/SkelCL/AllPairs.h:115-263,
// detail/AllPairsDef.h:77-426 of the reference).
//
// From a Reduce and a Zip:  P[i][j] = id (+) z(A[i][0], B[0][j]) (+) ...
// (+) z(A[i][K-1], B[K-1][j]), folded in k order; extra arguments are the
// Reduce's first, then the Zip's.  When the pair is x*y / x+y over float with
// identity 0 the contraction runs on the tcgen05 tensor cores (3xBF16 split,
// FP32 accumulation); setPrecise(true) keeps it on the CUDA-core kernel.
// From one user function f(lmatrix_t*, rmatrix_t*, dim, ...): P[i][j] =
// f(row i of A, column j of B), with getElementFromRow / getElementFromColumn.
#ifndef SKELCL_ALLPAIRS_H_
#define SKELCL_ALLPAIRS_H_

#include <string>

#include <pvsutil/Assert.h>

#include "Matrix.h"
#include "Out.h"
#include "Reduce.h"
#include "Source.h"
#include "Zip.h"
#include "detail/Skeleton.h"

namespace skelcl {

template <typename> class AllPairs;

template <typename Tleft, typename Tright, typename Tout>
class AllPairs<Tout(Tleft, Tright)> : public detail::Skeleton {
public:
  AllPairs(const Reduce<Tout(Tout)>& reduce, const Zip<Tout(Tleft, Tright)>& zip) : _special(true) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_ALLPAIRS;
    s.source = reduce.source();
    s.func = reduce.func();
    s.source2 = zip.source();
    s.func2 = zip.func();
    s.identity = reduce.id();
    s.types = {detail::typeName<Tleft>(), detail::typeName<Tright>(), detail::typeName<Tout>()};
    _program = s.build();
  }

  AllPairs(const std::string& source, const std::string& func = std::string("func"))
      : _special(false) {
    detail::ProgramSpec s;
    s.kind = SCL_KIND_ALLPAIRS_GENERIC;
    s.source = source;
    s.func = func;
    s.types = {detail::typeName<Tleft>(), detail::typeName<Tright>(), detail::typeName<Tout>()};
    _program = s.build();
  }

  template <typename... Args>
  Matrix<Tout> operator()(const Matrix<Tleft>& left, const Matrix<Tright>& right,
                          Args&&... args) const {
    Matrix<Tout> output;
    (*this)(out(output), left, right, std::forward<Args>(args)...);
    return output;
  }

  template <typename... Args>
  Matrix<Tout>& operator()(Out<Matrix<Tout>> output, const Matrix<Tleft>& left,
                           const Matrix<Tright>& right, Args&&... args) const {
    ASSERT(left.rowCount() > 0 && right.columnCount() > 0);
    ASSERT(left.columnCount() == right.rowCount());
    ASSERT(left.columnCount() > 0);
    Matrix<Tout>& o = output.container();
    const MatrixSize want(left.rowCount(), right.columnCount());
    if (o.size() != want) o.resize(want);
    void* bufs[3];
    bufs[0] = left.devicePtr();
    bufs[1] = right.devicePtr();
    detail::prepareArgs(args...);
    detail::ArgBlob blob = detail::packArgs(args...);
    bufs[2] = o.deviceOutputPtr();
    scl_shape sh = detail::makeShape(0);
    sh.rows = left.rowCount();
    sh.cols = right.columnCount();
    sh.dim = left.columnCount();
    scl_tuning t = tuning();
    if (_precise) t.variant = SCL_VARIANT_SIMT;
    launched(scl_launch_allpairs(_program.get(), &sh, bufs, blob.data(), blob.size(), &t),
             "AllPairs");
    o.dataOnDeviceModified();
    detail::markModified(args...);
    return o;
  }

  // Keep the Reduce(+)/Zip(*) contraction on the CUDA cores (sequential FP32
  // fold in k order) instead of the tensor cores.
  AllPairs& setPrecise(bool precise) {
    _precise = precise;
    return *this;
  }
  // Variant the last call used (SCL_VARIANT_SIMT or SCL_VARIANT_TC3XBF16).
  uint32_t lastVariant() const {
    uint32_t v = 0;
    scl_program_last_variant(_program.get(), &v);
    return v;
  }

private:
  bool _special;
  bool _precise = false;
  detail::Program _program;
};

}  // namespace skelcl

#endif  // SKELCL_ALLPAIRS_H_
