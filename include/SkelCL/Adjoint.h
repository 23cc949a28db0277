// Reverse-mode differentiation of skeleton programs: a small tape and the
// adjoint skeletons behind it (no counterpart in the reference).
//
//   skelcl::ad::Tape tape;
//   auto x = tape.variable(xs);                          // a Vector<float> input
//   skelcl::ad::Map<float(float)> sq("float func(float x){ return x*x + 1.0f; }",
//                                    "float dfunc(float x, float g){ return 2.0f*x*g; }");
//   skelcl::ad::Scan<float> scan("float func(float x, float y){ return x + y; }");
//   skelcl::ad::Reduce<float> sum("float func(float x, float y){ return x + y; }");
//   auto loss = sum(tape, scan(tape, sq(tape, x)));
//   tape.backward(loss);                                 // seeds d loss = 1
//   x.grad();                                            // d loss / d xs
//
// Forward calls run immediately (they are the ordinary skeletons); each call
// also records its adjoint, and Tape::backward runs the adjoints in reverse:
//   Map / Zip         the user's vector-Jacobian product, spliced into the
//                     element-wise adjoint kernel: d(x, g) -> dx
//                     (dl(x, y, g) -> dx, dr(x, y, g) -> dy for Zip)
//   Reduce (+)        a broadcast of the output gradient
//                     (.segmented: per vector of a Segments, one launch)
//   Scan (+)          the reverse scan of the output gradient
//                     (.segmented: the segmented reverse scan, one launch)
//   MapOverlap        (linear, float) the transposed stencil: the weights are
//                     read back by running the forward on an impulse, the
//                     adjoint is a zero-padded MapOverlap with them, plus the
//                     edge fold for NEAREST padding
//   AllPairs (x*y, +) two AllPairs: dA = G B^T, dB = A^T G (transposed
//                     operands read in place)
// Gradients of a value used several times are summed.  Extra arguments are
// captured (device pointers, scalar bytes) when the forward runs: containers
// passed as extra arguments must stay alive and unchanged until backward().
#ifndef SKELCL_ADJOINT_H_
#define SKELCL_ADJOINT_H_

#include <cctype>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "Matrix.h"
#include "Reduce.h"
#include "Segments.h"
#include "Source.h"
#include "Vector.h"
#include "Zip.h"
#include "detail/Padding.h"
#include "detail/Skeleton.h"

namespace skelcl {
namespace ad {

namespace detail {

template <typename T> struct DType;
template <> struct DType<float> { static constexpr int value = SCL_DTYPE_F32; };
template <> struct DType<double> { static constexpr int value = SCL_DTYPE_F64; };

// True when function `func` of `src` is `return a <op> b;` over its two
// parameters (either order).
inline bool isBinaryOp(const std::string& src, const std::string& func, char op) {
  size_t at = src.find(func);
  while (at != std::string::npos) {
    const bool left_ok = at == 0 || !(std::isalnum((unsigned char)src[at - 1]) || src[at - 1] == '_');
    const size_t after = at + func.size();
    const bool right_ok = after < src.size() && !(std::isalnum((unsigned char)src[after]) || src[after] == '_');
    if (left_ok && right_ok) break;
    at = src.find(func, at + 1);
  }
  if (at == std::string::npos) return false;
  const size_t lp = src.find('(', at), rp = src.find(')', lp), lb = src.find('{', rp);
  if (lp == std::string::npos || rp == std::string::npos || lb == std::string::npos) return false;
  int depth = 0;
  size_t rb = lb;
  for (; rb < src.size(); ++rb) {
    if (src[rb] == '{') ++depth;
    if (src[rb] == '}' && --depth == 0) break;
  }
  if (rb >= src.size()) return false;
  // parameter names: last identifier of each comma-separated declaration
  std::vector<std::string> names;
  std::string params = src.substr(lp + 1, rp - lp - 1), cur;
  params += ',';
  for (char c : params) {
    if (c == ',') {
      size_t e = cur.find_last_not_of(" \t\r\n");
      size_t b = e == std::string::npos ? e : cur.find_last_of(" \t\r\n*&", e);
      names.push_back(e == std::string::npos ? "" : cur.substr(b == std::string::npos ? 0 : b + 1, e - (b == std::string::npos ? 0 : b + 1) + 1));
      cur.clear();
    } else {
      cur += c;
    }
  }
  if (names.size() != 2) return false;
  std::string body;
  for (size_t i = lb; i <= rb; ++i)
    if (!std::isspace((unsigned char)src[i])) body += src[i];
  const std::string a = names[0], b = names[1], o(1, op);
  return body == "{return" + a + o + b + ";}" || body == "{return" + b + o + a + ";}" ||
         body == "{return(" + a + o + b + ");}" || body == "{return(" + b + o + a + ");}";
}

template <typename T> Vector<T> sameShape(const Vector<T>& v) { return Vector<T>(v.size()); }
template <typename T> Matrix<T> sameShape(const Matrix<T>& m) { return Matrix<T>(m.size()); }
template <typename U, typename T> Vector<U> shapedLike(const Vector<T>& v) { return Vector<U>(v.size()); }
template <typename U, typename T> Matrix<U> shapedLike(const Matrix<T>& m) { return Matrix<U>(m.size()); }

template <typename T> size_t count(const Vector<T>& v) { return v.size(); }
template <typename T> size_t count(const Matrix<T>& m) { return m.size().elemCount(); }

template <typename C>
struct Node {
  C* value = nullptr;
  std::unique_ptr<C> owned;
  std::unique_ptr<C> grad;
  bool requiresGrad = true;
};

inline void check(int status, const char* what) { skelcl::detail::checkStatus(status, what); }

}  // namespace detail

class Tape;

// A container on a tape: its value and, after Tape::backward, its gradient.
template <typename C>
class Var {
public:
  Var() = default;
  const C& value() const { return *_n->value; }
  bool requiresGrad() const { return _n && _n->requiresGrad; }
  bool hasGrad() const { return _n && _n->grad != nullptr; }
  // The gradient; a variable that backward() did not reach has none.
  C& grad() const {
    if (!hasGrad()) ABORT_WITH_ERROR("ad::Var::grad(): no gradient reached this value");
    return *_n->grad;
  }
  const std::shared_ptr<detail::Node<C>>& node() const { return _n; }

private:
  friend class Tape;
  explicit Var(std::shared_ptr<detail::Node<C>> n) : _n(std::move(n)) {}
  std::shared_ptr<detail::Node<C>> _n;
};

class Tape {
public:
  // An input whose gradient is wanted; `c` must outlive backward().
  template <typename C>
  Var<C> variable(C& c) {
    auto n = std::make_shared<detail::Node<C>>();
    n->value = &c;
    return Var<C>(n);
  }
  // An input treated as a constant (no gradient).
  template <typename C>
  Var<C> constant(const C& c) {
    auto n = std::make_shared<detail::Node<C>>();
    n->value = const_cast<C*>(&c);
    n->requiresGrad = false;
    return Var<C>(n);
  }
  // A value computed by a recorded skeleton call (owned by the tape).
  template <typename C>
  Var<C> result(C&& c, bool requiresGrad) {
    auto n = std::make_shared<detail::Node<C>>();
    n->owned.reset(new C(std::move(c)));
    n->value = n->owned.get();
    n->requiresGrad = requiresGrad;
    _results.push_back([n]() { n->grad.reset(); });
    return Var<C>(n);
  }
  void record(std::function<void()> adjoint) { _steps.push_back(std::move(adjoint)); }

  // Runs the recorded adjoints in reverse with d out = seed.  Gradients of
  // intermediate values start from zero on every call; those of variables
  // add up across calls.
  template <typename C>
  void backward(const Var<C>& out, const C& seed) {
    for (auto& reset : _results) reset();
    auto& n = *out.node();
    if (detail::count(seed) != detail::count(*n.value))
      ABORT_WITH_ERROR("ad::Tape::backward: the seed's size differs from the output's");
    n.grad.reset(new C(detail::sameShape(*n.value)));
    detail::check(scl_d2d(n.grad->deviceOutputPtr(), seed.devicePtr(),
                          detail::count(seed) * sizeof(typename C::value_type)),
                  "ad seed");
    n.grad->dataOnDeviceModified();
    for (auto it = _steps.rbegin(); it != _steps.rend(); ++it) (*it)();
  }
  // Scalar output (a one-element Vector, e.g. from Reduce): seed 1.
  template <typename T>
  void backward(const Var<Vector<T>>& out) {
    if (out.value().size() != 1) ABORT_WITH_ERROR("ad::Tape::backward: give a seed for non-scalar outputs");
    Vector<T> one(1, T(1));
    backward(out, one);
  }
  void clear() {
    _steps.clear();
    _results.clear();
  }
  size_t size() const { return _steps.size(); }

  // Where the adjoint of a node is written: a new gradient is overwritten,
  // an existing one is added to (*accumulate set).
  template <typename C>
  static void* gradTarget(detail::Node<C>& n, bool* accumulate) {
    if (!n.grad) {
      n.grad.reset(new C(detail::sameShape(*n.value)));
      *accumulate = false;
      return n.grad->deviceOutputPtr();
    }
    *accumulate = true;
    return n.grad->devicePtr();
  }
  // For adjoints that cannot add into their output: `write(ptr)` fills a
  // fresh buffer, which is then added to an existing gradient.
  template <typename C, typename F>
  static void writeGrad(detail::Node<C>& n, F write) {
    typedef typename C::value_type T;
    if (!n.grad) {
      bool acc = false;
      void* p = gradTarget(n, &acc);
      write(p);
      n.grad->dataOnDeviceModified();
      return;
    }
    C tmp = detail::sameShape(*n.value);
    write(tmp.deviceOutputPtr());
    detail::check(scl_adjoint_accumulate(n.grad->devicePtr(), tmp.devicePtr(), detail::count(tmp),
                                         detail::DType<T>::value),
                  "ad gradient accumulation");
    n.grad->dataOnDeviceModified();
  }  // `tmp` is freed in stream order, after the accumulation

private:
  std::vector<std::function<void()>> _steps;
  std::vector<std::function<void()>> _results;  // clear an intermediate's gradient
};

// ---- Map -------------------------------------------------------------------------
template <typename> class Map;

template <typename Tin, typename Tout>
class Map<Tout(Tin)> {
public:
  // `vjp` defines `Tin vjpFunc(Tin x, Tout g, extra...)` = g * d func / d x.
  Map(const Source& source, const Source& vjp, const std::string& func = "func",
      const std::string& vjpFunc = "dfunc") {
    skelcl::detail::ProgramSpec f;
    f.kind = SCL_KIND_MAP;
    f.source = source;
    f.func = func;
    f.types = {skelcl::detail::typeName<Tin>(), skelcl::detail::typeName<Tout>()};
    _fwd = f.build();
    skelcl::detail::ProgramSpec a = f;
    a.kind = SCL_KIND_MAP_ADJOINT;
    a.source = vjp;
    a.func = vjpFunc;
    _adj = a.build();
  }

  template <template <typename> class C, typename... Args>
  Var<C<Tout>> operator()(Tape& tape, const Var<C<Tin>>& x, Args&&... args) const {
    const C<Tin>& in = x.value();
    C<Tout> o = detail::shapedLike<Tout>(in);
    skelcl::detail::prepareArgs(args...);
    skelcl::detail::ArgBlob blob = skelcl::detail::packArgs(args...);
    void* bufs[2] = {in.devicePtr(), o.deviceOutputPtr()};
    scl_shape sh = skelcl::detail::makeShape(detail::count(in));
    detail::check(scl_launch_map(_fwd.get(), &sh, bufs, blob.data(), blob.size(), nullptr), "ad::Map");
    o.dataOnDeviceModified();
    Var<C<Tout>> y = tape.result(std::move(o), x.requiresGrad());
    if (x.requiresGrad()) {
      auto xn = x.node();
      auto yn = y.node();
      auto adj = _adj;
      tape.record([xn, yn, adj, blob]() {
        if (!yn->grad) return;
        bool acc = false;
        void* gx = Tape::gradTarget(*xn, &acc);
        void* b[3] = {xn->value->devicePtr(), yn->grad->devicePtr(), gx};
        scl_shape s = skelcl::detail::makeShape(detail::count(*xn->value));
        s.flags = acc ? SCL_SHAPE_ACCUMULATE : 0u;
        detail::check(scl_launch_map(adj.get(), &s, b, blob.data(), blob.size(), nullptr), "ad::Map adjoint");
        xn->grad->dataOnDeviceModified();
      });
    }
    return y;
  }

private:
  skelcl::detail::Program _fwd, _adj;
};

// ---- Zip -------------------------------------------------------------------------
template <typename> class Zip;

template <typename Tl, typename Tr, typename Tout>
class Zip<Tout(Tl, Tr)> {
public:
  // `vjp` defines `Tl dl(Tl x, Tr y, Tout g, extra...)` and (optionally)
  // `Tr dr(Tl x, Tr y, Tout g, extra...)`, the gradients for each operand.
  Zip(const Source& source, const Source& vjp, const std::string& func = "func",
      const std::string& dlFunc = "dl", const std::string& drFunc = "dr")
      : _hasRight(!drFunc.empty()) {
    skelcl::detail::ProgramSpec f;
    f.kind = SCL_KIND_ZIP;
    f.source = source;
    f.func = func;
    f.types = {skelcl::detail::typeName<Tl>(), skelcl::detail::typeName<Tr>(),
               skelcl::detail::typeName<Tout>()};
    _fwd = f.build();
    skelcl::detail::ProgramSpec a = f;
    a.kind = SCL_KIND_ZIP_ADJOINT;
    a.source = vjp;
    a.func = dlFunc;
    a.func2 = drFunc;
    _adj = a.build();
  }

  template <template <typename> class C, typename... Args>
  Var<C<Tout>> operator()(Tape& tape, const Var<C<Tl>>& x, const Var<C<Tr>>& y, Args&&... args) const {
    const C<Tl>& l = x.value();
    const C<Tr>& r = y.value();
    ASSERT_MESSAGE(detail::count(l) <= detail::count(r), "ad::Zip: the right operand is shorter");
    C<Tout> o = detail::shapedLike<Tout>(l);
    skelcl::detail::prepareArgs(args...);
    skelcl::detail::ArgBlob blob = skelcl::detail::packArgs(args...);
    void* bufs[3] = {l.devicePtr(), r.devicePtr(), o.deviceOutputPtr()};
    scl_shape sh = skelcl::detail::makeShape(detail::count(l));
    detail::check(scl_launch_zip(_fwd.get(), &sh, bufs, blob.data(), blob.size(), nullptr), "ad::Zip");
    o.dataOnDeviceModified();
    const bool need = x.requiresGrad() || y.requiresGrad();
    Var<C<Tout>> z = tape.result(std::move(o), need);
    if (y.requiresGrad() && !_hasRight)
      ABORT_WITH_ERROR("ad::Zip: the right operand needs a gradient but no right derivative was given");
    if (need) {
      auto xn = x.node();
      auto yn = y.node();
      auto zn = z.node();
      auto adj = _adj;
      tape.record([xn, yn, zn, adj, blob]() {
        if (!zn->grad) return;
        bool ax = false, ay = false;
        void* gx = xn->requiresGrad ? Tape::gradTarget(*xn, &ax) : nullptr;
        void* gy = yn->requiresGrad ? Tape::gradTarget(*yn, &ay) : nullptr;
        void* b[5] = {xn->value->devicePtr(), yn->value->devicePtr(), zn->grad->devicePtr(), gx, gy};
        scl_shape s = skelcl::detail::makeShape(detail::count(*zn->value));
        s.flags = (ax ? SCL_SHAPE_ACCUMULATE : 0u) | (ay ? SCL_SHAPE_ACCUMULATE_RIGHT : 0u);
        detail::check(scl_launch_map(adj.get(), &s, b, blob.data(), blob.size(), nullptr), "ad::Zip adjoint");
        if (gx) xn->grad->dataOnDeviceModified();
        if (gy) yn->grad->dataOnDeviceModified();
      });
    }
    return z;
  }

private:
  bool _hasRight;
  skelcl::detail::Program _fwd, _adj;
};

// ---- Reduce (+) ------------------------------------------------------------------
template <typename T>
class Reduce {
public:
  // `source` must be the addition `T func(T x, T y){ return x + y; }`.
  explicit Reduce(const Source& source, const std::string& id = "0", const std::string& func = "func") {
    if (!detail::isBinaryOp(source, func, '+'))
      ABORT_WITH_ERROR("ad::Reduce differentiates sums only: the function must be `return x + y;`");
    skelcl::detail::ProgramSpec f;
    f.kind = SCL_KIND_REDUCE;
    f.source = source;
    f.func = func;
    f.identity = id;
    f.types = {skelcl::detail::typeName<T>()};
    _fwd = f.build();
  }

  Var<Vector<T>> operator()(Tape& tape, const Var<Vector<T>>& x) const {
    const Vector<T>& in = x.value();
    Vector<T> o(1);
    void* bufs[2] = {in.devicePtr(), o.deviceOutputPtr()};
    scl_shape sh = skelcl::detail::makeShape(in.size());
    detail::check(scl_launch_reduce(_fwd.get(), &sh, bufs, nullptr, 0, nullptr), "ad::Reduce");
    o.dataOnDeviceModified();
    Var<Vector<T>> y = tape.result(std::move(o), x.requiresGrad());
    if (x.requiresGrad()) {
      auto xn = x.node();
      auto yn = y.node();
      tape.record([xn, yn]() {
        if (!yn->grad) return;
        bool acc = false;
        void* gx = Tape::gradTarget(*xn, &acc);
        detail::check(scl_adjoint_broadcast(yn->grad->devicePtr(), gx, xn->value->size(),
                                            detail::DType<T>::value, acc ? 1 : 0),
                      "ad::Reduce adjoint");
        xn->grad->dataOnDeviceModified();
      });
    }
    return y;
  }

  // One sum per vector of `segments` (stored back to back in x), one launch;
  // the adjoint broadcasts each vector's gradient over its elements, also in
  // one launch.  Elements outside every vector get a zero gradient.
  Var<Vector<T>> segmented(Tape& tape, const Var<Vector<T>>& x, const Segments& segments) const {
    const Vector<T>& in = x.value();
    ASSERT_MESSAGE(segments.total() <= in.size(), "ad::Reduce::segmented: segments beyond the input");
    const size_t ns = segments.count();
    Vector<T> o(ns);
    if (ns > 0) {
      void* bufs[2] = {nullptr, o.deviceOutputPtr()};
      bufs[0] = in.size() ? (void*)in.devicePtr() : bufs[1];
      scl_shape sh = skelcl::detail::makeShape(in.size());
      sh.seg_offsets = segments.devicePtr();
      sh.n_segments = ns;
      sh.seg_plan = segments.plan();
      detail::check(scl_launch_reduce(_fwd.get(), &sh, bufs, nullptr, 0, nullptr), "ad::Reduce::segmented");
      o.dataOnDeviceModified();
    }
    Var<Vector<T>> y = tape.result(std::move(o), x.requiresGrad());
    if (x.requiresGrad() && ns > 0 && in.size() > 0) {
      auto xn = x.node();
      auto yn = y.node();
      const Segments segs = segments;
      tape.record([xn, yn, segs]() {
        if (!yn->grad) return;
        const size_t n = xn->value->size();
        bool acc = false;
        void* gx = Tape::gradTarget(*xn, &acc);
        if (!acc && segs.total() < n)
          detail::check(scl_memset(gx, 0, n * sizeof(T)), "ad::Reduce::segmented adjoint");
        detail::check(scl_adjoint_broadcast_segments(yn->grad->devicePtr(), gx, segs.devicePtr(), segs.count(),
                                                     n, detail::DType<T>::value, acc ? 1 : 0),
                      "ad::Reduce::segmented adjoint");
        xn->grad->dataOnDeviceModified();
      });
    }
    return y;
  }

private:
  skelcl::detail::Program _fwd;
};

// ---- Scan (+) --------------------------------------------------------------------
template <typename T>
class Scan {
public:
  // `source` must be the addition; exclusive like skelcl::Scan unless
  // setInclusive(true).
  explicit Scan(const Source& source, const std::string& id = "0", const std::string& func = "func") {
    if (!detail::isBinaryOp(source, func, '+'))
      ABORT_WITH_ERROR("ad::Scan differentiates prefix sums only: the function must be `return x + y;`");
    skelcl::detail::ProgramSpec f;
    f.kind = SCL_KIND_SCAN;
    f.source = source;
    f.func = func;
    f.identity = id;
    f.types = {skelcl::detail::typeName<T>()};
    _fwd = f.build();
  }
  Scan& setInclusive(bool inclusive) {
    _inclusive = inclusive;
    return *this;
  }

  Var<Vector<T>> operator()(Tape& tape, const Var<Vector<T>>& x) const {
    const Vector<T>& in = x.value();
    Vector<T> o(in.size());
    void* bufs[2] = {in.devicePtr(), o.deviceOutputPtr()};
    scl_shape sh = skelcl::detail::makeShape(in.size());
    sh.flags = _inclusive ? SCL_SHAPE_INCLUSIVE : 0u;
    detail::check(scl_launch_scan(_fwd.get(), &sh, bufs, nullptr, 0, nullptr), "ad::Scan");
    o.dataOnDeviceModified();
    Var<Vector<T>> y = tape.result(std::move(o), x.requiresGrad());
    if (x.requiresGrad()) {
      auto xn = x.node();
      auto yn = y.node();
      auto prog = _fwd;
      const uint32_t flags = SCL_SHAPE_REVERSE | (_inclusive ? SCL_SHAPE_INCLUSIVE : 0u);
      tape.record([xn, yn, prog, flags]() {
        if (!yn->grad) return;
        Tape::writeGrad(*xn, [&](void* gx) {
          void* b[2] = {yn->grad->devicePtr(), gx};
          scl_shape s = skelcl::detail::makeShape(xn->value->size());
          s.flags = flags;
          detail::check(scl_launch_scan(prog.get(), &s, b, nullptr, 0, nullptr), "ad::Scan adjoint");
        });
      });
    }
    return y;
  }

  // One scan per vector of `segments` (stored back to back in x), one launch;
  // the adjoint is the segmented reverse scan, also one launch.  Elements
  // outside every vector are 0 in the result and get a zero gradient.
  Var<Vector<T>> segmented(Tape& tape, const Var<Vector<T>>& x, const Segments& segments) const {
    const Vector<T>& in = x.value();
    ASSERT_MESSAGE(segments.total() <= in.size(), "ad::Scan::segmented: segments beyond the input");
    const size_t n = in.size();
    Vector<T> o(n);
    if (n > 0) {
      void* bufs[2] = {in.devicePtr(), o.deviceOutputPtr()};
      if (segments.total() < n || segments.count() == 0)
        detail::check(scl_memset(bufs[1], 0, n * sizeof(T)), "ad::Scan::segmented");
      if (segments.count() > 0) {
        scl_shape sh = skelcl::detail::makeShape(n);
        sh.flags = _inclusive ? SCL_SHAPE_INCLUSIVE : 0u;
        sh.seg_offsets = segments.devicePtr();
        sh.n_segments = segments.count();
        sh.seg_plan = segments.plan();
        detail::check(scl_launch_scan(_fwd.get(), &sh, bufs, nullptr, 0, nullptr), "ad::Scan::segmented");
      }
      o.dataOnDeviceModified();
    }
    Var<Vector<T>> y = tape.result(std::move(o), x.requiresGrad());
    if (x.requiresGrad() && n > 0) {
      auto xn = x.node();
      auto yn = y.node();
      auto prog = _fwd;
      const Segments segs = segments;
      const uint32_t flags = SCL_SHAPE_REVERSE | (_inclusive ? SCL_SHAPE_INCLUSIVE : 0u);
      tape.record([xn, yn, prog, segs, flags, n]() {
        if (!yn->grad) return;
        Tape::writeGrad(*xn, [&](void* gx) {
          if (segs.total() < n || segs.count() == 0)
            detail::check(scl_memset(gx, 0, n * sizeof(T)), "ad::Scan::segmented adjoint");
          if (segs.count() == 0) return;
          void* b[2] = {yn->grad->devicePtr(), gx};
          scl_shape s = skelcl::detail::makeShape(n);
          s.flags = flags;
          s.seg_offsets = segs.devicePtr();
          s.n_segments = segs.count();
          s.seg_plan = segs.plan();
          detail::check(scl_launch_scan(prog.get(), &s, b, nullptr, 0, nullptr), "ad::Scan::segmented adjoint");
        });
      });
    }
    return y;
  }

private:
  bool _inclusive = false;
  skelcl::detail::Program _fwd;
};

// ---- MapOverlap (linear, float) -------------------------------------------------------
template <typename> class MapOverlap;

template <>
class MapOverlap<float(float)> {
public:
  // A stencil that is linear in the matrix, with the same coefficients at
  // every pixel (e.g. a convolution whose weights come as an extra argument).
  MapOverlap(const Source& source, unsigned overlap_range = 1,
             skelcl::detail::Padding padding = skelcl::detail::Padding::NEAREST, float neutral = 0.0f,
             const std::string& func = "func")
      : _range((int)overlap_range), _nearest(padding == skelcl::detail::Padding::NEAREST) {
    skelcl::detail::ProgramSpec f;
    f.kind = SCL_KIND_MAPOVERLAP;
    f.source = source;
    f.func = func;
    f.overlapRange = _range;
    f.padding = _nearest ? SCL_PAD_NEAREST : SCL_PAD_NEUTRAL;
    f.neutral = skelcl::detail::sourceLiteral(neutral);
    f.types = {"float", "float"};
    _fwd = f.build();
    // the transposed stencil: a zero-padded MapOverlap over the weights
    const std::string R = std::to_string(_range), W = std::to_string(2 * _range + 1);
    skelcl::detail::ProgramSpec a = f;
    a.source = "float scl_stencil_adjoint(input_matrix_t g, __global const float* w) {\n"
               "  float s = 0.0f;\n"
               "  for (int dy = -" + R + "; dy <= " + R + "; ++dy)\n"
               "    for (int dx = -" + R + "; dx <= " + R + "; ++dx)\n"
               "      s += w[(dy + " + R + ") * " + W + " + (dx + " + R + ")] * getData(g, dx, dy);\n"
               "  return s;\n}\n";
    a.func = "scl_stencil_adjoint";
    a.padding = SCL_PAD_NEUTRAL;
    a.neutral = "0.0f";
    _adj = a.build();
  }

  template <typename... Args>
  Var<Matrix<float>> operator()(Tape& tape, const Var<Matrix<float>>& x, Args&&... args) const {
    const Matrix<float>& in = x.value();
    Matrix<float> o(in.size());
    skelcl::detail::prepareArgs(args...);
    skelcl::detail::ArgBlob blob = skelcl::detail::packArgs(args...);
    run(_fwd, in.devicePtr(), o.deviceOutputPtr(), in.rowCount(), in.columnCount(), blob);
    o.dataOnDeviceModified();
    Var<Matrix<float>> y = tape.result(std::move(o), x.requiresGrad());
    if (x.requiresGrad()) {
      auto xn = x.node();
      auto yn = y.node();
      auto fwd = _fwd, adj = _adj;
      const int R = _range;
      const bool nearest = _nearest;
      tape.record([xn, yn, fwd, adj, R, nearest, blob]() {
        if (!yn->grad) return;
        Vector<float> w = weights(fwd, R, blob);
        const uint64_t rows = xn->value->rowCount(), cols = xn->value->columnCount();
        Tape::writeGrad(*xn, [&](void* gx) {
          skelcl::detail::ArgBlob wb = skelcl::detail::packArgs(w);
          run(adj, yn->grad->devicePtr(), gx, rows, cols, wb);
          if (nearest)
            detail::check(scl_mapoverlap_adjoint_edges(yn->grad->devicePtr(), w.devicePtr(),
                                                       static_cast<float*>(gx), rows, cols, R),
                          "ad::MapOverlap adjoint (edges)");
        });
      });
    }
    return y;
  }

  // The transposed-stencil weights: the forward's response to a unit impulse
  // minus its response to zero, on a (2R+1)^2 matrix; entry (dy+R, dx+R)
  // multiplies g[y+dy][x+dx] in the adjoint.
  static Vector<float> weights(const skelcl::detail::Program& fwd, int R,
                               const skelcl::detail::ArgBlob& blob) {
    const size_t W = (size_t)(2 * R + 1);
    Matrix<float> impulse(MatrixSize(W, W), 0.0f), zero(MatrixSize(W, W), 0.0f);
    impulse[R][R] = 1.0f;
    Matrix<float> ri(MatrixSize(W, W)), rz(MatrixSize(W, W));
    run(fwd, impulse.devicePtr(), ri.deviceOutputPtr(), W, W, blob);
    run(fwd, zero.devicePtr(), rz.deviceOutputPtr(), W, W, blob);
    ri.dataOnDeviceModified();
    rz.dataOnDeviceModified();
    Vector<float> w(W * W);
    for (size_t i = 0; i < W; ++i)
      for (size_t j = 0; j < W; ++j) w[i * W + j] = ri[i][j] - rz[i][j];
    w.dataOnHostModified();
    return w;
  }

private:
  static void run(const skelcl::detail::Program& p, void* in, void* out, uint64_t rows, uint64_t cols,
                  const skelcl::detail::ArgBlob& blob) {
    void* bufs[2] = {in, out};
    scl_shape sh = skelcl::detail::makeShape(0);
    sh.rows = rows;
    sh.cols = cols;
    detail::check(scl_launch_mapoverlap(p.get(), &sh, bufs, blob.data(), blob.size(), nullptr),
                  "ad::MapOverlap");
  }

  int _range;
  bool _nearest;
  skelcl::detail::Program _fwd, _adj;
};

// ---- AllPairs (x*y, +) ---------------------------------------------------------------
template <typename> class AllPairs;

template <>
class AllPairs<float(float, float)> {
public:
  // The Reduce must be `x + y` with identity 0 and the Zip `x * y`: P = A B.
  AllPairs(const skelcl::Reduce<float(float)>& reduce, const skelcl::Zip<float(float, float)>& zip) {
    if (!detail::isBinaryOp(reduce.source(), reduce.func(), '+') ||
        !detail::isBinaryOp(zip.source(), zip.func(), '*'))
      ABORT_WITH_ERROR("ad::AllPairs differentiates the x*y / x+y contraction only");
    skelcl::detail::ProgramSpec s;
    s.kind = SCL_KIND_ALLPAIRS;
    s.source = reduce.source();
    s.func = reduce.func();
    s.source2 = zip.source();
    s.func2 = zip.func();
    s.identity = reduce.id();
    s.types = {"float", "float", "float"};
    _prog = s.build();
  }
  // Keep the contraction on the CUDA cores (forward and adjoint).
  AllPairs& setPrecise(bool precise) {
    _precise = precise;
    return *this;
  }

  Var<Matrix<float>> operator()(Tape& tape, const Var<Matrix<float>>& a, const Var<Matrix<float>>& b) const {
    const Matrix<float>& A = a.value();
    const Matrix<float>& B = b.value();
    ASSERT_MESSAGE(A.columnCount() == B.rowCount(), "ad::AllPairs: inner dimensions differ");
    const uint64_t M = A.rowCount(), K = A.columnCount(), N = B.columnCount();
    Matrix<float> P(MatrixSize(M, N));
    run(_prog, _precise, A.devicePtr(), B.devicePtr(), P.deviceOutputPtr(), M, N, K, 0);
    P.dataOnDeviceModified();
    const bool need = a.requiresGrad() || b.requiresGrad();
    Var<Matrix<float>> p = tape.result(std::move(P), need);
    if (need) {
      auto an = a.node();
      auto bn = b.node();
      auto pn = p.node();
      auto prog = _prog;
      const bool precise = _precise;
      tape.record([an, bn, pn, prog, precise, M, N, K]() {
        if (!pn->grad) return;
        void* G = pn->grad->devicePtr();
        if (an->requiresGrad)  // dA = G B^T: M x K over N, B read transposed
          Tape::writeGrad(*an, [&](void* dA) {
            run(prog, precise, G, bn->value->devicePtr(), dA, M, K, N, SCL_SHAPE_TRANS_RIGHT);
          });
        if (bn->requiresGrad)  // dB = A^T G: K x N over M, A read transposed
          Tape::writeGrad(*bn, [&](void* dB) {
            run(prog, precise, an->value->devicePtr(), G, dB, K, N, M, SCL_SHAPE_TRANS_LEFT);
          });
      });
    }
    return p;
  }

private:
  static void run(const skelcl::detail::Program& prog, bool precise, void* left, void* right, void* out,
                  uint64_t rows, uint64_t cols, uint64_t dim, uint32_t flags) {
    void* bufs[3] = {left, right, out};
    scl_shape sh = skelcl::detail::makeShape(0);
    sh.rows = rows;
    sh.cols = cols;
    sh.dim = dim;
    sh.flags = flags;
    scl_tuning t;
    std::memset(&t, 0, sizeof(t));
    if (precise) t.variant = SCL_VARIANT_SIMT;
    detail::check(scl_launch_allpairs(prog.get(), &sh, bufs, nullptr, 0, &t), "ad::AllPairs");
  }

  bool _precise = false;
  skelcl::detail::Program _prog;
};

}  // namespace ad
}  // namespace skelcl

#endif  // SKELCL_ADJOINT_H_
