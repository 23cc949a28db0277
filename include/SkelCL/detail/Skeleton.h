// Skeleton base class, extra-argument marshalling and the program handle.
//
// Replaces the reference's detail::Skeleton (include/SkelCL/detail/Skeleton.h
// :52-142, src/Skeleton.cpp:48-86), detail::kernelUtil::setKernelArgs /
// keepAlive (include/SkelCL/detail/KernelUtil.h:77-360) and detail::Program
// (include/SkelCL/detail/Program.h:61-132).  Extra arguments are packed into
// the C ABI's argument blob in call order with the reference's kinds:
// Vector -> device pointer, Matrix -> device pointer + column count,
// Local -> __local bytes, Out<C> -> its container (marked device-modified
// after the call), anything else -> its bytes by value.
#ifndef SKELCL_SKELETON_H_
#define SKELCL_SKELETON_H_

#include <cstdint>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include "../Local.h"
#include "../Matrix.h"
#include "../Out.h"
#include "../Source.h"
#include "../Vector.h"
#include "Runtime.h"
#include "Util.h"

namespace skelcl {
namespace detail {

// ---- argument blob ------------------------------------------------------------
class ArgBlob {
public:
  void add(uint32_t kind, const void* payload, uint32_t size) {
    const size_t at = _bytes.size();
    const size_t padded = (size + 7u) & ~7u;
    _bytes.resize(at + 8 + padded, 0);
    std::memcpy(&_bytes[at], &kind, 4);
    std::memcpy(&_bytes[at + 4], &size, 4);
    if (size) std::memcpy(&_bytes[at + 8], payload, size);
  }
  const void* data() const { return _bytes.empty() ? nullptr : _bytes.data(); }
  size_t size() const { return _bytes.size(); }

private:
  std::vector<unsigned char> _bytes;
};

template <typename A>
struct ArgTraits {  // scalars and structs: by value
  static void prepare(const A&) {}
  static void pack(ArgBlob& b, const A& a) {
    static_assert(std::is_trivially_copyable<A>::value,
                  "extra skeleton arguments must be containers, Local, Out<> or trivially copyable values");
    b.add(SCL_ARG_VALUE, &a, sizeof(A));
  }
  static void modified(const A&) {}
};

template <typename T>
struct ArgTraits<Vector<T>> {
  static void prepare(const Vector<T>& v) { v.copyDataToDevices(); }
  static void pack(ArgBlob& b, const Vector<T>& v) {
    void* p = v.devicePtr();
    b.add(SCL_ARG_BUFFER, &p, sizeof(p));
  }
  static void modified(const Vector<T>&) {}
};

template <typename T>
struct ArgTraits<Matrix<T>> {
  static void prepare(const Matrix<T>& m) { m.copyDataToDevices(); }
  static void pack(ArgBlob& b, const Matrix<T>& m) {
    unsigned char rec[12];
    void* p = m.devicePtr();
    uint32_t cols = (uint32_t)m.columnCount();
    std::memcpy(rec, &p, 8);
    std::memcpy(rec + 8, &cols, 4);
    b.add(SCL_ARG_MATRIX, rec, 12);
  }
  static void modified(const Matrix<T>&) {}
};

template <typename C>
struct ArgTraits<Out<C>> {
  static void prepare(const Out<C>& o) { ArgTraits<C>::prepare(o.container()); }
  static void pack(ArgBlob& b, const Out<C>& o) { ArgTraits<C>::pack(b, o.container()); }
  static void modified(const Out<C>& o) { o.container().dataOnDeviceModified(); }
};

template <>
struct ArgTraits<Local> {
  static void prepare(const Local&) {}
  static void pack(ArgBlob& b, const Local& l) {
    uint64_t n = l.getSizeInBytes();
    b.add(SCL_ARG_LOCAL, &n, 8);
  }
  static void modified(const Local&) {}
};

template <typename... Args>
void prepareArgs(const Args&... args) {
  int dummy[] = {0, (ArgTraits<typename std::decay<Args>::type>::prepare(args), 0)...};
  (void)dummy;
}
template <typename... Args>
ArgBlob packArgs(const Args&... args) {
  ArgBlob b;
  int dummy[] = {0, (ArgTraits<typename std::decay<Args>::type>::pack(b, args), 0)...};
  (void)dummy;
  return b;
}
template <typename... Args>
void markModified(const Args&... args) {
  int dummy[] = {0, (ArgTraits<typename std::decay<Args>::type>::modified(args), 0)...};
  (void)dummy;
}

// ---- literals for the generated source -------------------------------------------
template <typename T>
std::string sourceLiteral(const T& v) {
  if constexpr (std::is_floating_point<T>::value) {
    std::ostringstream s;
    s << std::hexfloat << v;
    return s.str() + (std::is_same<T, float>::value ? "f" : "");
  } else if constexpr (std::is_integral<T>::value) {
    std::ostringstream s;
    if (std::is_signed<T>::value) s << (long long)v << "ll";
    else s << (unsigned long long)v << "ull";
    return s.str();
  } else {
    // Non-arithmetic neutral elements: all bytes zero (value-initialised).
    return "SCL_TYPE_0()";
  }
}

// ---- program handle ------------------------------------------------------------------
class Program {
public:
  Program() = default;
  explicit Program(const scl_program_desc& desc) {
    ensureInitialized();
    scl_program* p = nullptr;
    std::vector<char> log(1 << 16, '\0');
    int st = scl_program_build(&desc, &p, log.data(), log.size());
    if (st != SCL_OK) {
      std::string msg = std::string("building skeleton program failed (status ") +
                        std::to_string(st) + "): " + scl_last_error_string();
      ABORT_WITH_ERROR(msg);
    }
    _handle = std::shared_ptr<scl_program>(p, [](scl_program* q) {
      if (scl_is_initialized()) scl_program_release(q);
    });
    _gen = runtimeGeneration();
  }
  scl_program* get() const {
    if (_handle && _gen != runtimeGeneration())
      ABORT_WITH_ERROR("skeleton used after skelcl::terminate(); construct it again");
    return _handle.get();
  }
  std::string hash() const {
    char h[41] = {0};
    if (_handle) scl_program_hash(_handle.get(), h);
    return h;
  }

private:
  std::shared_ptr<scl_program> _handle;
  unsigned long _gen = 0;
};

// Description of a program: owns the strings the C ABI points to.
struct ProgramSpec {
  int kind = 0;
  std::string source, func = "func", source2, func2 = "func", identity = "0", neutral;
  std::vector<std::string> types;
  int overlapRange = 0;
  int padding = SCL_PAD_NEAREST;
  uint32_t flags = 0;

  Program build() const {
    std::string common = CommonDefinitions::getString();
    scl_program_desc d;
    std::memset(&d, 0, sizeof(d));
    d.kind = kind;
    d.source = source.c_str();
    d.func = func.c_str();
    d.source2 = source2.empty() ? nullptr : source2.c_str();
    d.func2 = func2.c_str();
    d.identity = identity.c_str();
    d.n_types = (int)types.size();
    for (size_t i = 0; i < types.size() && i < 3; ++i) d.type_names[i] = types[i].c_str();
    d.overlap_range = overlapRange;
    d.padding = padding;
    d.neutral = neutral.empty() ? nullptr : neutral.c_str();
    d.common_source = common.empty() ? nullptr : common.c_str();
    d.flags = flags;
    return Program(d);
  }
};

// ---- skeleton base ---------------------------------------------------------------------
class Skeleton {
public:
  Skeleton() : _workGroupSize(256), _wgSet(false) {}
  explicit Skeleton(unsigned workGroupSize) : _workGroupSize(workGroupSize), _wgSet(true) {}
  Skeleton(const Skeleton&) = default;
  Skeleton& operator=(const Skeleton&) = default;
  virtual ~Skeleton() = default;

  size_t workGroupSize() const { return _workGroupSize; }
  void setWorkGroupSize(size_t size) {
    _workGroupSize = size;
    _wgSet = true;
  }
  // Launch tuning: the work-group size (threads per block) when one was set;
  // everything else is left to the library's defaults / autotuner.
  scl_tuning tuning() const {
    scl_tuning t;
    std::memset(&t, 0, sizeof(t));
    if (_wgSet) t.workgroup = (uint32_t)_workGroupSize;
    return t;
  }

protected:
  static void launched(int status, const char* what) { checkStatus(status, what); }

private:
  size_t _workGroupSize;
  bool _wgSet;
};

template <typename T>
size_t elementCount(const Vector<T>& v) {
  return v.size();
}
template <typename T>
size_t elementCount(const Matrix<T>& m) {
  return m.size().elemCount();
}
template <typename T>
void resizeLike(Vector<T>& out, size_t n) {
  if (out.size() < n) out.resize(n);
}
template <typename T, typename U>
void resizeLike(Matrix<T>& out, const Matrix<U>& in) {
  if (out.size() != in.size()) out.resize(in.size());
}
template <typename T, typename U>
void resizeLike(Vector<T>& out, const Vector<U>& in) {
  if (out.size() < in.size()) out.resize(in.size());
}

inline scl_shape makeShape(uint64_t n) {
  scl_shape s;
  std::memset(&s, 0, sizeof(s));
  s.n = n;
  return s;
}

}  // namespace detail
}  // namespace skelcl

#endif  // SKELCL_SKELETON_H_
