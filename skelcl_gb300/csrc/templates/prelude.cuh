// ---------------------------------------------------------------------------
// OpenCL C -> CUDA prelude.  Prepended to every NVRTC program so that SkelCL
// user functions written in OpenCL C compile unchanged for sm_103a.
//
// What it provides (the device-side vocabulary user strings rely on):
//  * address-space qualifiers __global/__local/__constant/__private as no-ops
//  * work-item functions get_global_id & co.  They are exact in the
//    one-element-per-thread kernel shape the splicer selects whenever a user
//    function calls them (get_global_id(0) == element index, as
//    include/SkelCL/detail/MapDef.h:187-195 relies on)
//  * barrier(CLK_*_MEM_FENCE) -> __syncthreads
//  * OpenCL vector types (float4 ...) with .x/.y/.z/.w and .s0.. members and
//    component-wise arithmetic; the host mirrors are in
//    include/SkelCL/detail/Types.h (layout: packed members, no padding)
//  * T_matrix_t + get/set for Matrix extra arguments
//    (include/SkelCL/detail/MatrixDef.h:834-867)
//  * skelcl_get_device_id() == 0 (one device; src/Program.cpp:236)
// ---------------------------------------------------------------------------
#define SCL_PRELUDE 1
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;
typedef unsigned long long scl_u64;
typedef long long scl_i64;

#define __kernel
#define __global
#define __local
#define __constant
#define __private
#define __read_only
#define __write_only
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
#define skelcl_get_device_id() 0

#ifndef SCL_WI_SWAP
#define SCL_WI_SWAP 0
#endif
#ifndef SCL_WORK_DIM
#define SCL_WORK_DIM 1
#endif

extern __shared__ __align__(128) unsigned char scl_dyn_smem[];

// Every template kernel's first statement is SCL_EXTRA_SETUP, which begins
// with this wait.  The host launches template kernels with programmatic
// stream serialization, so a grid may be scheduled before the previous
// kernel of the stream has finished; griddepcontrol.wait returns once that
// kernel has completed and its writes are visible (at once for a launch
// without the attribute).  Nothing before it touches global memory.
#define SCL_GRID_DEPENDENCY_WAIT asm volatile("griddepcontrol.wait;" ::: "memory");

__device__ __forceinline__ unsigned scl_cl_dim(unsigned d) {
  return SCL_WI_SWAP ? (d == 0u ? 1u : (d == 1u ? 0u : d)) : d;
}
__device__ __forceinline__ size_t get_local_id(uint d) {
  d = scl_cl_dim(d);
  return d == 0 ? threadIdx.x : (d == 1 ? threadIdx.y : (d == 2 ? threadIdx.z : 0));
}
__device__ __forceinline__ size_t get_group_id(uint d) {
  d = scl_cl_dim(d);
  return d == 0 ? blockIdx.x : (d == 1 ? blockIdx.y : (d == 2 ? blockIdx.z : 0));
}
__device__ __forceinline__ size_t get_local_size(uint d) {
  d = scl_cl_dim(d);
  return d == 0 ? blockDim.x : (d == 1 ? blockDim.y : (d == 2 ? blockDim.z : 1));
}
__device__ __forceinline__ size_t get_num_groups(uint d) {
  d = scl_cl_dim(d);
  return d == 0 ? gridDim.x : (d == 1 ? gridDim.y : (d == 2 ? gridDim.z : 1));
}
__device__ __forceinline__ size_t get_global_id(uint d) {
  return get_group_id(d) * get_local_size(d) + get_local_id(d);
}
__device__ __forceinline__ size_t get_global_size(uint d) {
  return get_num_groups(d) * get_local_size(d);
}
__device__ __forceinline__ size_t get_global_offset(uint) { return 0; }
__device__ __forceinline__ uint get_work_dim() { return SCL_WORK_DIM; }
__device__ __forceinline__ void barrier(int) { __syncthreads(); }
__device__ __forceinline__ void mem_fence(int) { __threadfence(); }
__device__ __forceinline__ void read_mem_fence(int) { __threadfence(); }
__device__ __forceinline__ void write_mem_fence(int) { __threadfence(); }

// ---- OpenCL scalar built-ins missing from CUDA -----------------------------
template <typename T> __device__ __forceinline__ T clamp(T x, T lo, T hi) {
  return x < lo ? lo : (x > hi ? hi : x);
}
__device__ __forceinline__ float clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ double clamp(double x, double lo, double hi) { return fmin(fmax(x, lo), hi); }
__device__ __forceinline__ float mad(float a, float b, float c) { return a * b + c; }
__device__ __forceinline__ double mad(double a, double b, double c) { return a * b + c; }
__device__ __forceinline__ int mad24(int a, int b, int c) { return a * b + c; }
__device__ __forceinline__ uint mad24(uint a, uint b, uint c) { return a * b + c; }
__device__ __forceinline__ int mul24(int a, int b) { return a * b; }
__device__ __forceinline__ uint mul24(uint a, uint b) { return a * b; }
__device__ __forceinline__ float mix(float x, float y, float a) { return x + (y - x) * a; }
__device__ __forceinline__ double mix(double x, double y, double a) { return x + (y - x) * a; }
__device__ __forceinline__ float sign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
__device__ __forceinline__ double sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }
__device__ __forceinline__ float step(float e, float x) { return x < e ? 0.f : 1.f; }
__device__ __forceinline__ float degrees(float r) { return r * 57.29577951308232f; }
__device__ __forceinline__ float radians(float d) { return d * 0.017453292519943295f; }
__device__ __forceinline__ float native_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ float native_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ float native_exp(float x) { return __expf(x); }
__device__ __forceinline__ float native_log(float x) { return __logf(x); }
__device__ __forceinline__ float native_sin(float x) { return __sinf(x); }
__device__ __forceinline__ float native_cos(float x) { return __cosf(x); }
__device__ __forceinline__ float native_divide(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float native_recip(float a) { return 1.0f / a; }
__device__ __forceinline__ float half_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ float half_exp(float x) { return __expf(x); }
__device__ __forceinline__ float as_float(int x) { return __int_as_float(x); }
__device__ __forceinline__ float as_float(uint x) { return __uint_as_float(x); }
__device__ __forceinline__ int as_int(float x) { return __float_as_int(x); }
__device__ __forceinline__ uint as_uint(float x) { return __float_as_uint(x); }
template <typename T> __device__ __forceinline__ T select(T a, T b, int c) { return c ? b : a; }
#define convert_int(x) ((int)(x))
#define convert_uint(x) ((uint)(x))
#define convert_float(x) ((float)(x))
#define convert_double(x) ((double)(x))
#define convert_long(x) ((long)(x))
#define convert_ulong(x) ((ulong)(x))
#define convert_char(x) ((char)(x))
#define convert_uchar(x) ((uchar)(x))
#define convert_short(x) ((short)(x))
#define convert_ushort(x) ((ushort)(x))
#define convert_int_rtz(x) ((int)(x))
#define convert_int_sat(x) ((int)(x))
#define convert_uchar_sat(x) ((uchar)((x) < 0 ? 0 : ((x) > 255 ? 255 : (x))))

// ---- OpenCL vector types ----------------------------------------------------
// Component names x/y/z/w alias s0..s3 (OpenCL C 1.2 section 6.1.7).
#define SCL_VT2(T, N)                                                       \
  struct scl_##N##2 { union { struct { T x, y; }; struct { T s0, s1; }; }; };
#define SCL_VT4(T, N)                                                       \
  struct scl_##N##4 { union { struct { T x, y, z, w; };                     \
                              struct { T s0, s1, s2, s3; }; }; };
#define SCL_VT8(T, N)                                                       \
  struct scl_##N##8 { T s0, s1, s2, s3, s4, s5, s6, s7; };
#define SCL_VT16(T, N)                                                      \
  struct scl_##N##16 { T s0, s1, s2, s3, s4, s5, s6, s7,                    \
                       s8, s9, sa, sb, sc, sd, se, sf; };

#define SCL_VOPS(V, T, K)                                                   \
  __device__ __forceinline__ V operator-(V a) {                             \
    T* p = (T*)&a; _Pragma("unroll") for (int i = 0; i < K; ++i) p[i] = -p[i]; return a; } \
  __device__ __forceinline__ V operator+(V a) { return a; }                  \
  SCL_VBIN(V, T, K, +) SCL_VBIN(V, T, K, -) SCL_VBIN(V, T, K, *) SCL_VBIN(V, T, K, /)

#define SCL_VBIN(V, T, K, OP)                                               \
  __device__ __forceinline__ V operator OP(V a, V b) {                      \
    T* p = (T*)&a; const T* q = (const T*)&b;                               \
    _Pragma("unroll") for (int i = 0; i < K; ++i) p[i] = p[i] OP q[i]; return a; } \
  __device__ __forceinline__ V operator OP(V a, T s) {                      \
    T* p = (T*)&a; _Pragma("unroll") for (int i = 0; i < K; ++i) p[i] = p[i] OP s; return a; } \
  __device__ __forceinline__ V operator OP(T s, V a) {                      \
    T* p = (T*)&a; _Pragma("unroll") for (int i = 0; i < K; ++i) p[i] = s OP p[i]; return a; } \
  __device__ __forceinline__ V& operator OP##=(V& a, V b) { a = a OP b; return a; } \
  __device__ __forceinline__ V& operator OP##=(V& a, T s) { a = a OP s; return a; }

#define SCL_VFAMILY(T, N)                                                   \
  SCL_VT2(T, N) SCL_VT4(T, N) SCL_VT8(T, N) SCL_VT16(T, N)                  \
  SCL_VOPS(scl_##N##2, T, 2) SCL_VOPS(scl_##N##4, T, 4)                      \
  SCL_VOPS(scl_##N##8, T, 8) SCL_VOPS(scl_##N##16, T, 16)                    \
  typedef scl_##N##4 scl_##N##3;

SCL_VFAMILY(char, char)
SCL_VFAMILY(unsigned char, uchar)
SCL_VFAMILY(short, short)
SCL_VFAMILY(unsigned short, ushort)
SCL_VFAMILY(int, int)
SCL_VFAMILY(unsigned int, uint)
SCL_VFAMILY(long, long)
SCL_VFAMILY(unsigned long, ulong)
SCL_VFAMILY(float, float)
SCL_VFAMILY(double, double)

#define char2 scl_char2
#define char3 scl_char3
#define char4 scl_char4
#define char8 scl_char8
#define char16 scl_char16
#define uchar2 scl_uchar2
#define uchar3 scl_uchar3
#define uchar4 scl_uchar4
#define uchar8 scl_uchar8
#define uchar16 scl_uchar16
#define short2 scl_short2
#define short3 scl_short3
#define short4 scl_short4
#define short8 scl_short8
#define short16 scl_short16
#define ushort2 scl_ushort2
#define ushort3 scl_ushort3
#define ushort4 scl_ushort4
#define ushort8 scl_ushort8
#define ushort16 scl_ushort16
#define int2 scl_int2
#define int3 scl_int3
#define int4 scl_int4
#define int8 scl_int8
#define int16 scl_int16
#define uint2 scl_uint2
#define uint3 scl_uint3
#define uint4 scl_uint4
#define uint8 scl_uint8
#define uint16 scl_uint16
#define long2 scl_long2
#define long3 scl_long3
#define long4 scl_long4
#define long8 scl_long8
#define long16 scl_long16
#define ulong2 scl_ulong2
#define ulong3 scl_ulong3
#define ulong4 scl_ulong4
#define ulong8 scl_ulong8
#define ulong16 scl_ulong16
#define float2 scl_float2
#define float3 scl_float3
#define float4 scl_float4
#define float8 scl_float8
#define float16 scl_float16
#define double2 scl_double2
#define double3 scl_double3
#define double4 scl_double4
#define double8 scl_double8
#define double16 scl_double16

// ---- Matrix extra arguments: T_matrix_t + get/set ---------------------------
#define SCL_MATRIX_T(T, N) typedef struct { T* data; unsigned int col_count; } N##_matrix_t;
SCL_MATRIX_T(char, char)
SCL_MATRIX_T(unsigned char, uchar)
SCL_MATRIX_T(short, short)
SCL_MATRIX_T(unsigned short, ushort)
SCL_MATRIX_T(int, int)
SCL_MATRIX_T(unsigned int, uint)
SCL_MATRIX_T(long, long)
SCL_MATRIX_T(unsigned long, ulong)
SCL_MATRIX_T(float, float)
SCL_MATRIX_T(double, double)
SCL_MATRIX_T(scl_float2, float2)
SCL_MATRIX_T(scl_float4, float4)
SCL_MATRIX_T(scl_int2, int2)
SCL_MATRIX_T(scl_int4, int4)
SCL_MATRIX_T(scl_double2, double2)
SCL_MATRIX_T(scl_double4, double4)
#define unsigned_int_matrix_t uint_matrix_t
#define char_MATRIX_T
#define uchar_MATRIX_T
#define short_MATRIX_T
#define ushort_MATRIX_T
#define int_MATRIX_T
#define uint_MATRIX_T
#define unsigned_int_MATRIX_T
#define long_MATRIX_T
#define ulong_MATRIX_T
#define float_MATRIX_T
#define double_MATRIX_T
#define float2_MATRIX_T
#define float4_MATRIX_T
#define int2_MATRIX_T
#define int4_MATRIX_T
#define double2_MATRIX_T
#define double4_MATRIX_T
#define MATRIX_GET
#define MATRIX_SET
#define get(m, y, x) (m).data[(int)((y) * (m).col_count + (x))]
#define set(m, y, x, v) (m).data[(int)((y) * (m).col_count + (x))] = (v)

// ---- skeleton-side helpers ---------------------------------------------------
#define SCL_TID() ((scl_u64)blockIdx.x * blockDim.x + threadIdx.x)
#define SCL_NTH() ((scl_u64)gridDim.x * blockDim.x)
// 16-, 8- and 4-byte raw words for vectorised global accesses.
struct __align__(16) scl_raw16 { unsigned int a, b, c, d; };
struct __align__(8) scl_raw8 { unsigned int a, b; };

template <typename T, int V> struct scl_pack { T v[V]; };

template <typename T, int V>
__device__ __forceinline__ scl_pack<T, V> scl_load(const T* p) {
  scl_pack<T, V> r;
  constexpr int B = (int)sizeof(T) * V;
  if constexpr (B == 16) {
    scl_raw16 w = *reinterpret_cast<const scl_raw16*>(p);
    memcpy(&r, &w, 16);
  } else if constexpr (B == 8) {
    scl_raw8 w = *reinterpret_cast<const scl_raw8*>(p);
    memcpy(&r, &w, 8);
  } else if constexpr (B == 4) {
    unsigned int w = *reinterpret_cast<const unsigned int*>(p);
    memcpy(&r, &w, 4);
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) r.v[i] = p[i];
  }
  return r;
}

template <typename T, int V>
__device__ __forceinline__ void scl_store(T* p, const scl_pack<T, V>& r) {
  constexpr int B = (int)sizeof(T) * V;
  if constexpr (B == 16) {
    scl_raw16 w; memcpy(&w, &r, 16);
    *reinterpret_cast<scl_raw16*>(p) = w;
  } else if constexpr (B == 8) {
    scl_raw8 w; memcpy(&w, &r, 8);
    *reinterpret_cast<scl_raw8*>(p) = w;
  } else if constexpr (B == 4) {
    unsigned int w; memcpy(&w, &r, 4);
    *reinterpret_cast<unsigned int*>(p) = w;
  } else {
#pragma unroll
    for (int i = 0; i < V; ++i) p[i] = r.v[i];
  }
}

// Elements per 16-byte access for the widest of up to three element types;
// 1 when a type does not tile 16 bytes.
template <int S0, int S1 = 1, int S2 = 1>
struct scl_vec_width {
  static constexpr int S = S0 > S1 ? (S0 > S2 ? S0 : S2) : (S1 > S2 ? S1 : S2);
  static constexpr int value = (S <= 16 && 16 % S == 0 && 16 % S0 == 0 &&
                                16 % S1 == 0 && 16 % S2 == 0) ? 16 / S : 1;
};

// Segment-plan windows: a vector of at most this many elements is folded or
// scanned by one thread, a longer one by a warp.
#define SCL_WIN_THREAD 256

// Device-side status word: bit 0 = a bounded wait gave up.
#define SCL_DEV_ERR_TIMEOUT 1u
__device__ __forceinline__ void scl_raise(unsigned int* err, unsigned int bit) {
  if (err) atomicOr(err, bit);
}
__device__ __forceinline__ void scl_nanosleep(unsigned int ns) {
  asm volatile("nanosleep.u32 %0;" :: "r"(ns));
}

// Bounded wait for phase 0 of the mbarrier at shared address bar_s: false
// after spin_limit polls without completion.
__device__ __forceinline__ bool scl_mbar_wait(unsigned int bar_s, unsigned int spin_limit) {
  unsigned int done = 0, polls = 0;
  while (!done) {
    asm volatile(
        "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 0;"
        " selp.u32 %0, 1, 0, p; }"
        : "=r"(done) : "r"(bar_s) : "memory");
    if (!done) {
      if (++polls > spin_limit) return false;
      if (polls > 16) scl_nanosleep(32);
    }
  }
  return true;
}

// Starts bringing src[0 .. len) into shared memory so that src[p] lands at
// ts[p + shift] (ts 16-byte aligned, room for len + 16 / sizeof(T)
// elements); returns shift, the elements between src and the 16-byte
// boundary below it, so that 16-byte-aligned global addresses meet
// 16-byte-aligned shared ones.  The 16-byte-aligned interior of the
// range goes by bulk asynchronous copies that thread 0 issues on the
// mbarrier bar_s (initialised by the caller, phase 0); *tx receives the bytes
// it counts (0: nothing issued, no wait needed).  The ragged ends (under 16
// bytes each) are read by ordinary loads of the calling threads, so nothing
// outside the range is read.  Elements that do not tile 16 bytes, or do not
// sit on their own size, are all read by ordinary loads (shift 0).  The
// caller waits on the mbarrier (thread 0) and then synchronises the block.
template <typename T, int B>
__device__ __forceinline__ int scl_stage_bulk(const T* src, int len, T* ts, unsigned int bar_s,
                                              unsigned int* tx) {
  constexpr int V = scl_vec_width<sizeof(T)>::value;
  *tx = 0u;
  const unsigned long long addr = (unsigned long long)src;
  if (V == 1 || addr % sizeof(T) != 0 || len <= 0) {
    for (int p = threadIdx.x; p < len; p += B) ts[p] = src[p];
    return 0;
  }
  const int shift = (int)((addr & 15u) / sizeof(T));
  const int head = shift ? V - shift : 0;  // elements before the first boundary
  const int lo = head < len ? head : len;
  const int hi_raw = (shift + len) / V * V - shift;  // end of the aligned interior
  const int hi = hi_raw > lo ? hi_raw : lo;
  if (hi > lo) {
    const unsigned int bytes = (unsigned int)((hi - lo) * (int)sizeof(T));
    *tx = bytes;
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                   :: "r"(bar_s), "r"(bytes) : "memory");
      const unsigned int dst = (unsigned int)__cvta_generic_to_shared(ts + lo + shift);
      constexpr unsigned int CHUNK = 8192;  // bytes per copy
      for (unsigned int o = 0; o < bytes; o += CHUNK) {
        const unsigned int sz = bytes - o < CHUNK ? bytes - o : CHUNK;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
            :: "r"(dst + o), "l"((const void*)((const char*)(src + lo) + o)), "r"(sz), "r"(bar_s)
            : "memory");
      }
    }
  }
  // the ragged ends
  const int ntail = len - hi;
  if ((int)threadIdx.x < lo) ts[threadIdx.x + shift] = src[threadIdx.x];
  if ((int)threadIdx.x < ntail) ts[hi + threadIdx.x + shift] = src[hi + threadIdx.x];
  return shift;
}

__device__ __forceinline__ unsigned int scl_ld_acquire(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void scl_st_release(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
