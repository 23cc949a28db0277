// ---------------------------------------------------------------------------
// Element-wise skeletons for sm_103a: Map (all six specialisations) and Zip.
//
// Semantics follow the reference kernels SCL_MAP / SCL_ZIP
// (include/SkelCL/detail/MapDef.h:187-195,306-313,442-450,653-665,
//  src/Map.cpp, include/SkelCL/detail/ZipDef.h:197-206,390-397):
// out[i] = f(in[i], extra...) for every i < n.
//
// Two kernel shapes:
//  * scl_*_k<U>   grid-stride, 16-byte vector accesses, U independent vectors
//                 in flight per thread (HBM-bound shape; the user function
//                 must not use work-item functions or barriers)
//  * scl_*_simple one element per thread in whole blocks, exactly the
//                 reference NDRange: get_global_id(0) is the element index
//                 and barrier() / __local work (test/MapTests.cpp:348-365)
//
// Names provided by the generated header: SCL_KIND, SCL_TYPE_n, SCL_FUNC,
// SCL_EXTRA_PARAMS / SCL_EXTRA_SETUP / SCL_EXTRA_ARGS.
// ---------------------------------------------------------------------------

#if SCL_KIND == 1  // ---------------------------- Map<Tout(Tin)>
template <int U>
__global__ void scl_map_k(const SCL_TYPE_0* in, SCL_TYPE_1* out, scl_u64 n,
                          int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0), sizeof(SCL_TYPE_1)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  const scl_u64 nvec = aligned ? n / V : 0;
  for (scl_u64 j = tid; j < nvec; j += nth * U) {
    scl_pack<SCL_TYPE_0, V> a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) a[u] = scl_load<SCL_TYPE_0, V>(in + k * V);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
        scl_pack<SCL_TYPE_1, V> r;
#pragma unroll
        for (int e = 0; e < V; ++e) r.v[e] = SCL_FUNC(a[u].v[e] SCL_EXTRA_ARGS);
        scl_store<SCL_TYPE_1, V>(out + k * V, r);
      }
    }
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth) out[i] = SCL_FUNC(in[i] SCL_EXTRA_ARGS);
}
extern "C" __global__ void scl_map_simple(const SCL_TYPE_0* in, SCL_TYPE_1* out,
                                          scl_u64 n SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) out[i] = SCL_FUNC(in[i] SCL_EXTRA_ARGS);
}

#elif SCL_KIND == 2  // ------------------------- Map<void(Tin)>
template <int U>
__global__ void scl_map_k(const SCL_TYPE_0* in, scl_u64 n, int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  const scl_u64 nvec = aligned ? n / V : 0;
  for (scl_u64 j = tid; j < nvec; j += nth * U) {
    scl_pack<SCL_TYPE_0, V> a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) a[u] = scl_load<SCL_TYPE_0, V>(in + k * V);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
#pragma unroll
        for (int e = 0; e < V; ++e) SCL_FUNC(a[u].v[e] SCL_EXTRA_ARGS);
      }
    }
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth) SCL_FUNC(in[i] SCL_EXTRA_ARGS);
}
extern "C" __global__ void scl_map_simple(const SCL_TYPE_0* in, scl_u64 n SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) SCL_FUNC(in[i] SCL_EXTRA_ARGS);
}

#elif SCL_KIND == 3  // ------------------------- Map<Tout(Index)>
template <int U>
__global__ void scl_map_k(SCL_TYPE_0* out, scl_u64 n, scl_u64 offset,
                          int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  const scl_u64 nvec = aligned ? n / V : 0;
  for (scl_u64 k = tid; k < nvec; k += nth) {
    scl_pack<SCL_TYPE_0, V> r;
#pragma unroll
    for (int e = 0; e < V; ++e) r.v[e] = SCL_FUNC((Index)(k * V + e + offset) SCL_EXTRA_ARGS);
    scl_store<SCL_TYPE_0, V>(out + k * V, r);
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth)
    out[i] = SCL_FUNC((Index)(i + offset) SCL_EXTRA_ARGS);
}
extern "C" __global__ void scl_map_simple(SCL_TYPE_0* out, scl_u64 n,
                                          scl_u64 offset SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) out[i] = SCL_FUNC((Index)(i + offset) SCL_EXTRA_ARGS);
}

#elif SCL_KIND == 4  // ------------------------- Map<void(Index)>
template <int U>
__global__ void scl_map_k(scl_u64 n, scl_u64 offset, int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  for (scl_u64 i = tid; i < n; i += nth) SCL_FUNC((Index)(i + offset) SCL_EXTRA_ARGS);
}
extern "C" __global__ void scl_map_simple(scl_u64 n, scl_u64 offset SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) SCL_FUNC((Index)(i + offset) SCL_EXTRA_ARGS);
}

#elif SCL_KIND == 5  // ------------------------- Map<Tout(IndexPoint)>
// Columns run along x (coalesced row-major stores); rows along the grid's y.
template <int U>
__global__ void scl_map_k(SCL_TYPE_0* out, scl_u64 rows, scl_u64 cols,
                          scl_u64 row_offset, int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  for (scl_u64 y = blockIdx.y; y < rows; y += gridDim.y)
    for (scl_u64 x = (scl_u64)blockIdx.x * blockDim.x + threadIdx.x; x < cols;
         x += (scl_u64)gridDim.x * blockDim.x) {
      IndexPoint p;
      p.x = x;
      p.y = y + row_offset;
      out[y * cols + x] = SCL_FUNC(p SCL_EXTRA_ARGS);
    }
}
// Reference NDRange: dim 0 = rows, dim 1 = columns (MapDef.h:653-665).
extern "C" __global__ void scl_map_simple(SCL_TYPE_0* out, scl_u64 rows, scl_u64 cols,
                                          scl_u64 row_offset SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t y = get_global_id(0), x = get_global_id(1);
  if (y < rows && x < cols) {
    IndexPoint p;
    p.x = x;
    p.y = y + row_offset;
    out[y * cols + x] = SCL_FUNC(p SCL_EXTRA_ARGS);
  }
}

#elif SCL_KIND == 6  // ------------------------- Map<void(IndexPoint)>
template <int U>
__global__ void scl_map_k(scl_u64 rows, scl_u64 cols, scl_u64 row_offset,
                          int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  for (scl_u64 y = blockIdx.y; y < rows; y += gridDim.y)
    for (scl_u64 x = (scl_u64)blockIdx.x * blockDim.x + threadIdx.x; x < cols;
         x += (scl_u64)gridDim.x * blockDim.x) {
      IndexPoint p;
      p.x = x;
      p.y = y + row_offset;
      SCL_FUNC(p SCL_EXTRA_ARGS);
    }
}
extern "C" __global__ void scl_map_simple(scl_u64 rows, scl_u64 cols,
                                          scl_u64 row_offset SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t y = get_global_id(0), x = get_global_id(1);
  if (y < rows && x < cols) {
    IndexPoint p;
    p.x = x;
    p.y = y + row_offset;
    SCL_FUNC(p SCL_EXTRA_ARGS);
  }
}

#elif SCL_KIND == 7  // ------------------------- Zip<Tout(Tl,Tr)>
template <int U>
__global__ void scl_map_k(const SCL_TYPE_0* left, const SCL_TYPE_1* right,
                          SCL_TYPE_2* out, scl_u64 n, int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0), sizeof(SCL_TYPE_1),
                                  sizeof(SCL_TYPE_2)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  const scl_u64 nvec = aligned ? n / V : 0;
  for (scl_u64 j = tid; j < nvec; j += nth * U) {
    scl_pack<SCL_TYPE_0, V> a[U];
    scl_pack<SCL_TYPE_1, V> b[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
        a[u] = scl_load<SCL_TYPE_0, V>(left + k * V);
        b[u] = scl_load<SCL_TYPE_1, V>(right + k * V);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
        scl_pack<SCL_TYPE_2, V> r;
#pragma unroll
        for (int e = 0; e < V; ++e) r.v[e] = SCL_FUNC(a[u].v[e], b[u].v[e] SCL_EXTRA_ARGS);
        scl_store<SCL_TYPE_2, V>(out + k * V, r);
      }
    }
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth)
    out[i] = SCL_FUNC(left[i], right[i] SCL_EXTRA_ARGS);
}
extern "C" __global__ void scl_map_simple(const SCL_TYPE_0* left, const SCL_TYPE_1* right,
                                          SCL_TYPE_2* out, scl_u64 n SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) out[i] = SCL_FUNC(left[i], right[i] SCL_EXTRA_ARGS);
}

#elif SCL_KIND == 8  // ------------------------- Zip<void(Tl,Tr)>
template <int U>
__global__ void scl_map_k(const SCL_TYPE_0* left, const SCL_TYPE_1* right, scl_u64 n,
                          int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0), sizeof(SCL_TYPE_1)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  const scl_u64 nvec = aligned ? n / V : 0;
  for (scl_u64 k = tid; k < nvec; k += nth) {
    scl_pack<SCL_TYPE_0, V> a = scl_load<SCL_TYPE_0, V>(left + k * V);
    scl_pack<SCL_TYPE_1, V> b = scl_load<SCL_TYPE_1, V>(right + k * V);
#pragma unroll
    for (int e = 0; e < V; ++e) SCL_FUNC(a.v[e], b.v[e] SCL_EXTRA_ARGS);
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth) SCL_FUNC(left[i], right[i] SCL_EXTRA_ARGS);
}
extern "C" __global__ void scl_map_simple(const SCL_TYPE_0* left, const SCL_TYPE_1* right,
                                          scl_u64 n SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) SCL_FUNC(left[i], right[i] SCL_EXTRA_ARGS);
}
#endif

// ---------------------------------------------------------------------------
// Adjoints of Map and Zip (no counterpart in the reference).  The user gives
// the vector-Jacobian product as source:
//   Map<Tout(Tin)>:     Tin  d (Tin x, Tout g, extra...)          -> SCL_FUNC
//   Zip<Tout(Tl,Tr)>:   Tl   dl(Tl x, Tr y, Tout g, extra...)     -> SCL_FUNC
//                       Tr   dr(Tl x, Tr y, Tout g, extra...)     -> SCL_FUNC2
// and the kernels write gx[i] = d(x[i], g[i]) or, with `acc` set, add it to
// gx[i] (bit 0: gx, bit 1: gy).  A null gx / gy is skipped.
// ---------------------------------------------------------------------------
#if SCL_KIND == 14  // ------------------------ adjoint of Map<Tout(Tin)>
template <int U>
__global__ void scl_map_k(const SCL_TYPE_0* x, const SCL_TYPE_1* g, SCL_TYPE_0* gx, scl_u64 n,
                          int acc, int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0), sizeof(SCL_TYPE_1)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  const scl_u64 nvec = aligned ? n / V : 0;
  for (scl_u64 j = tid; j < nvec; j += nth * U) {
    scl_pack<SCL_TYPE_0, V> a[U], o[U];
    scl_pack<SCL_TYPE_1, V> b[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
        a[u] = scl_load<SCL_TYPE_0, V>(x + k * V);
        b[u] = scl_load<SCL_TYPE_1, V>(g + k * V);
        if (acc) o[u] = scl_load<SCL_TYPE_0, V>(gx + k * V);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
        scl_pack<SCL_TYPE_0, V> r;
#pragma unroll
        for (int e = 0; e < V; ++e) {
          r.v[e] = SCL_FUNC(a[u].v[e], b[u].v[e] SCL_EXTRA_ARGS);
          if (acc) r.v[e] = o[u].v[e] + r.v[e];
        }
        scl_store<SCL_TYPE_0, V>(gx + k * V, r);
      }
    }
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth) {
    SCL_TYPE_0 r = SCL_FUNC(x[i], g[i] SCL_EXTRA_ARGS);
    gx[i] = acc ? gx[i] + r : r;
  }
}
extern "C" __global__ void scl_map_simple(const SCL_TYPE_0* x, const SCL_TYPE_1* g,
                                          SCL_TYPE_0* gx, scl_u64 n, int acc SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) {
    SCL_TYPE_0 r = SCL_FUNC(x[i], g[i] SCL_EXTRA_ARGS);
    gx[i] = acc ? gx[i] + r : r;
  }
}

#elif SCL_KIND == 15  // ----------------------- adjoint of Zip<Tout(Tl,Tr)>
#ifndef SCL_HAS_FUNC2
#define SCL_FUNC2(...) SCL_TYPE_1()
#endif
template <int U>
__global__ void scl_map_k(const SCL_TYPE_0* x, const SCL_TYPE_1* y, const SCL_TYPE_2* g,
                          SCL_TYPE_0* gx, SCL_TYPE_1* gy, scl_u64 n, int acc,
                          int aligned SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0), sizeof(SCL_TYPE_1),
                                  sizeof(SCL_TYPE_2)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  const scl_u64 nvec = aligned ? n / V : 0;
  const bool wx = gx != nullptr, wy = gy != nullptr;
  const bool ax = wx && (acc & 1), ay = wy && (acc & 2);
  for (scl_u64 j = tid; j < nvec; j += nth * U) {
    scl_pack<SCL_TYPE_0, V> a[U], ox[U];
    scl_pack<SCL_TYPE_1, V> b[U], oy[U];
    scl_pack<SCL_TYPE_2, V> c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
        a[u] = scl_load<SCL_TYPE_0, V>(x + k * V);
        b[u] = scl_load<SCL_TYPE_1, V>(y + k * V);
        c[u] = scl_load<SCL_TYPE_2, V>(g + k * V);
        if (ax) ox[u] = scl_load<SCL_TYPE_0, V>(gx + k * V);
        if (ay) oy[u] = scl_load<SCL_TYPE_1, V>(gy + k * V);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
        if (wx) {
          scl_pack<SCL_TYPE_0, V> r;
#pragma unroll
          for (int e = 0; e < V; ++e) {
            r.v[e] = SCL_FUNC(a[u].v[e], b[u].v[e], c[u].v[e] SCL_EXTRA_ARGS);
            if (ax) r.v[e] = ox[u].v[e] + r.v[e];
          }
          scl_store<SCL_TYPE_0, V>(gx + k * V, r);
        }
        if (wy) {
          scl_pack<SCL_TYPE_1, V> r;
#pragma unroll
          for (int e = 0; e < V; ++e) {
            r.v[e] = SCL_FUNC2(a[u].v[e], b[u].v[e], c[u].v[e] SCL_EXTRA_ARGS);
            if (ay) r.v[e] = oy[u].v[e] + r.v[e];
          }
          scl_store<SCL_TYPE_1, V>(gy + k * V, r);
        }
      }
    }
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth) {
    if (wx) {
      SCL_TYPE_0 r = SCL_FUNC(x[i], y[i], g[i] SCL_EXTRA_ARGS);
      gx[i] = ax ? gx[i] + r : r;
    }
    if (wy) {
      SCL_TYPE_1 r = SCL_FUNC2(x[i], y[i], g[i] SCL_EXTRA_ARGS);
      gy[i] = ay ? gy[i] + r : r;
    }
  }
}
extern "C" __global__ void scl_map_simple(const SCL_TYPE_0* x, const SCL_TYPE_1* y,
                                          const SCL_TYPE_2* g, SCL_TYPE_0* gx, SCL_TYPE_1* gy,
                                          scl_u64 n, int acc SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const size_t i = get_global_id(0);
  if (i < n) {
    if (gx) {
      SCL_TYPE_0 r = SCL_FUNC(x[i], y[i], g[i] SCL_EXTRA_ARGS);
      gx[i] = (acc & 1) ? gx[i] + r : r;
    }
    if (gy) {
      SCL_TYPE_1 r = SCL_FUNC2(x[i], y[i], g[i] SCL_EXTRA_ARGS);
      gy[i] = (acc & 2) ? gy[i] + r : r;
    }
  }
}
#endif
