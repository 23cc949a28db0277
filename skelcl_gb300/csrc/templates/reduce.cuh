// ---------------------------------------------------------------------------
// Reduce for sm_103a: ONE launch.  Replaces the reference's two kernels
// SCL_REDUCE_1 (8192 work-items, strided fold) and SCL_REDUCE_2 (one work-group
// tree) of include/SkelCL/detail/ReduceKernel.cl:51-128 and
// include/SkelCL/detail/ReduceDef.h:98-245.
//
// Semantics kept from the reference:
//  * the identity is not used to seed the fold: every partial starts from a
//    real element (ReduceKernel.cl:60-61), so a non-neutral `id` string has
//    no effect, as in the reference;
//  * the operator is assumed associative and commutative (the reference folds
//    element j, j+8192, j+2*8192 ... and then a tree);
//  * the result is a one-element vector (ReduceDef.h:113-121).
// Empty input (the reference reads out of bounds there) yields SCL_IDENTITY.
//
// Shape: grid-stride 16-byte loads, per-thread fold in T, then warp-shuffle
// and block folds in the carry type SCL_CARRY_T (double for float element
// types: "cross-block carries in FP64"), one partial per block, and the last
// block to finish (atomic ticket) folds the partials in block order and
// resets the ticket for the next launch.
// ---------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T scl_shfl_down(const T& v, int off) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  unsigned int w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __shfl_down_sync(0xffffffffu, w[i], off);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}
template <typename T>
__device__ __forceinline__ T scl_shfl_up(const T& v, int off) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  unsigned int w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __shfl_up_sync(0xffffffffu, w[i], off);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}
template <typename T>
__device__ __forceinline__ T scl_shfl_idx(const T& v, int src) {
  constexpr int W = (int)((sizeof(T) + 3) / 4);
  unsigned int w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __shfl_sync(0xffffffffu, w[i], src);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}
// Coherent (L1-bypassing) copy of a value written by another block.
template <typename T>
__device__ __forceinline__ T scl_ld_cg(const T* p) {
  T r;
  if constexpr (sizeof(T) % 4 == 0) {
    unsigned int w[sizeof(T) / 4];
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); ++i)
      w[i] = *((const volatile unsigned int*)p + i);
    memcpy(&r, w, sizeof(T));
  } else {
    unsigned char b[sizeof(T)];
#pragma unroll
    for (int i = 0; i < (int)sizeof(T); ++i) b[i] = *((const volatile unsigned char*)p + i);
    memcpy(&r, b, sizeof(T));
  }
  return r;
}
template <typename T>
__device__ __forceinline__ void scl_st_cg(T* p, const T& v) {
  if constexpr (sizeof(T) % 4 == 0) {
    unsigned int w[sizeof(T) / 4];
    memcpy(w, &v, sizeof(T));
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); ++i) *((volatile unsigned int*)p + i) = w[i];
  } else {
    unsigned char b[sizeof(T)];
    memcpy(b, &v, sizeof(T));
#pragma unroll
    for (int i = 0; i < (int)sizeof(T); ++i) *((volatile unsigned char*)p + i) = b[i];
  }
}

#if SCL_KIND == 9 || SCL_KIND == 16
#if SCL_KIND == 16
typedef SCL_TYPE_2 scl_T;  // the zipped element type folded by the Reduce
#else
typedef SCL_TYPE_0 scl_T;
#endif
typedef SCL_CARRY_T scl_C;

// Fold (have, value) pairs across a warp; lane 0 ends with the warp's fold.
__device__ __forceinline__ void scl_warp_fold(bool& have, scl_C& c SCL_USER_PARAMS) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    scl_C o = scl_shfl_down(c, off);
    bool oh = __shfl_down_sync(0xffffffffu, have ? 1 : 0, off) != 0;
    if ((threadIdx.x & 31) + off < 32 && oh) {
      c = have ? (scl_C)SCL_FUNC_C(c, o SCL_OP_ARGS) : o;
      have = true;
    }
  }
}

// Block fold; the result is valid in thread 0.
__device__ __forceinline__ void scl_block_fold(bool& have, scl_C& c SCL_USER_PARAMS) {
  __shared__ scl_C s_val[32];
  __shared__ int s_have[32];
  scl_warp_fold(have, c SCL_EXTRA_ARGS);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  if (lane == 0) {
    s_val[warp] = c;
    s_have[warp] = have ? 1 : 0;
  }
  __syncthreads();
  if (warp == 0) {
    have = lane < nwarps && s_have[lane];
    if (have) c = s_val[lane];
    scl_warp_fold(have, c SCL_EXTRA_ARGS);
  }
  __syncthreads();
}

#if SCL_KIND == 9
template <int U>
__global__ void scl_reduce_k(const scl_T* in, scl_T* out, scl_u64 n, int aligned,
                             scl_C* partials, unsigned int* ticket,
                             unsigned int* err SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(scl_T)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  if (n == 0) {
    if (tid == 0) out[0] = (scl_T)(SCL_IDENTITY);
    return;
  }
  const scl_u64 nvec = aligned ? n / V : 0;
  bool have = false;
  scl_T acc;
  scl_u64 j = tid;
  if (j < nvec) {
    scl_pack<scl_T, V> p = scl_load<scl_T, V>(in + j * V);
    acc = p.v[0];
#pragma unroll
    for (int e = 1; e < V; ++e) acc = SCL_FUNC(acc, p.v[e] SCL_OP_ARGS);
    have = true;
    j += nth;
  }
  for (; j < nvec; j += nth * U) {
    scl_pack<scl_T, V> a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) a[u] = scl_load<scl_T, V>(in + k * V);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const scl_u64 k = j + (scl_u64)u * nth;
      if (k < nvec) {
#pragma unroll
        for (int e = 0; e < V; ++e) acc = SCL_FUNC(acc, a[u].v[e] SCL_OP_ARGS);
      }
    }
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth) {
    acc = have ? SCL_FUNC(acc, in[i] SCL_OP_ARGS) : in[i];
    have = true;
  }
  scl_C c;
  if (have) c = (scl_C)acc;
  scl_block_fold(have, c SCL_EXTRA_ARGS);

  __shared__ int s_last;
  if (threadIdx.x == 0) {
    // every block holds at least one element (the host sizes the grid so)
    scl_st_cg(&partials[blockIdx.x], c);
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  have = false;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    scl_C v = scl_ld_cg(&partials[b]);
    c = have ? (scl_C)SCL_FUNC_C(c, v SCL_OP_ARGS) : v;
    have = true;
  }
  scl_block_fold(have, c SCL_EXTRA_ARGS);
  if (threadIdx.x == 0) {
    out[0] = (scl_T)c;
    *ticket = 0u;  // ready for the next launch on this workspace
  }
}

// Segments of at most short_max elements (empty ones included: SCL_IDENTITY):
// one warp each, warps striding over the segments (warp `wid` of `nw`), U
// elements per lane in flight, folded in the element type (no block boundary
// is crossed; FP64 folds here would make the FP64 pipe the bound for tiny
// segments); longer segments are left to the tiles.
template <int U>
__device__ __forceinline__ void scl_reduce_short_run(const scl_T* in, scl_T* out, const scl_u64* seg_off,
                                                     scl_u64 n_seg, scl_u64 short_max, scl_u64 wid,
                                                     scl_u64 nw SCL_USER_PARAMS) {
  const int lane = threadIdx.x & 31;
  scl_u64 sg = wid;
  // the next segment's offsets are loaded while this one is folded
  scl_u64 lo_next = sg < n_seg ? seg_off[sg] : 0, hi_next = sg < n_seg ? seg_off[sg + 1] : 0;
  for (; sg < n_seg; sg += nw) {
    const scl_u64 lo = lo_next;
    const scl_u64 len = hi_next > lo ? hi_next - lo : 0;
    if (sg + nw < n_seg) {
      lo_next = seg_off[sg + nw];
      hi_next = seg_off[sg + nw + 1];
    }
    if (len > short_max) continue;
    bool have = false;
    scl_T acc;
    for (scl_u64 b = 0; b < len; b += 32 * U) {
      scl_T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const scl_u64 e = b + (scl_u64)(u * 32 + lane);
        if (e < len) v[u] = in[lo + e];
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (b + (scl_u64)(u * 32 + lane) < len) {
          acc = have ? SCL_FUNC(acc, v[u] SCL_OP_ARGS) : v[u];
          have = true;
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const scl_T o = scl_shfl_down(acc, off);
      const bool oh = __shfl_down_sync(0xffffffffu, have ? 1 : 0, off) != 0;
      if (lane + off < 32 && oh) {
        acc = have ? SCL_FUNC(acc, o SCL_OP_ARGS) : o;
        have = true;
      }
    }
    if (lane == 0) out[sg] = have ? acc : (scl_T)(SCL_IDENTITY);
  }
}

// The warp-per-segment kernel on its own (segmented launches without a
// segment plan; with one, scl_reduce_seg<R, 1> runs the same code in the
// blocks past the tiles).
template <int U>
__global__ void __launch_bounds__(256)
scl_reduce_short(const scl_T* in, scl_T* out, const scl_u64* seg_off, scl_u64 n_seg,
                 scl_u64 short_max SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  scl_reduce_short_run<U>(in, out, seg_off, n_seg, short_max,
                          ((scl_u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                          ((scl_u64)gridDim.x * blockDim.x) >> 5 SCL_EXTRA_ARGS);
}

// Window role of a planned segmented Reduce (the blocks past the tiles):
// block r takes window record r of the plan, {first vector, end vector,
// first element, elements}: consecutive vectors of at most short_max elements
// that start in one window of short_max elements (all but the last end
// inside it, so the record spans at most 2 * short_max = WT elements).  The
// record's elements are brought into shared memory by bulk asynchronous
// copies (element e0 + p at ts[p + shift]; bounded wait) while each thread
// reads its first vector's offsets.  Then a vector of at most SCL_WIN_THREAD
// elements is folded by one thread (four interleaved folds of the elements
// e = 0, 1, 2, 3 mod 4, combined at the end; in element order below 8
// elements), a longer one by a warp: lane l folds elements l, l + 32, ... in
// order and the lanes' folds combine in a shuffle tree (a strided fold and a
// tree, as in the flat reduce; the operator is taken to be commutative), each
// warp reading the offsets of its next 32 vectors at once.  An empty vector
// yields SCL_IDENTITY.  Folds in the element type.
template <int WT>
__device__ __forceinline__ void scl_reduce_window_run(const scl_T* in, scl_T* out, const scl_u64* seg_off,
                                                      const scl_u64* win_rec, scl_u64 r, scl_T* ts,
                                                      unsigned int spin_limit,
                                                      unsigned int* err SCL_USER_PARAMS) {
  constexpr int B = 256, NW = B / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const scl_T ident = (scl_T)(SCL_IDENTITY);
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_ok;
  const unsigned int bar_s = (unsigned int)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar_s));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const scl_u64 lo = win_rec[4 * r], top = win_rec[4 * r + 1], e0 = win_rec[4 * r + 2];
  const scl_u64 ln = win_rec[4 * r + 3];
  const int len = (int)(ln < (scl_u64)WT ? ln : (scl_u64)WT);  // (more only for bad offsets)
  unsigned int tx;
  const int shift = scl_stage_bulk<scl_T, B>(in + e0, len, ts, bar_s, &tx);
  // this thread's first vector's offsets are read while the copy lands
  scl_u64 sg = lo + threadIdx.x;
  scl_u64 a_n = 0, b_n = 0;
  if (sg < top) {
    a_n = seg_off[sg];
    b_n = seg_off[sg + 1];
  }
  if (threadIdx.x == 0) {
    bool ok = tx == 0u || scl_mbar_wait(bar_s, spin_limit);
    if (!ok) {
      scl_raise(err, SCL_DEV_ERR_TIMEOUT);
      scl_mbar_wait(bar_s, 1u << 21);  // the copy may still land here: stay (bounded) until it has
    }
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  if (!s_ok) return;
  // short vectors (and empty ones): a thread each
  for (; sg < top; sg += B) {
    const scl_u64 a = a_n, b0 = b_n, b = b0 > a ? b0 : a;
    if (sg + B < top) {
      a_n = seg_off[sg + B];
      b_n = seg_off[sg + B + 1];
    }
    if (b == a) {
      out[sg] = ident;
      continue;
    }
    if (b - a > SCL_WIN_THREAD || a < e0 || b > e0 + (scl_u64)len) continue;
    const scl_T* v = ts + (int)(a - e0) + shift;
    const int nv = (int)(b - a);
    scl_T acc;
    if (nv < 8) {
      acc = v[0];
      for (int e = 1; e < nv; ++e) acc = SCL_FUNC(acc, v[e] SCL_OP_ARGS);
    } else {
      // four interleaved folds (elements e = j mod 4), then combined
      scl_T c0 = v[0], c1 = v[1], c2 = v[2], c3 = v[3];
      int e = 4;
      for (; e + 3 < nv; e += 4) {
        c0 = SCL_FUNC(c0, v[e] SCL_OP_ARGS);
        c1 = SCL_FUNC(c1, v[e + 1] SCL_OP_ARGS);
        c2 = SCL_FUNC(c2, v[e + 2] SCL_OP_ARGS);
        c3 = SCL_FUNC(c3, v[e + 3] SCL_OP_ARGS);
      }
      if (e < nv) c0 = SCL_FUNC(c0, v[e] SCL_OP_ARGS);
      if (e + 1 < nv) c1 = SCL_FUNC(c1, v[e + 1] SCL_OP_ARGS);
      if (e + 2 < nv) c2 = SCL_FUNC(c2, v[e + 2] SCL_OP_ARGS);
      acc = SCL_FUNC(SCL_FUNC(c0, c1 SCL_OP_ARGS), SCL_FUNC(c2, c3 SCL_OP_ARGS) SCL_OP_ARGS);
    }
    out[sg] = acc;
  }
  // longer vectors: warp w takes vectors lo + w, lo + w + NW, ... (its next
  // 32 offset pairs read at once, one per lane)
  for (scl_u64 g = lo + warp; g < top; g += (scl_u64)NW * 32) {
    const scl_u64 mine = g + (scl_u64)NW * lane;
    scl_u64 a_l = 0, b_l = 0;
    if (mine < top) {
      a_l = seg_off[mine];
      b_l = seg_off[mine + 1];
    }
    const int cnt = (int)((top - g + NW - 1) / NW < 32 ? (top - g + NW - 1) / NW : 32);
    for (int k = 0; k < cnt; ++k) {
      const scl_u64 sg = g + (scl_u64)NW * k;
      const scl_u64 a = __shfl_sync(0xffffffffu, a_l, k), b0 = __shfl_sync(0xffffffffu, b_l, k);
      const scl_u64 b = b0 > a ? b0 : a;
      if (b - a <= SCL_WIN_THREAD) continue;  // (a thread's, above)
      if (a < e0 || b > e0 + (scl_u64)len) continue;  // (only for offsets changed since the plan)
      const int pa = (int)(a - e0) + shift, pb = (int)(b - e0) + shift;
      scl_T acc = ts[pa + lane];  // (every lane has an element: more than 32 of them)
      for (int p = pa + lane + 32; p < pb; p += 32) acc = SCL_FUNC(acc, ts[p] SCL_OP_ARGS);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const scl_T o = scl_shfl_down(acc, off);
        if (lane + off < 32) acc = SCL_FUNC(acc, o SCL_OP_ARGS);
      }
      if (lane == 0) out[sg] = acc;
    }
  }
}

// Segmented Reduce (no counterpart in the reference): out[s] = the fold of
// segment [seg_off[s], seg_off[s+1]) of the flat vector, for every segment,
// in one launch.  Tiles of R x 256 vectors never span segments (segment s
// owns tiles tile_start[s] .. tile_start[s+1]-1, at least one); each tile
// folds its elements into partials[tile], and the last tile of a segment to
// finish (per-segment ticket, reset afterwards) folds that segment's
// partials.  An empty segment yields SCL_IDENTITY.  Blocks past the last
// tile (the grid is an upper bound) return at once; with MERGED (a segment
// plan numbered the tiles) they fold the segments of at most short_max
// elements instead, one window of them per block (scl_reduce_window_run):
// one launch for a whole segmented Reduce.
template <int R, int MERGED = 0>
__global__ void __launch_bounds__(256)
scl_reduce_seg(const scl_T* in, scl_T* out, const scl_u64* seg_off,
               const unsigned int* tile_start, scl_u64 n_seg, int aligned, scl_C* partials,
               unsigned int* tickets, unsigned int* err, scl_u64 short_max,
               const scl_u64* win_rec, unsigned int spin_limit,
               const unsigned int* tile_seg, unsigned int n_tiles SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  (void)short_max;
  (void)win_rec;
  (void)spin_limit;
  // the tile count, from the host when a plan knows it (~0u: read it)
  const unsigned int nt = n_tiles != ~0u ? n_tiles : tile_start[n_seg];
  if constexpr (MERGED != 0) {
    if (blockIdx.x >= nt) {  // (block-uniform: the whole block takes the window role)
      constexpr int WT = 8 * 256 * scl_vec_width<sizeof(scl_T)>::value;  // 32 KB of elements
      scl_reduce_window_run<WT>(in, out, seg_off, win_rec, blockIdx.x - nt,
                                reinterpret_cast<scl_T*>(scl_dyn_smem), spin_limit, err SCL_EXTRA_ARGS);
      return;
    }
  }
  constexpr int V = scl_vec_width<sizeof(scl_T)>::value;
  constexpr int B = 256;
  constexpr scl_u64 TILE = (scl_u64)R * B * V;
  const unsigned int tile = blockIdx.x;
  __shared__ long long s_seg;
  if (threadIdx.x == 0) {
    long long sg = -1;
    if (tile < nt) {
      if (tile_seg) {  // (a segment plan's table)
        sg = (long long)tile_seg[tile];
      } else {
        scl_u64 lo = 0, hi = n_seg - 1;
        while (lo < hi) {
          const scl_u64 mid = (lo + hi + 1) / 2;
          if (tile_start[mid] <= tile) lo = mid; else hi = mid - 1;
        }
        sg = (long long)lo;
      }
    }
    s_seg = sg;
  }
  __syncthreads();
  if (s_seg < 0) return;
  const scl_u64 sg = (scl_u64)s_seg;
  const unsigned int first = tile_start[sg], count = tile_start[sg + 1] - first;
  const scl_u64 off = seg_off[sg], len = seg_off[sg + 1] > off ? seg_off[sg + 1] - off : 0;
  if (len == 0) {
    if (threadIdx.x == 0) out[sg] = (scl_T)(SCL_IDENTITY);
    return;
  }
  const scl_T* src = in + off;
  const scl_u64 begin = (scl_u64)(tile - first) * TILE;
  const scl_u64 end = begin + TILE < len ? begin + TILE : len;
  bool have = false;
  scl_T acc;
  const bool vec = aligned && ((off * sizeof(scl_T)) % 16 == 0) && end - begin == TILE;
  if (vec) {  // R vectors per thread, loaded 8 at a time
    constexpr int G = R < 8 ? R : 8;
#pragma unroll 1
    for (int r0 = 0; r0 < R; r0 += G) {
      scl_pack<scl_T, V> a[G];
#pragma unroll
      for (int r = 0; r < G; ++r)
        a[r] = scl_load<scl_T, V>(src + begin + ((scl_u64)(r0 + r) * B + threadIdx.x) * V);
#pragma unroll
      for (int r = 0; r < G; ++r)
#pragma unroll
        for (int e = 0; e < V; ++e) {
          acc = have ? SCL_FUNC(acc, a[r].v[e] SCL_OP_ARGS) : a[r].v[e];
          have = true;
        }
    }
  } else {
    // ragged or unaligned: scalar head up to the first 16-byte boundary,
    // 16-byte body, scalar tail
    scl_u64 h = begin, bend = begin;
    if (V > 1 && ((scl_u64)(src + begin)) % sizeof(scl_T) == 0) {
      const scl_u64 mis = ((scl_u64)(src + begin)) & 15u;
      h = begin + (mis ? (16u - mis) / sizeof(scl_T) : 0);
      if (h > end) h = end;
      bend = h + (end - h) / V * V;
    }
    for (scl_u64 i = begin + threadIdx.x; i < h; i += B) {
      acc = have ? SCL_FUNC(acc, src[i] SCL_OP_ARGS) : src[i];
      have = true;
    }
    for (scl_u64 i = h + (scl_u64)threadIdx.x * V; i < bend; i += (scl_u64)B * V) {
      scl_pack<scl_T, V> a = scl_load<scl_T, V>(src + i);
#pragma unroll
      for (int e = 0; e < V; ++e) {
        acc = have ? SCL_FUNC(acc, a.v[e] SCL_OP_ARGS) : a.v[e];
        have = true;
      }
    }
    for (scl_u64 i = (bend > h ? bend : h) + threadIdx.x; i < end; i += B) {
      acc = have ? SCL_FUNC(acc, src[i] SCL_OP_ARGS) : src[i];
      have = true;
    }
  }
  scl_C c;
  if (have) c = (scl_C)acc;
  scl_block_fold(have, c SCL_EXTRA_ARGS);
  if (count == 1) {  // the segment's only tile
    if (threadIdx.x == 0) out[sg] = (scl_T)c;
    return;
  }
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    scl_st_cg(&partials[tile], c);
    __threadfence();
    s_last = (atomicAdd(&tickets[sg], 1u) == count - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  have = false;
  for (unsigned int b = threadIdx.x; b < count; b += B) {
    scl_C v = scl_ld_cg(&partials[first + b]);
    c = have ? (scl_C)SCL_FUNC_C(c, v SCL_OP_ARGS) : v;
    have = true;
  }
  scl_block_fold(have, c SCL_EXTRA_ARGS);
  if (threadIdx.x == 0) {
    out[sg] = (scl_T)c;
    tickets[sg] = 0u;
  }
}

#endif  // SCL_KIND == 9

#if SCL_KIND == 16
// Fused Zip -> Reduce (no counterpart in the reference, which materialises
// the zipped vector): out[0] = fold over i of USR_ZIP(left[i], right[i]),
// in one pass over both inputs with the single-pass reduce above (per-thread
// fold, FP64 carries for float, last-block combine).  Extra arguments: the
// Reduce's first, then the Zip's.
template <int U>
__global__ void scl_zipreduce_k(const SCL_TYPE_0* left, const SCL_TYPE_1* right, scl_T* out,
                                scl_u64 n, int aligned, scl_C* partials, unsigned int* ticket,
                                unsigned int* err SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int V = scl_vec_width<sizeof(SCL_TYPE_0), sizeof(SCL_TYPE_1)>::value;
  const scl_u64 tid = SCL_TID(), nth = SCL_NTH();
  if (n == 0) {
    if (tid == 0) out[0] = (scl_T)(SCL_IDENTITY);
    return;
  }
  const scl_u64 nvec = aligned ? n / V : 0;
  bool have = false;
  scl_T acc;
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
#pragma unroll
        for (int e = 0; e < V; ++e) {
          const scl_T z = USR_ZIP(a[u].v[e], b[u].v[e] SCL_SECOND_ARGS);
          acc = have ? SCL_FUNC(acc, z SCL_OP_ARGS) : z;
          have = true;
        }
      }
    }
  }
  for (scl_u64 i = nvec * V + tid; i < n; i += nth) {
    const scl_T z = USR_ZIP(left[i], right[i] SCL_SECOND_ARGS);
    acc = have ? SCL_FUNC(acc, z SCL_OP_ARGS) : z;
    have = true;
  }
  scl_C c;
  if (have) c = (scl_C)acc;
  scl_block_fold(have, c SCL_EXTRA_ARGS);

  __shared__ int s_last;
  if (threadIdx.x == 0) {
    scl_st_cg(&partials[blockIdx.x], c);  // every block holds at least one element
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  have = false;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    scl_C v = scl_ld_cg(&partials[b]);
    c = have ? (scl_C)SCL_FUNC_C(c, v SCL_OP_ARGS) : v;
    have = true;
  }
  scl_block_fold(have, c SCL_EXTRA_ARGS);
  if (threadIdx.x == 0) {
    out[0] = (scl_T)c;
    *ticket = 0u;
  }
}
#endif  // SCL_KIND == 16
#endif
