// Segmented launches (no counterpart in the reference): thousands of
// vectors of uneven length stored back to back in one flat buffer, segment s
// = [seg_offsets[s], seg_offsets[s+1]), processed by one launch per skeleton.
//
// segments_prepare() is the pre-pass of the segmented Scan and Reduce: it
// copies the caller's offsets into the program workspace clamped to the
// buffer and made non-decreasing (raising a device status bit if they were
// not), and numbers the tiles: segment s owns tiles tile_start[s] ..
// tile_start[s+1]-1, so no tile spans two segments: max(1, ceil(len / tile))
// of them, or, for tiles laid on a grid of vg elements with phase a (the
// scan's 16-byte grid), as many as cover the segment once its start (end,
// for a reverse scan) is rounded onto the grid.  tile_start[n_segments] is
// the tile count.
#include <cstdint>
#include <cstring>

#include "internal.h"

namespace scl {
namespace {

constexpr int kPrepThreads = 1024;

__device__ __forceinline__ uint64_t warp_incl_max(uint64_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o && u > v) v = u;
  }
  return v;
}
__device__ __forceinline__ uint64_t warp_incl_sum(uint64_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}
// Block-wide inclusive scan (max or sum) of one value per thread.
template <bool MAX>
__device__ uint64_t block_incl(uint64_t v, uint64_t* s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = MAX ? warp_incl_max(v) : warp_incl_sum(v);
  if (lane == 31) s_warp[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = s_warp[lane];
    w = MAX ? warp_incl_max(w) : warp_incl_sum(w);
    s_warp[lane] = w;
  }
  __syncthreads();
  if (warp > 0) {
    const uint64_t p = s_warp[warp - 1];
    v = MAX ? (p > v ? p : v) : v + p;
  }
  __syncthreads();
  return v;
}

__global__ void __launch_bounds__(kPrepThreads)
segments_prepare_kernel(const uint64_t* off_in, uint64_t n_seg, uint64_t n_total, uint64_t tile,
                        uint64_t vg, uint64_t a, int reverse, uint64_t* off_out,
                        unsigned int* tile_start, unsigned int* err) {
  __shared__ uint64_t s_warp[32];
  __shared__ uint64_t s_carry;
  __shared__ int s_bad;
  if (threadIdx.x == 0) {
    s_carry = 0;
    s_bad = 0;
  }
  __syncthreads();
  // 1. offsets: clamped to the buffer, running maximum
  for (uint64_t c = 0; c <= n_seg; c += kPrepThreads) {
    const uint64_t s = c + threadIdx.x;
    uint64_t o = 0;
    if (s <= n_seg) {
      o = off_in[s];
      if (o > n_total) {
        o = n_total;
        s_bad = 1;
      }
    }
    uint64_t m = block_incl<true>(o, s_warp);
    const uint64_t carry = s_carry;
    if (carry > m) m = carry;
    if (s <= n_seg) {
      if (m != o) s_bad = 1;  // a decreasing offset
      off_out[s] = m;
    }
    __syncthreads();
    if (threadIdx.x == kPrepThreads - 1) s_carry = m;
    __syncthreads();
  }
  // 2. tiles per segment, exclusive sum
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (uint64_t c = 0; c < n_seg; c += kPrepThreads) {
    const uint64_t s = c + threadIdx.x;
    uint64_t cnt = 0;
    if (s < n_seg) {
      const uint64_t lo = off_out[s], hi = off_out[s + 1];
      // the segment's first tile starts (ends, reverse) on the grid {a + k*vg}
      const uint64_t m = reverse ? (a + vg - hi % vg) % vg : (lo + vg - a) % vg;
      cnt = hi == lo ? 1 : (hi - lo + m + tile - 1) / tile;
    }
    const uint64_t incl = block_incl<false>(cnt, s_warp);
    const uint64_t carry = s_carry;
    if (s < n_seg) tile_start[s] = (unsigned int)(carry + incl - cnt);
    __syncthreads();
    if (threadIdx.x == kPrepThreads - 1) s_carry = carry + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    tile_start[n_seg] = (unsigned int)s_carry;
    if (s_bad && err) atomicOr(err, kDevErrSegments);
  }
}

// gx[i] (+)= g[s] for every element i of segment s (elements outside every
// segment are left alone).  Each block takes a chunk of CH elements; its
// threads walk the offsets forward from the chunk's first segment.  With a
// 16-byte aligned gx, a vector of 16 bytes inside one segment is written with
// one store.
template <typename T>
__global__ void broadcast_segments_kernel(const T* __restrict__ g, T* __restrict__ gx,
                                          const uint64_t* __restrict__ off, uint64_t n_seg,
                                          uint64_t n_total, int acc, int aligned) {
  constexpr int CH = 8192, V = 16 / sizeof(T);
  const uint64_t c0 = (uint64_t)blockIdx.x * CH;
  const uint64_t c1 = c0 + CH < n_total ? c0 + CH : n_total;
  __shared__ uint64_t s_first;
  if (threadIdx.x == 0) {
    // last segment s with off[s] <= c0 (0 if none)
    uint64_t lo = 0, hi = n_seg - 1;
    while (lo < hi) {
      const uint64_t mid = (lo + hi + 1) / 2;
      if (off[mid] <= c0) lo = mid; else hi = mid - 1;
    }
    s_first = lo;
  }
  __syncthreads();
  uint64_t s = s_first;
  auto one = [&](uint64_t i) {
    while (s + 1 < n_seg && i >= off[s + 1]) ++s;
    if (i < off[s] || i >= off[s + 1]) return;
    const T v = g[s];
    gx[i] = acc ? gx[i] + v : v;
  };
  if (!aligned) {
    for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) one(i);
    return;
  }
  for (uint64_t i = c0 + (uint64_t)threadIdx.x * V; i < c1; i += (uint64_t)blockDim.x * V) {
    while (s + 1 < n_seg && i >= off[s + 1]) ++s;
    if (i + V <= c1 && i >= off[s] && i + V <= off[s + 1]) {
      const T v = g[s];
      T r[V];
      if (acc) {
        const uint4 q = *reinterpret_cast<const uint4*>(gx + i);
        memcpy(r, &q, 16);
#pragma unroll
        for (int e = 0; e < V; ++e) r[e] += v;
      } else {
#pragma unroll
        for (int e = 0; e < V; ++e) r[e] = v;
      }
      uint4 q;
      memcpy(&q, r, 16);
      *reinterpret_cast<uint4*>(gx + i) = q;
    } else {
      const uint64_t s_keep = s;
      for (int e = 0; e < V && i + e < c1; ++e) one(i + e);
      s = s_keep;
    }
  }
}

}  // namespace

int segments_prepare(const uint64_t* seg_offsets, uint64_t n_seg, uint64_t n_total, uint64_t tile,
                     uint64_t vg, uint64_t a, int reverse, uint64_t* off_out,
                     unsigned int* tile_start, cudaStream_t stream) {
  segments_prepare_kernel<<<1, kPrepThreads, 0, stream>>>(seg_offsets, n_seg, n_total, tile, vg, a,
                                                          reverse, off_out, tile_start, rt().dev_err);
  SCL_CUDA(cudaGetLastError());
  ++rt().launches;
  return SCL_OK;
}

}  // namespace scl

using namespace scl;

extern "C" int scl_adjoint_broadcast_segments(const void* g, void* gx, const uint64_t* seg_offsets,
                                              uint64_t n_segments, uint64_t n, int dtype,
                                              int accumulate) {
  if (int st = require_init()) return st;
  if (dtype != SCL_DTYPE_F32 && dtype != SCL_DTYPE_F64)
    return fail(SCL_ERR_ARG, "segmented broadcast: dtype must be SCL_DTYPE_F32 or _F64");
  if (n == 0 || n_segments == 0) return SCL_OK;
  if (!g || !gx || !seg_offsets) return fail(SCL_ERR_ARG, "segmented broadcast: null pointer");
  const uint64_t blocks = (n + 8191) / 8192;
  if (blocks > 0x7fffffffull) return fail(SCL_ERR_ARG, "segmented broadcast: vector too large");
  const int acc = accumulate ? 1 : 0;
  const int aligned = (reinterpret_cast<uintptr_t>(gx) & 15u) == 0 ? 1 : 0;
  if (dtype == SCL_DTYPE_F32)
    broadcast_segments_kernel<float><<<(unsigned)blocks, 256, 0, rt().stream>>>(
        (const float*)g, (float*)gx, seg_offsets, n_segments, n, acc, aligned);
  else
    broadcast_segments_kernel<double><<<(unsigned)blocks, 256, 0, rt().stream>>>(
        (const double*)g, (double*)gx, seg_offsets, n_segments, n, acc, aligned);
  SCL_CUDA(cudaGetLastError());
  ++rt().launches;
  return SCL_OK;
}
