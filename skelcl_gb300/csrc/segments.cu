// Segmented launches (no counterpart in the reference): thousands of
// vectors of uneven length stored back to back in one flat buffer, segment s
// = [seg_offsets[s], seg_offsets[s+1]), processed by one launch per skeleton
// and length class.
//
// segments_prepare() is the pre-pass of the segmented Scan and Reduce, three
// small launches: it copies the caller's offsets into the program workspace
// clamped to the buffer (raising a device status bit if an offset lies past
// the buffer or decreases; every consumer reads segment s as
// [off[s], max(off[s], off[s+1])), so no access leaves the buffer), and
// numbers the tiles of the segments longer than `short_max` elements:
// segment s owns tiles tile_start[s] .. tile_start[s+1]-1, so no tile spans
// two segments: ceil(len / tile) of them, or, for tiles laid on a grid of vg
// elements with phase a (the scan's 16-byte grid), as many as cover the
// segment once its start (end, for a reverse scan) is rounded onto the grid.
// Shorter segments, empty ones included, get no tiles: one warp each handles
// them in a separate kernel.  tile_start[n_segments] is the tile count.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

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

constexpr int kSegThreads = 256, kSegPerThread = 8;
constexpr uint64_t kSegPerBlock = (uint64_t)kSegThreads * kSegPerThread;

// Tiles of a segment [lo, hi) (hi >= lo): none when it is short.
__device__ __forceinline__ uint64_t seg_tiles(uint64_t lo, uint64_t hi, uint64_t tile, uint64_t vg,
                                              uint64_t a, int reverse, uint64_t short_max) {
  const uint64_t len = hi - lo;
  if (len <= short_max) return 0;
  // the segment's first tile starts (ends, reverse) on the grid {a + k*vg}
  const uint64_t m = reverse ? (a + vg - hi % vg) % vg : (lo + vg - a) % vg;
  return (len + m + tile - 1) / tile;
}

// 1. clamp the offsets (written to off_out unless it is null), count each
//    segment's tiles, one sum per block
__global__ void __launch_bounds__(kSegThreads)
seg_clamp_count_kernel(const uint64_t* off_in, uint64_t n_seg, uint64_t n_total, uint64_t tile,
                       uint64_t vg, uint64_t a, int reverse, uint64_t short_max, uint64_t* off_out,
                       uint64_t* block_sums, unsigned int* err) {
  __shared__ uint64_t s_warp[32];
  const uint64_t s0 = (uint64_t)blockIdx.x * kSegPerBlock + (uint64_t)threadIdx.x * kSegPerThread;
  uint64_t sum = 0;
  bool bad = false;
#pragma unroll
  for (int k = 0; k < kSegPerThread; ++k) {
    const uint64_t sg = s0 + k;
    if (sg >= n_seg) break;
    const uint64_t rlo = off_in[sg], rhi = off_in[sg + 1];
    bad = bad || rlo > n_total || rhi < rlo;
    const uint64_t lo = rlo < n_total ? rlo : n_total;
    uint64_t hi = rhi < n_total ? rhi : n_total;
    if (hi < lo) hi = lo;
    if (off_out) off_out[sg] = lo;
    if (sg + 1 == n_seg) {
      if (off_out) off_out[n_seg] = rhi < n_total ? rhi : n_total;
      bad = bad || rhi > n_total;
    }
    sum += seg_tiles(lo, hi, tile, vg, a, reverse, short_max);
  }
  if (bad && err) atomicOr(err, kDevErrSegments);
  const uint64_t incl = block_incl<false>(sum, s_warp);
  if (threadIdx.x == kSegThreads - 1) block_sums[blockIdx.x] = incl;
}

// 2. exclusive sum over the blocks' sums (one block); the total at [nb]
__global__ void __launch_bounds__(kPrepThreads)
seg_scan_sums_kernel(uint64_t* block_sums, uint64_t nb) {
  __shared__ uint64_t s_warp[32];
  __shared__ uint64_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (uint64_t c = 0; c < nb; c += kPrepThreads) {
    const uint64_t b = c + threadIdx.x;
    const uint64_t v = b < nb ? block_sums[b] : 0;
    const uint64_t incl = block_incl<false>(v, s_warp);
    const uint64_t carry = s_carry;
    if (b < nb) block_sums[b] = carry + incl - v;
    __syncthreads();
    if (threadIdx.x == kPrepThreads - 1) s_carry = carry + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[nb] = s_carry;
}

// 3. every segment's first tile
__global__ void __launch_bounds__(kSegThreads)
seg_tile_start_kernel(const uint64_t* off, uint64_t n_seg, uint64_t tile, uint64_t vg, uint64_t a,
                      int reverse, uint64_t short_max, const uint64_t* block_sums, uint64_t nb,
                      unsigned int* tile_start) {
  __shared__ uint64_t s_warp[32];
  const uint64_t s0 = (uint64_t)blockIdx.x * kSegPerBlock + (uint64_t)threadIdx.x * kSegPerThread;
  uint64_t cnt[kSegPerThread], sum = 0;
#pragma unroll
  for (int k = 0; k < kSegPerThread; ++k) {
    const uint64_t sg = s0 + k;
    cnt[k] = 0;
    if (sg < n_seg) {
      const uint64_t lo = off[sg];
      uint64_t hi = off[sg + 1];
      if (hi < lo) hi = lo;
      cnt[k] = seg_tiles(lo, hi, tile, vg, a, reverse, short_max);
    }
    sum += cnt[k];
  }
  const uint64_t incl = block_incl<false>(sum, s_warp);
  uint64_t start = block_sums[blockIdx.x] + incl - sum;
#pragma unroll
  for (int k = 0; k < kSegPerThread; ++k) {
    const uint64_t sg = s0 + k;
    if (sg < n_seg) tile_start[sg] = (unsigned int)start;
    start += cnt[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) tile_start[n_seg] = (unsigned int)block_sums[nb];
}

// gx[i] (+)= g[s] for every element i of segment s (elements outside every
// segment are left alone).  Each warp takes a chunk of CH elements: it finds
// the last segment starting at or before the chunk (a search of the warp, 32
// probes per round), then walks the segments that start before the chunk's
// end, the offsets and values of 32 of them read at once, and writes each
// one's part of the chunk with lane-strided stores (16 bytes at a time when
// gx is 16-byte aligned, single elements at the part's ragged ends).
template <typename T>
__global__ void __launch_bounds__(256)
broadcast_segments_kernel(const T* __restrict__ g, T* __restrict__ gx, const uint64_t* __restrict__ off,
                          uint64_t n_seg, uint64_t n_total, int acc, int aligned) {
  constexpr int CH = 1024, V = 16 / sizeof(T);
  const int lane = threadIdx.x & 31;
  const uint64_t c0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * CH;
  if (c0 >= n_total) return;  // (warp-uniform)
  const uint64_t c1 = c0 + CH < n_total ? c0 + CH : n_total;
  // last segment with off[s] <= c0 (0 if none): each round the lanes probe 32
  // offsets spread over [lo, hi] and the count at or below c0 narrows it (by
  // 32 for increasing offsets; decreasing ones still end the search)
  uint64_t lo = 0, hi = n_seg - 1;
  while (lo < hi) {  // (warp-uniform)
    const uint64_t span = hi - lo;
    const uint64_t p = lo + 1 + span * (uint64_t)lane / 32;
    const int below = __popc(__ballot_sync(0xffffffffu, off[p] <= c0));
    if (below == 0) {
      hi = lo;
    } else {
      const uint64_t p_last = lo + 1 + span * (uint64_t)(below - 1) / 32;
      hi = below < 32 ? lo + span * (uint64_t)below / 32 : hi;
      lo = p_last;
    }
  }
  // this warp's part [r0, r1) of one segment, value v, as offsets from c0
  // (a multiple of CH, so offsets and indices share their 16-byte phase)
  T* const base = gx + c0;
  auto one = [&](int r, T v) { base[r] = acc ? base[r] + v : v; };
  auto put = [&](int r0, int r1, T v) {
    if (!aligned) {
      for (int r = r0 + lane; r < r1; r += 32) one(r, v);
      return;
    }
    const int h0 = (r0 + V - 1) & ~(V - 1);
    const int h = h0 < r1 ? h0 : r1;                        // end of the ragged head
    const int t0 = r1 & ~(V - 1), t = t0 > h ? t0 : h;      // start of the ragged tail
    if (r0 + lane < h) one(r0 + lane, v);
    for (int q = h + lane * V; q < t; q += 32 * V) {
      T r[V];
      if (acc) {
        const uint4 w = *reinterpret_cast<const uint4*>(base + q);
        memcpy(r, &w, 16);
#pragma unroll
        for (int e = 0; e < V; ++e) r[e] += v;
      } else {
#pragma unroll
        for (int e = 0; e < V; ++e) r[e] = v;
      }
      uint4 w;
      memcpy(&w, r, 16);
      *reinterpret_cast<uint4*>(base + q) = w;
    }
    if (t + lane < r1) one(t + lane, v);
  };
  for (uint64_t sb = lo; sb < n_seg; sb += 32) {
    const uint64_t my = sb + lane;
    uint64_t a_l = n_total, b_l = n_total;
    T v_l = T(0);
    if (my < n_seg) {
      a_l = off[my];
      b_l = off[my + 1];
      v_l = g[my];
    }
    const int cnt = n_seg - sb < 32 ? (int)(n_seg - sb) : 32;
    bool past = false;
    for (int k = 0; k < cnt; ++k) {
      const uint64_t a = __shfl_sync(0xffffffffu, a_l, k), b0 = __shfl_sync(0xffffffffu, b_l, k);
      const T v = __shfl_sync(0xffffffffu, v_l, k);
      if (a >= c1) {  // this and (for increasing offsets) every later segment start past the chunk
        past = true;
        break;
      }
      const uint64_t b = b0 > a ? b0 : a;
      const uint64_t i0 = a > c0 ? a : c0, i1 = b < c1 ? b : c1;
      if (i0 < i1) put((int)(i0 - c0), (int)(i1 - c0), v);
    }
    if (past) break;
  }
}

// tile_seg[t] = s for every tile t of segment s (tiles tile_start[s] ..
// tile_start[s+1]-1), one thread per segment.
__global__ void __launch_bounds__(256) seg_tile_owner_kernel(const unsigned int* __restrict__ tile_start,
                                                             uint64_t n_seg, unsigned int* __restrict__ tile_seg) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_seg;
       s += (uint64_t)gridDim.x * blockDim.x)
    for (unsigned int t = tile_start[s]; t < tile_start[s + 1]; ++t) tile_seg[t] = (unsigned int)s;
}

}  // namespace

size_t segments_prepare_scratch(uint64_t n_seg) {
  return ((n_seg + kSegPerBlock - 1) / kSegPerBlock + 1) * sizeof(uint64_t);
}

int segments_prepare(const uint64_t* seg_offsets, uint64_t n_seg, uint64_t n_total, uint64_t tile,
                     uint64_t vg, uint64_t a, int reverse, uint64_t short_max, uint64_t* off_out,
                     unsigned int* tile_start, uint64_t* scratch, cudaStream_t stream) {
  const uint64_t nb = (n_seg + kSegPerBlock - 1) / kSegPerBlock;
  if (nb == 0) return SCL_OK;
  if (nb > 0x7fffffffull) return fail(SCL_ERR_ARG, "too many segments");
  // off_out == seg_offsets: the offsets are already clamped; number the
  // tiles without writing them again
  seg_clamp_count_kernel<<<(unsigned)nb, kSegThreads, 0, stream>>>(
      seg_offsets, n_seg, n_total, tile, vg, a, reverse, short_max,
      off_out == seg_offsets ? nullptr : off_out, scratch, rt().dev_err);
  seg_scan_sums_kernel<<<1, kPrepThreads, 0, stream>>>(scratch, nb);
  seg_tile_start_kernel<<<(unsigned)nb, kSegThreads, 0, stream>>>(off_out, n_seg, tile, vg, a, reverse,
                                                                  short_max, scratch, nb, tile_start);
  SCL_CUDA(cudaGetLastError());
  rt().launches += 3;
  return SCL_OK;
}

// ---- segment plans ------------------------------------------------------------
namespace {
std::mutex g_plan_mu;
std::map<uint32_t, std::unique_ptr<SegPlan>> g_plans;
uint32_t g_next_plan = 1;

void free_plan(SegPlan* p) {
  if (!rt().initialized) return;
  cudaStreamSynchronize(rt().stream);
  cudaFree(p->off);
  cudaFree(p->tickets);
  cudaFree(p->scratch);
  for (auto& c : p->cfgs) {
    cudaFree(c.tile_start);
    cudaFree(c.win_rec);
    cudaFree(c.tile_seg);
  }
}
}  // namespace

// Window records of the short segments: consecutive segments starting in the
// same window of short_max elements form one record {first segment, end
// segment, first element, elements}; a last segment longer than short_max
// belongs to the tiles and is left out (its start ends the record's
// elements).  All but the last segment of a record end inside its window, so
// a record spans at most 2 * short_max elements.  Records whose segments are
// all empty stay (the Reduce writes their identities); windows that own no
// segment get none.  `off` holds n_seg + 1 clamped offsets.
void segplan_window_records(const uint64_t* off, uint64_t n_seg, uint64_t short_max,
                            std::vector<uint64_t>* rec) {
  rec->clear();
  for (uint64_t sg = 0; sg < n_seg;) {
    const uint64_t w = off[sg] / short_max, w0 = w * short_max, w1 = w0 + short_max;
    uint64_t hi = sg + 1;
    while (hi < n_seg && off[hi] >= w0 && off[hi] < w1) ++hi;
    const uint64_t la = off[hi - 1], lb = std::max(la, off[hi]);
    const uint64_t top = lb - la > short_max ? hi - 1 : hi;
    if (top > sg) {
      const uint64_t e0 = off[sg];
      uint64_t e1 = top == hi ? lb : off[top];
      if (e1 < e0) e1 = e0;
      rec->insert(rec->end(), {sg, top, e0, e1 - e0});
    }
    sg = hi;
  }
}

SegPlan* segplan_find(uint32_t id) {
  std::lock_guard<std::mutex> g(g_plan_mu);
  auto it = g_plans.find(id);
  return it == g_plans.end() ? nullptr : it->second.get();
}

int segplan_config(SegPlan* p, uint64_t tile, uint64_t vg, uint64_t a, int reverse, uint64_t short_max,
                   const SegPlanCfg** out) {
  for (auto& c : p->cfgs)
    if (c.tile == tile && c.vg == vg && c.a == a && c.reverse == reverse && c.short_max == short_max) {
      *out = &c;
      return SCL_OK;
    }
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  SCL_CUDA(cudaStreamIsCapturing(rt().stream, &capture));
  if (capture != cudaStreamCaptureStatusNone)
    return fail(SCL_ERR_ARG,
                "segment plan: this tile shape is first used inside a stream capture; make the call "
                "once before capturing (building its tile numbering reads the tile count back)");
  SegPlanCfg c;
  c.tile = tile;
  c.vg = vg;
  c.a = a;
  c.reverse = reverse;
  c.short_max = short_max;
  rt().device_allocs++;
  SCL_CUDA(cudaMalloc(&c.tile_start, (p->n_seg + 1) * sizeof(unsigned int)));
  if (int st = segments_prepare(p->off, p->n_seg, p->n_total, tile, vg, a, reverse, short_max, p->off,
                                c.tile_start, p->scratch, rt().stream)) {
    cudaFree(c.tile_start);
    return st;
  }
  // the window records of the short segments (on the host, once)
  std::vector<uint64_t> off(p->n_seg + 1);
  SCL_CUDA(cudaMemcpyAsync(off.data(), p->off, off.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                           rt().stream));
  SCL_CUDA(cudaStreamSynchronize(rt().stream));
  std::vector<uint64_t> rec;
  segplan_window_records(off.data(), p->n_seg, short_max, &rec);
  c.n_rec = rec.size() / 4;
  if (c.n_rec) {
    rt().device_allocs++;
    cudaError_t e = cudaMalloc(&c.win_rec, rec.size() * sizeof(uint64_t));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c.win_rec, rec.data(), rec.size() * sizeof(uint64_t), cudaMemcpyHostToDevice,
                          rt().stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(rt().stream);
    if (e != cudaSuccess) {
      cudaFree(c.tile_start);
      cudaFree(c.win_rec);
      return cuda_fail(e, "segment plan: window records");
    }
  }
  unsigned int tiles = 0;
  SCL_CUDA(cudaMemcpyAsync(&tiles, c.tile_start + p->n_seg, sizeof(tiles), cudaMemcpyDeviceToHost,
                           rt().stream));
  SCL_CUDA(cudaStreamSynchronize(rt().stream));
  c.tiles = tiles;
  // each tile's segment, so that a tile finds its segment with one load
  if (tiles) {
    rt().device_allocs++;
    cudaError_t e = cudaMalloc(&c.tile_seg, (size_t)tiles * sizeof(unsigned int));
    if (e == cudaSuccess) {
      const uint64_t nb = std::min<uint64_t>((p->n_seg + 255) / 256, 65535);
      seg_tile_owner_kernel<<<(unsigned)nb, 256, 0, rt().stream>>>(c.tile_start, p->n_seg, c.tile_seg);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
      cudaFree(c.tile_start);
      cudaFree(c.win_rec);
      cudaFree(c.tile_seg);
      return cuda_fail(e, "segment plan: tile owners");
    }
  }
  p->cfgs.push_back(c);
  *out = &p->cfgs.back();
  return SCL_OK;
}

}  // namespace scl

using namespace scl;

extern "C" int scl_segplan_create(const uint64_t* seg_offsets, uint64_t n_segments, uint64_t n,
                                  uint32_t* plan) {
  if (int st = require_init()) return st;
  if (!plan) return fail(SCL_ERR_ARG, "scl_segplan_create: null plan");
  *plan = 0;
  if (!seg_offsets || n_segments == 0) return fail(SCL_ERR_ARG, "scl_segplan_create: no segments");
  const uint64_t nb = (n_segments + kSegPerBlock - 1) / kSegPerBlock;
  if (nb > 0x7fffffffull) return fail(SCL_ERR_ARG, "scl_segplan_create: too many segments");
  std::unique_ptr<SegPlan> p(new SegPlan);
  p->n_seg = n_segments;
  p->n_total = n;
  rt().device_allocs += 3;
  cudaError_t e = cudaMalloc(&p->off, (n_segments + 1) * sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMalloc(&p->tickets, n_segments * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&p->scratch, segments_prepare_scratch(n_segments));
  if (e == cudaSuccess) e = cudaMemsetAsync(p->tickets, 0, n_segments * sizeof(unsigned int), rt().stream);
  if (e != cudaSuccess) {
    free_plan(p.get());
    cudaGetLastError();
    return fail(SCL_ERR_OOM, "scl_segplan_create: device memory for the plan");
  }
  // the clamped copy of the offsets (no tiles counted yet)
  seg_clamp_count_kernel<<<(unsigned)nb, kSegThreads, 0, rt().stream>>>(
      seg_offsets, n_segments, n, ~0ull, 1, 0, 0, ~0ull, p->off, p->scratch, rt().dev_err);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    free_plan(p.get());
    return cuda_fail(e, "segment plan: clamp kernel");
  }
  ++rt().launches;
  std::lock_guard<std::mutex> g(g_plan_mu);
  p->id = g_next_plan++;
  if (g_next_plan == 0) g_next_plan = 1;
  *plan = p->id;
  g_plans[p->id] = std::move(p);
  return SCL_OK;
}

extern "C" int scl_segplan_release(uint32_t plan) {
  std::unique_ptr<SegPlan> p;
  {
    std::lock_guard<std::mutex> g(g_plan_mu);
    auto it = g_plans.find(plan);
    if (it == g_plans.end()) return plan == 0 ? SCL_OK : fail(SCL_ERR_ARG, "scl_segplan_release: no such plan");
    p = std::move(it->second);
    g_plans.erase(it);
  }
  free_plan(p.get());
  return SCL_OK;
}

extern "C" int scl_adjoint_broadcast_segments(const void* g, void* gx, const uint64_t* seg_offsets,
                                              uint64_t n_segments, uint64_t n, int dtype,
                                              int accumulate) {
  if (int st = require_init()) return st;
  if (dtype != SCL_DTYPE_F32 && dtype != SCL_DTYPE_F64)
    return fail(SCL_ERR_ARG, "segmented broadcast: dtype must be SCL_DTYPE_F32 or _F64");
  if (n == 0 || n_segments == 0) return SCL_OK;
  if (!g || !gx || !seg_offsets) return fail(SCL_ERR_ARG, "segmented broadcast: null pointer");
  const uint64_t blocks = (n + 8191) / 8192;  // 8 warps of 1024 elements each
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

extern "C" int scl_debug_window_records(const uint64_t* offsets, uint64_t n_segments, uint64_t short_max,
                                        uint64_t* records, uint64_t capacity, uint64_t* count) {
  if (!offsets || !count) return fail(SCL_ERR_ARG, "scl_debug_window_records: null argument");
  if (short_max == 0) return fail(SCL_ERR_ARG, "scl_debug_window_records: short_max must be positive");
  std::vector<uint64_t> rec;
  segplan_window_records(offsets, n_segments, short_max, &rec);
  *count = rec.size() / 4;
  if (records) {
    if (capacity < *count) return fail(SCL_ERR_ARG, "scl_debug_window_records: capacity too small");
    std::memcpy(records, rec.data(), rec.size() * sizeof(uint64_t));
  }
  return SCL_OK;
}
