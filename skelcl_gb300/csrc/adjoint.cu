// Adjoint building blocks that need no user code (no counterpart in the
// reference): the broadcast that is the adjoint of Reduce(+), gradient
// accumulation, the edge part of the transposed stencil for NEAREST padding,
// and the transpose the CUDA-core AllPairs uses for transposed operands.
#include <cstdint>
#include <cstring>

#include "internal.h"

namespace scl {
namespace {

constexpr int kBlock = 256;

int grid_for(uint64_t units) {
  const int sm = rt().sm_count > 0 ? rt().sm_count : 148;
  uint64_t g = (units + kBlock - 1) / kBlock;
  const uint64_t cap = (uint64_t)sm * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// gx[i] = g (+ gx[i]); 16-byte accesses when gx is aligned
template <typename T>
__global__ void broadcast_kernel(const T* __restrict__ g, T* __restrict__ gx, uint64_t n, int acc,
                                 int aligned) {
  constexpr int V = 16 / sizeof(T);
  const T v = *g;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nvec = aligned ? n / V : 0;
  for (uint64_t k = tid; k < nvec; k += nth) {
    T r[V];
    if (acc) {
      const uint4 q = reinterpret_cast<const uint4*>(gx)[k];
      memcpy(r, &q, 16);
#pragma unroll
      for (int e = 0; e < V; ++e) r[e] += v;
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) r[e] = v;
    }
    uint4 q;
    memcpy(&q, r, 16);
    reinterpret_cast<uint4*>(gx)[k] = q;
  }
  for (uint64_t i = nvec * V + tid; i < n; i += nth) gx[i] = acc ? gx[i] + v : v;
}

// dst[i] += src[i]
template <typename T>
__global__ void accumulate_kernel(T* __restrict__ dst, const T* __restrict__ src, uint64_t n,
                                  int aligned) {
  constexpr int V = 16 / sizeof(T);
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nvec = aligned ? n / V : 0;
  for (uint64_t k = tid; k < nvec; k += nth) {
    const uint4 qa = reinterpret_cast<const uint4*>(dst)[k];
    const uint4 qb = reinterpret_cast<const uint4*>(src)[k];
    T a[V], b[V];
    memcpy(a, &qa, 16);
    memcpy(b, &qb, 16);
#pragma unroll
    for (int e = 0; e < V; ++e) a[e] += b[e];
    uint4 q;
    memcpy(&q, a, 16);
    reinterpret_cast<uint4*>(dst)[k] = q;
  }
  for (uint64_t i = nvec * V + tid; i < n; i += nth) dst[i] += src[i];
}

// Edge part of the NEAREST transposed stencil.  The forward read
// in[clamp(y+dy)][clamp(x+dx)]; every read position p' outside the matrix
// was served by the edge pixel clamp(p').  Its adjoint therefore adds, to each
// edge pixel p, the zero-padded transposed stencil of g evaluated at every
// outside position p' with clamp(p') = p.  One warp per edge pixel: the lanes
// share the taps, loop over the outside positions, and add their sums with
// shuffles.
__global__ void stencil_edges_kernel(const float* __restrict__ g, const float* __restrict__ w,
                                     float* __restrict__ gin, int64_t rows, int64_t cols, int R,
                                     int64_t n_edge) {
  const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= n_edge) return;  // whole warps leave together (blockDim is a multiple of 32)
  int64_t y, x;
  // top row, bottom row (rows > 1), left column, right column (cols > 1),
  // the columns without their first and last pixels
  const int64_t inner = rows > 2 ? rows - 2 : 0;
  if (e < cols) {
    y = 0; x = e;
  } else if (rows > 1 && e < 2 * cols) {
    y = rows - 1; x = e - cols;
  } else {
    const int64_t base = rows > 1 ? 2 * cols : cols;
    const int64_t k = e - base;
    if (k < inner) { y = 1 + k; x = 0; }
    else { y = 1 + (k - inner); x = cols - 1; }
  }
  const int64_t y0 = (y == 0) ? -R : y, y1 = (y == rows - 1) ? rows - 1 + R : y;
  const int64_t x0 = (x == 0) ? -R : x, x1 = (x == cols - 1) ? cols - 1 + R : x;
  const int W = 2 * R + 1;
  float acc = 0.0f;
  // each lane takes every 32nd tap, and for it every outside position
  for (int tap = lane; tap < W * W; tap += 32) {
    const int dy = tap / W - R, dx = tap % W - R;
    const float wt = w[tap];
    for (int64_t py = y0; py <= y1; ++py) {
      const int64_t qy = py + dy;
      if (qy < 0 || qy >= rows) continue;
      for (int64_t px = x0; px <= x1; ++px) {
        if (py == y && px == x) continue;  // inside: already in gin
        const int64_t qx = px + dx;
        if (qx < 0 || qx >= cols) continue;
        acc += wt * g[qy * cols + qx];
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) gin[y * cols + x] += acc;
}

template <typename T>
__global__ void transpose_kernel(const T* __restrict__ src, T* __restrict__ dst, uint64_t rows,
                                 uint64_t cols) {
  __shared__ T tile[32][33];
  const uint64_t r0 = (uint64_t)blockIdx.y * 32, c0 = (uint64_t)blockIdx.x * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const uint64_t r = r0 + j, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = src[r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const uint64_t c = c0 + j, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[c * rows + r] = tile[threadIdx.x][j];
  }
}

int dtype_size(int dtype) { return dtype == SCL_DTYPE_F32 ? 4 : (dtype == SCL_DTYPE_F64 ? 8 : 0); }

}  // namespace

int transpose_launch(const void* src, void* dst, uint64_t rows, uint64_t cols, size_t elem,
                     cudaStream_t stream) {
  const uint64_t gx = (cols + 31) / 32, gy = (rows + 31) / 32;
  if (gx > 0x7fffffffull || gy > 65535) return fail(SCL_ERR_ARG, "transpose: matrix too large");
  dim3 grid((unsigned)gx, (unsigned)gy), block(32, 8);
  if (elem == 4)
    transpose_kernel<uint32_t><<<grid, block, 0, stream>>>((const uint32_t*)src, (uint32_t*)dst, rows, cols);
  else if (elem == 8)
    transpose_kernel<uint64_t><<<grid, block, 0, stream>>>((const uint64_t*)src, (uint64_t*)dst, rows, cols);
  else
    return fail(SCL_ERR_UNSUPPORTED, "transpose: elements of 4 or 8 bytes only");
  SCL_CUDA(cudaGetLastError());
  ++rt().launches;
  return SCL_OK;
}

}  // namespace scl

using namespace scl;

extern "C" int scl_adjoint_broadcast(const void* g, void* gx, uint64_t n, int dtype, int accumulate) {
  if (int st = require_init()) return st;
  if (!dtype_size(dtype)) return fail(SCL_ERR_ARG, "broadcast: dtype must be SCL_DTYPE_F32 or _F64");
  if (n == 0) return SCL_OK;
  if (!g || !gx) return fail(SCL_ERR_ARG, "broadcast: null buffer");
  const int aligned = aligned16(gx) ? 1 : 0;
  const int V = 16 / dtype_size(dtype);
  const int grid = grid_for(aligned ? (n + V - 1) / V : n);
  const int acc = accumulate ? 1 : 0;
  if (dtype == SCL_DTYPE_F32)
    broadcast_kernel<float><<<grid, kBlock, 0, rt().stream>>>((const float*)g, (float*)gx, n, acc, aligned);
  else
    broadcast_kernel<double><<<grid, kBlock, 0, rt().stream>>>((const double*)g, (double*)gx, n, acc, aligned);
  SCL_CUDA(cudaGetLastError());
  ++rt().launches;
  return SCL_OK;
}

extern "C" int scl_adjoint_accumulate(void* dst, const void* src, uint64_t n, int dtype) {
  if (int st = require_init()) return st;
  if (!dtype_size(dtype)) return fail(SCL_ERR_ARG, "accumulate: dtype must be SCL_DTYPE_F32 or _F64");
  if (n == 0) return SCL_OK;
  if (!dst || !src) return fail(SCL_ERR_ARG, "accumulate: null buffer");
  const int aligned = (aligned16(dst) && aligned16(src)) ? 1 : 0;
  const int V = 16 / dtype_size(dtype);
  const int grid = grid_for(aligned ? (n + V - 1) / V : n);
  if (dtype == SCL_DTYPE_F32)
    accumulate_kernel<float><<<grid, kBlock, 0, rt().stream>>>((float*)dst, (const float*)src, n, aligned);
  else
    accumulate_kernel<double><<<grid, kBlock, 0, rt().stream>>>((double*)dst, (const double*)src, n, aligned);
  SCL_CUDA(cudaGetLastError());
  ++rt().launches;
  return SCL_OK;
}

extern "C" int scl_mapoverlap_adjoint_edges(const float* g, const float* w, float* gin, uint64_t rows,
                                            uint64_t cols, int R) {
  if (int st = require_init()) return st;
  if (rows == 0 || cols == 0) return SCL_OK;
  if (!g || !w || !gin) return fail(SCL_ERR_ARG, "stencil adjoint: null buffer");
  if (R < 0 || R > 64) return fail(SCL_ERR_ARG, "stencil adjoint: overlap range must be 0..64");
  if (rows > (1ull << 40) || cols > (1ull << 40)) return fail(SCL_ERR_ARG, "stencil adjoint: matrix too large");
  if (R == 0) return SCL_OK;
  const int64_t r = (int64_t)rows, c = (int64_t)cols;
  const int64_t n_edge = c + (r > 1 ? c : 0) + (r > 2 ? r - 2 : 0) * (c > 1 ? 2 : 1);
  const int64_t grid = (n_edge + 7) / 8;  // 8 warps (edge pixels) per block
  if (grid > 0x7fffffffll) return fail(SCL_ERR_ARG, "stencil adjoint: matrix too large");
  stencil_edges_kernel<<<(unsigned)grid, 256, 0, rt().stream>>>(g, w, gin, r, c, R, n_edge);
  SCL_CUDA(cudaGetLastError());
  ++rt().launches;
  return SCL_OK;
}
