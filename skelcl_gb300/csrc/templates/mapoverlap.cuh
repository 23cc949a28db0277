// ---------------------------------------------------------------------------
// MapOverlap for sm_103a: 2D stencil over a row-major matrix.
//
// Reference: SCL_MAPOVERLAP (include/SkelCL/detail/MapOverlapKernel.cl:59-148)
// with the OL distribution's host-built padding rows
// (include/SkelCL/detail/OLDistributionDef.h:264-343).  Net semantics:
//   out[y][x] = f(view), getData(view, dx, dy) = in'[y+dy][x+dx]
// where in' is `in` extended by R on every side with
//   NEAREST: in[clamp(y+dy)][clamp(x+dx)]  (corners included)
//   NEUTRAL: the neutral element.
// dx runs along columns, dy along rows (test/MapOverlapTests.cpp:187-216).
// Here both axes are padded in-kernel; no padded copy of the matrix exists.
//
// Shape: a block of 32 x 8 threads owns a 32-column x (8*PY)-row output tile
// and stages the (8*PY+2R) x SCL_WIN_W input window in shared memory, either
// with one TMA 2D tile load (OOB elements filled with zero, then patched for
// NEAREST / non-zero NEUTRAL) or with cooperative coalesced loads.  Each
// thread computes PY vertically adjacent outputs; with the user loops
// unrolled, taps shared between those outputs and the user's weight loads
// are read once per thread instead of once per output.
// Generated names: SCL_OVERLAP_RANGE, SCL_PADDING (0 neutral, 1 nearest),
// SCL_NEUTRAL, SCL_NEUTRAL_IS_ZERO.
// ---------------------------------------------------------------------------
#if SCL_KIND == 11

__device__ __forceinline__ scl_u64 scl_clampi(long long v, long long hi) {
  return (scl_u64)(v < 0 ? 0 : (v > hi ? hi : v));
}

// Fill the positions of the window that lie outside the matrix.
template <int WIN_H>
__device__ __forceinline__ void scl_patch_border(SCL_TYPE_0* win, long long x_org, long long y_org,
                                                 scl_u64 rows, scl_u64 cols) {
  const int nthreads = blockDim.x * blockDim.y;
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  for (int k = t; k < WIN_H * SCL_WIN_W; k += nthreads) {
    const int ly = k / SCL_WIN_W, lx = k % SCL_WIN_W;
    const long long gy = y_org + ly, gx = x_org + lx;
    const bool inside = gy >= 0 && gy < (long long)rows && gx >= 0 && gx < (long long)cols;
    if (inside) continue;
#if SCL_PADDING == 1
    const long long cy = (long long)scl_clampi(gy, (long long)rows - 1);
    const long long cx = (long long)scl_clampi(gx, (long long)cols - 1);
    // the clamped position lies inside both the matrix and the window
    win[k] = win[(cy - y_org) * SCL_WIN_W + (cx - x_org)];
#else
    win[k] = (SCL_TYPE_0)(SCL_NEUTRAL);
#endif
  }
}

// Each thread computes PY vertically adjacent outputs in each of SCL_PX
// adjacent columns: with the user loops unrolled, the taps those outputs
// share are read once.
template <int PY>
__device__ __forceinline__ void scl_compute_tile(const SCL_TYPE_0* win, SCL_TYPE_1* out,
                                                 scl_u64 rows, scl_u64 cols, scl_u64 x0,
                                                 scl_u64 y0 SCL_USER_PARAMS) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  SCL_TYPE_1 res[PY][SCL_PX];
#pragma unroll
  for (int p = 0; p < PY; ++p) {
    const int ly = ty * PY + p;
#pragma unroll
    for (int c = 0; c < SCL_PX; ++c) {
      const int lx = tx * SCL_PX + c;
      input_matrix_t m;
      m.data = win + (ly + SCL_R) * SCL_WIN_W + SCL_XLEAD + lx;
      m.local_row = ly;
      m.local_column = lx;
      res[p][c] = USR_FUNC(m SCL_EXTRA_ARGS);
    }
  }
#pragma unroll
  for (int p = 0; p < PY; ++p) {
    const scl_u64 y = y0 + ty * PY + p;
#pragma unroll
    for (int c = 0; c < SCL_PX; ++c) {
      const scl_u64 x = x0 + (scl_u64)tx * SCL_PX + c;
      if (y < rows && x < cols) out[y * cols + x] = res[p][c];
    }
  }
}

// Cooperative-load variant: any shape, any alignment.
template <int PY>
__global__ void __launch_bounds__(256)
scl_mapoverlap_ldst(const SCL_TYPE_0* in, SCL_TYPE_1* out, scl_u64 rows, scl_u64 cols
                    SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int TH = 8 * PY, WIN_H = TH + 2 * SCL_R;
  SCL_TYPE_0* win = reinterpret_cast<SCL_TYPE_0*>(scl_dyn_smem);  // WIN_H x SCL_WIN_W
  const scl_u64 x0 = (scl_u64)blockIdx.x * SCL_TW, y0 = (scl_u64)blockIdx.y * TH;
  const long long x_org = (long long)x0 - SCL_XLEAD, y_org = (long long)y0 - SCL_R;
  const int nthreads = blockDim.x * blockDim.y;
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  for (int k = t; k < WIN_H * SCL_WIN_W; k += nthreads) {
    const int ly = k / SCL_WIN_W, lx = k % SCL_WIN_W;
    const long long gy = y_org + ly, gx = x_org + lx;
    SCL_TYPE_0 v;
    if (gy >= 0 && gy < (long long)rows && gx >= 0 && gx < (long long)cols) {
      v = in[(scl_u64)gy * cols + (scl_u64)gx];
    } else {
#if SCL_PADDING == 1
      v = in[scl_clampi(gy, (long long)rows - 1) * cols + scl_clampi(gx, (long long)cols - 1)];
#else
      v = (SCL_TYPE_0)(SCL_NEUTRAL);
#endif
    }
    win[k] = v;
  }
  __syncthreads();
  scl_compute_tile<PY>(win, out, rows, cols, x0, y0 SCL_EXTRA_ARGS);
}

// TMA variant: one elected thread loads the whole window with
// cp.async.bulk.tensor.2d (zero fill outside the matrix); border tiles are
// patched afterwards.  Requires cols * sizeof(T) % 16 == 0 (tensor-map stride
// rule) and a 16-byte aligned base; the host checks both.
struct __align__(64) scl_tmap { unsigned long long v[16]; };

template <int PY>
__global__ void __launch_bounds__(256)
scl_mapoverlap_tma(const __grid_constant__ scl_tmap tmap, SCL_TYPE_1* out, scl_u64 rows,
                   scl_u64 cols, unsigned int spin_limit, unsigned int* err SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int TH = 8 * PY, WIN_H = TH + 2 * SCL_R;
  SCL_TYPE_0* win = reinterpret_cast<SCL_TYPE_0*>(scl_dyn_smem);  // WIN_H x SCL_WIN_W
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_ok;
  const scl_u64 x0 = (scl_u64)blockIdx.x * SCL_TW, y0 = (scl_u64)blockIdx.y * TH;
  const long long x_org = (long long)x0 - SCL_XLEAD, y_org = (long long)y0 - SCL_R;
  const unsigned int bar_s = (unsigned int)__cvta_generic_to_shared(&bar);
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  constexpr unsigned int bytes = WIN_H * SCL_WIN_W * sizeof(SCL_TYPE_0);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar_s));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (t == 0) {
    const unsigned int dst = (unsigned int)__cvta_generic_to_shared(win);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(bar_s), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];"
        :: "r"(dst), "l"(&tmap), "r"((int)x_org), "r"((int)y_org), "r"(bar_s)
        : "memory");
    // Bounded wait on phase 0 by thread 0 only; the verdict is block-uniform.
    unsigned int done = 0, polls = 0;
    while (!done) {
      asm volatile(
          "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 0;"
          " selp.u32 %0, 1, 0, p; }"
          : "=r"(done) : "r"(bar_s) : "memory");
      if (!done) {
        if (++polls > spin_limit) break;
        scl_nanosleep(32);
      }
    }
    s_ok = done ? 1 : 0;
    if (!done) {
      scl_raise(err, SCL_DEV_ERR_TIMEOUT);
      // The copy may still land in this block's shared memory: thread 0 keeps
      // the block alive (bounded again) before it returns.
      for (unsigned int k = 0; k < spin_limit && !done; ++k) {
        scl_nanosleep(64);
        asm volatile(
            "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 0;"
            " selp.u32 %0, 1, 0, p; }"
            : "=r"(done) : "r"(bar_s) : "memory");
      }
    }
  }
  __syncthreads();
  if (!s_ok) return;
  const bool border = x_org < 0 || y_org < 0 || x_org + SCL_WIN_W > (long long)cols ||
                      y_org + WIN_H > (long long)rows;
#if SCL_PADDING == 1 || SCL_NEUTRAL_IS_ZERO == 0
  if (border) scl_patch_border<WIN_H>(win, x_org, y_org, rows, cols);
#endif
  __syncthreads();
  scl_compute_tile<PY>(win, out, rows, cols, x0, y0 SCL_EXTRA_ARGS);
}
#endif
