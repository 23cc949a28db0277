// ---------------------------------------------------------------------------
// Scan for sm_103a: single-pass decoupled look-back (Merrill & Garland,
// "Single-pass Parallel Prefix Scan with Decoupled Look-back", NVIDIA 2016).
//
// Replaces the reference's recursive Blelloch scan (SCL_SCAN, ceil(log_256 N)
// passes) and its uniform-add passes (SCL_UNIFORM_COMBINATION) of
// include/SkelCL/detail/ScanKernel.cl:74-250 / ScanDef.h:91-259.
//
// Semantics kept from the reference: the output is the EXCLUSIVE scan seeded
// with the identity (out[0] = id, out[i] = x[0] + ... + x[i-1]; ScanKernel.cl
// clears the last element to SCL_IDENTITY before the down-sweep and pads
// partial blocks with it), and the operator must be associative (the
// reference combines in tree order).  Extensions: SCL_SHAPE_INCLUSIVE gives
// the inclusive scan, SCL_SHAPE_REVERSE scans from the last element (the
// adjoint of a forward sum-scan is a reverse scan).
//
// Tile = R rows x 256 threads x V elements (V = 16 bytes / sizeof T), loaded
// with coalesced 16-byte accesses: row r of the tile is one contiguous span of
// 256*V elements, thread t holds elements [r*256*V + t*V, +V).
// In-tile: per-thread sequential fold, warp shuffles, one warp scans the R*8
// warp totals.  Across tiles: warp 0 publishes the tile aggregate, then looks
// back over up to 32 predecessors per step; every wait is bounded by
// `spin_limit` polls, after which the tile raises SCL_DEV_ERR_TIMEOUT and
// proceeds, so a launch always terminates.  Carries across tiles are held in
// SCL_CARRY_T (double for float element types).
// ---------------------------------------------------------------------------

#if SCL_KIND == 10
typedef SCL_TYPE_0 scl_T;
typedef SCL_CARRY_T scl_C;

#define SCL_SCAN_B 256
#define SCL_SCAN_W 8
#define SCL_FLAG_AGG 1u
#define SCL_FLAG_INC 2u

// Ordered inclusive warp scan: lane l gets x[0] + ... + x[l].
template <typename T>
__device__ __forceinline__ T scl_warp_incl(T v SCL_USER_PARAMS) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    T o = scl_shfl_up(v, off);
    if (lane >= off) v = SCL_FUNC(o, v SCL_EXTRA_ARGS);
  }
  return v;
}

template <int R>
__global__ void __launch_bounds__(SCL_SCAN_B)
scl_scan_k(const scl_T* in, scl_T* out, scl_u64 n, unsigned int flags, int aligned,
           unsigned int* status, scl_C* agg, scl_C* incl, unsigned int spin_limit,
           unsigned int* err SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int B = SCL_SCAN_B, W = SCL_SCAN_W;
  constexpr int V = scl_vec_width<sizeof(scl_T)>::value;
  constexpr int TILE = R * B * V;
  const bool inclusive = (flags & 1u) != 0, reverse = (flags & 2u) != 0;
  const scl_T ident = (scl_T)(SCL_IDENTITY);

  __shared__ unsigned int s_tile;
  __shared__ scl_T s_wsum[R * W];
  __shared__ scl_C s_prefix;
  const unsigned int num_tiles = (unsigned int)((n + TILE - 1) / TILE);
  if (threadIdx.x == 0) s_tile = atomicAdd(status + num_tiles, 1u);
  __syncthreads();
  const unsigned int tile = s_tile;
  const scl_u64 base = (scl_u64)tile * TILE;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // ---- load (logical order; reverse maps logical i to physical n-1-i)
  scl_T x[R][V];
  const bool full = aligned && base + TILE <= n && (!reverse || n % V == 0);
  if (full) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const scl_u64 q = (scl_u64)r * B + threadIdx.x;
      if (!reverse) {
        scl_pack<scl_T, V> p = scl_load<scl_T, V>(in + base + q * V);
#pragma unroll
        for (int e = 0; e < V; ++e) x[r][e] = p.v[e];
      } else {
        scl_pack<scl_T, V> p = scl_load<scl_T, V>(in + (n - base - (q + 1) * V));
#pragma unroll
        for (int e = 0; e < V; ++e) x[r][e] = p.v[V - 1 - e];
      }
    }
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const scl_u64 i = base + ((scl_u64)r * B + threadIdx.x) * V + e;
        x[r][e] = i < n ? in[reverse ? n - 1 - i : i] : ident;
      }
  }

  // ---- in-thread inclusive scan of each vector, then warp scans of totals
  scl_T wincl[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int e = 1; e < V; ++e) x[r][e] = SCL_FUNC(x[r][e - 1], x[r][e] SCL_EXTRA_ARGS);
    wincl[r] = scl_warp_incl(x[r][V - 1] SCL_EXTRA_ARGS);
    if (lane == 31) s_wsum[r * W + warp] = wincl[r];
  }
  __syncthreads();

  // ---- warp 0: scan the R*W warp totals (row-major = tile order), then the
  //      decoupled look-back for the tile prefix
  if (warp == 0) {
    scl_T carry = ident;
    scl_T tile_agg = ident;
#pragma unroll
    for (int c = 0; c < (R * W + 31) / 32; ++c) {
      const int q = c * 32 + lane;
      scl_T v = q < R * W ? s_wsum[q] : ident;
      scl_T vi = scl_warp_incl(v SCL_EXTRA_ARGS);
      scl_T ve = scl_shfl_up(vi, 1);
      if (lane == 0) ve = ident;
      if (q < R * W) s_wsum[q] = SCL_FUNC(carry, ve SCL_EXTRA_ARGS);  // exclusive prefix
      scl_T total = scl_shfl_idx(vi, 31);
      carry = SCL_FUNC(carry, total SCL_EXTRA_ARGS);
    }
    tile_agg = carry;
    const scl_C aggc = (scl_C)tile_agg;
    scl_C prefix = (scl_C)ident;
    if (tile == 0) {
      if (lane == 0) {
        scl_st_cg(&incl[0], aggc);
        scl_st_release(&status[0], SCL_FLAG_INC);
      }
    } else {
      if (lane == 0) {
        scl_st_cg(&agg[tile], aggc);
        scl_st_release(&status[tile], SCL_FLAG_AGG);
      }
      scl_C running = (scl_C)ident;  // fold of the tiles already visited (later ones)
      long long pred = (long long)tile - 1;
      while (true) {
        const long long idx = pred - lane;
        unsigned int f = SCL_FLAG_INC;
        bool timed_out = false;
        if (idx >= 0) {
          unsigned int polls = 0;
          f = scl_ld_acquire(&status[idx]);
          while (f == 0u) {
            if (++polls > spin_limit) { timed_out = true; break; }
            scl_nanosleep(polls < 64 ? 32u : 256u);
            f = scl_ld_acquire(&status[idx]);
          }
        }
        if (timed_out) {
          scl_raise(err, SCL_DEV_ERR_TIMEOUT);
          f = SCL_FLAG_INC;
        }
        const unsigned int pmask = __ballot_sync(0xffffffffu, f == SCL_FLAG_INC);
        const int first = pmask ? __ffs(pmask) - 1 : 32;
        scl_C v = (scl_C)ident;
        if (lane <= first && idx >= 0 && !timed_out)
          v = (f == SCL_FLAG_INC) ? scl_ld_cg(&incl[idx]) : scl_ld_cg(&agg[idx]);
        // ordered fold over lanes: higher lane = earlier tile
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          scl_C o = scl_shfl_down(v, off);
          if (lane + off < 32) v = (scl_C)SCL_FUNC_C(o, v SCL_EXTRA_ARGS);
        }
        const scl_C window = scl_shfl_idx(v, 0);
        running = (scl_C)SCL_FUNC_C(window, running SCL_EXTRA_ARGS);
        if (pmask) break;
        pred -= 32;
      }
      prefix = running;
      if (lane == 0) {
        scl_st_cg(&incl[tile], (scl_C)SCL_FUNC_C(prefix, aggc SCL_EXTRA_ARGS));
        scl_st_release(&status[tile], SCL_FLAG_INC);
      }
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();

  // ---- outputs
  const scl_T tile_carry = (scl_T)s_prefix;
  scl_T y[R][V];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    scl_T lane_excl = scl_shfl_up(wincl[r], 1);
    if (lane == 0) lane_excl = ident;
    const scl_T pre = SCL_FUNC(SCL_FUNC(tile_carry, s_wsum[r * W + warp] SCL_EXTRA_ARGS),
                               lane_excl SCL_EXTRA_ARGS);
#pragma unroll
    for (int e = 0; e < V; ++e) {
      if (inclusive) y[r][e] = SCL_FUNC(pre, x[r][e] SCL_EXTRA_ARGS);
      else y[r][e] = e == 0 ? pre : SCL_FUNC(pre, x[r][e - 1] SCL_EXTRA_ARGS);
    }
  }
  if (full) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const scl_u64 q = (scl_u64)r * B + threadIdx.x;
      scl_pack<scl_T, V> p;
      if (!reverse) {
#pragma unroll
        for (int e = 0; e < V; ++e) p.v[e] = y[r][e];
        scl_store<scl_T, V>(out + base + q * V, p);
      } else {
#pragma unroll
        for (int e = 0; e < V; ++e) p.v[V - 1 - e] = y[r][e];
        scl_store<scl_T, V>(out + (n - base - (q + 1) * V), p);
      }
    }
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const scl_u64 i = base + ((scl_u64)r * B + threadIdx.x) * V + e;
        if (i < n) out[reverse ? n - 1 - i : i] = y[r][e];
      }
  }
}
#endif
