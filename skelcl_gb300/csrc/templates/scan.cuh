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
// 256*V elements, thread t holds elements [r*256*V + t*V, +V).  The staged
// kernel's tiles are numbered by block index: blocks are dispatched in index
// order, so a tile only waits on tiles whose blocks have started, and the
// tile's copy is issued at once (an atomic ticket taken first, as the
// register kernel still does, put one L2 round trip in front of every tile's
// copy: 2^26 floats 102.4 against 98.2 us).  Were that order ever broken,
// the bounded waits below would end the launch with SCL_DEV_ERR_TIMEOUT
// instead of a hang.
// In-tile: per-thread sequential fold, warp shuffles, one warp scans the R*8
// warp totals, publishes the tile aggregate and looks back over up to 32
// predecessors per round trip (one lane per predecessor).  Every wait is
// bounded by `spin_limit` polls, after which the tile raises
// SCL_DEV_ERR_TIMEOUT and proceeds, so a launch always terminates.  Carries
// across tiles are held in SCL_CARRY_T (double for float element types).
//
// Tile status: one 16-byte slot {aggregate word, inclusive word} per tile,
// each slot alone on a 128-byte line (SCL_SLOT_STRIDE words apart), so a poll
// is one 16-byte load and publishers and pollers of different tiles never
// share a line (measured on GB300: sharing lines cost about a third of the
// scan's bandwidth).
//   mode 1, carry <= 4 bytes: word = 1<<32 | value bits; 0 = not published
//   mode 2, carry is double : word = ~(value bits); 0 = not published
//   mode 0, other carries   : flag word (release/acquire) + separate values
// ---------------------------------------------------------------------------

#if SCL_KIND == 10 || SCL_KIND == 17
typedef SCL_TYPE_0 scl_T;
typedef SCL_CARRY_T scl_C;
#if SCL_KIND == 17
// Fused Scan -> Map (no counterpart in the reference, which materialises the
// scanned vector): the staged kernel stores USR_MAP(scan value) instead of
// the scan value.  Extra arguments: the Scan's first, then the Map's.
typedef SCL_TYPE_1 scl_O;
#define SCL_EPILOGUE(v) USR_MAP(v SCL_SECOND_ARGS)
#else
typedef scl_T scl_O;
#define SCL_EPILOGUE(v) (v)
#endif

#define SCL_SCAN_B 256
#define SCL_SCAN_W 8
#define SCL_SLOT_STRIDE 16  // 64-bit words between tile slots (128 bytes)
#define SCL_FLAG_AGG 1u
#define SCL_FLAG_INC 2u

template <typename A, typename B> struct scl_same { static constexpr bool value = false; };
template <typename A> struct scl_same<A, A> { static constexpr bool value = true; };
template <typename C> struct scl_status_mode {
  static constexpr int value = sizeof(C) <= 4 ? 1 : (scl_same<C, double>::value ? 2 : 0);
};

// Staged kernel: when carries are wider than the elements (FP64 carries of a
// float scan), each thread folds its lane prefix into the staged tile before
// the look-back instead of keeping R warp prefixes in registers across it
// (measured on GB300, f32 2^26: 40 registers with spills -> 29 without, 4.5 %
// faster; for 4-byte carries keeping them is 1 % faster).
constexpr bool kLocalPrefix = !scl_same<scl_C, scl_T>::value;

__device__ __forceinline__ unsigned long long scl_ld_relaxed64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void scl_st_relaxed64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

template <typename C>
__device__ __forceinline__ unsigned long long scl_pack_word(const C& v) {
  if constexpr (scl_status_mode<C>::value == 1) {
    unsigned int bits = 0;
    memcpy(&bits, &v, sizeof(C));
    return (1ull << 32) | bits;
  } else {
    unsigned long long bits;
    memcpy(&bits, &v, 8);
    return ~bits;  // all-ones bits (never produced by arithmetic) would read as "not published"
  }
}
template <typename C>
__device__ __forceinline__ C scl_unpack_word(unsigned long long w) {
  C v;
  if constexpr (scl_status_mode<C>::value == 1) {
    unsigned int bits = (unsigned int)w;
    memcpy(&v, &bits, sizeof(C));
  } else {
    const unsigned long long bits = ~w;
    memcpy(&v, &bits, 8);
  }
  return v;
}

// Ordered inclusive warp scan: lane l gets x[0] + ... + x[l].
template <typename T>
__device__ __forceinline__ T scl_warp_incl(T v SCL_USER_PARAMS) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    T o = scl_shfl_up(v, off);
    if (lane >= off) v = SCL_FUNC(o, v SCL_OP_ARGS);
  }
  return v;
}

// Status storage of one launch (device pointers into the workspace).
struct scl_scan_status {
  unsigned long long* slots;  // modes 1, 2: slot of tile t at slots[t * SCL_SLOT_STRIDE]
  unsigned int* flags;        // mode 0
  scl_C* agg;                 // mode 0
  scl_C* incl;                // mode 0
};

// What a launch clears for the next one: the slots (or flags) [0, n) of the
// status region the previous launch used, and that region's ticket word.
// The host alternates launches between two regions, so no launch needs a
// separate clear before it (a launch recorded in a graph uses a third
// region that the graph clears itself).
struct scl_scan_clear {
  unsigned long long* slots;  // modes 1, 2
  unsigned int* flags;        // mode 0
  unsigned int* ticket;       // reset to 0 (block 0), or null
  unsigned long long n;
};

__device__ __forceinline__ void scl_scan_clear_other(const scl_scan_clear& c) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && c.ticket) *c.ticket = 0u;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < c.n;
       i += stride) {
    if constexpr (scl_status_mode<scl_C>::value != 0) {
      asm volatile("st.global.v2.u64 [%0], {%1, %1};" :: "l"(c.slots + i * SCL_SLOT_STRIDE), "l"(0ull)
                   : "memory");
    } else {
      c.flags[i] = 0u;
    }
  }
}

__device__ __forceinline__ void scl_publish(const scl_scan_status& st, unsigned int tile,
                                            bool inclusive, const scl_C& v) {
  if constexpr (scl_status_mode<scl_C>::value != 0) {
    scl_st_relaxed64(st.slots + (size_t)tile * SCL_SLOT_STRIDE + (inclusive ? 1 : 0),
                     scl_pack_word(v));
  } else {
    scl_st_cg(inclusive ? &st.incl[tile] : &st.agg[tile], v);
    scl_st_release(&st.flags[tile], inclusive ? SCL_FLAG_INC : SCL_FLAG_AGG);
  }
}

// Poll predecessor `idx` until it published something (or the wait gives up).
// Returns 2 = inclusive prefix, 1 = aggregate, 0 = gave up; value in *v.
__device__ __forceinline__ int scl_poll(const scl_scan_status& st, long long idx,
                                        unsigned int spin_limit, scl_C* v) {
  unsigned int polls = 0;
  while (true) {
    if constexpr (scl_status_mode<scl_C>::value != 0) {
      unsigned long long wa, wi;
      asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];"
                   : "=l"(wa), "=l"(wi) : "l"(st.slots + (size_t)idx * SCL_SLOT_STRIDE) : "memory");
      if (wi != 0ull) { *v = scl_unpack_word<scl_C>(wi); return 2; }
      if (wa != 0ull) { *v = scl_unpack_word<scl_C>(wa); return 1; }
    } else {
      const unsigned int f = scl_ld_acquire(&st.flags[idx]);
      if (f == SCL_FLAG_INC) { *v = scl_ld_cg(&st.incl[idx]); return 2; }
      if (f == SCL_FLAG_AGG) { *v = scl_ld_cg(&st.agg[idx]); return 1; }
    }
    if (++polls > spin_limit) return 0;
    if (polls > 32) scl_nanosleep(32);
  }
}

// Decoupled look-back of warp 0 (all 32 lanes) for tile number `tile`, whose
// sequence starts at tile `first`: returns the fold of every
// earlier tile of the sequence, combined as f(earlier, later).  Each round
// reads 32 predecessors (one per lane, lane l = tile - 1 - l); a round that
// finds an inclusive prefix ends the look-back, otherwise its aggregates are
// folded in and the next 32 are read.  (Measured on GB300 and not kept:
// 64 or 128 predecessors per round, several loads in flight per lane, in
// every round, or only after a first round without an inclusive prefix, or
// only for the first two waves of tiles -- all slower, 1.5-18 %; with the
// code present but never taken the time is unchanged.)
__device__ __forceinline__ scl_C scl_lookback(const scl_scan_status& st, long long tile, long long first,
                                              unsigned int spin_limit, unsigned int* err
                                                  SCL_USER_PARAMS) {
  const int lane = threadIdx.x & 31;
  const scl_C cid = (scl_C)(scl_T)(SCL_IDENTITY);
  scl_C running = cid;  // fold of the tiles already visited (later ones)
  long long pred = tile - 1;
  bool first_round = true;
  while (true) {
    const long long idx = pred - lane;
    scl_C v = cid;
    int kind = 2;  // before the sequence's first tile: nothing to add, stop here
    if (idx >= first) {
      kind = scl_poll(st, idx, spin_limit, &v);
      if (kind == 0) {
        scl_raise(err, SCL_DEV_ERR_TIMEOUT);
        v = cid;
        kind = 2;
      }
    }
    const unsigned int pmask = __ballot_sync(0xffffffffu, kind == 2);
    // the usual case: the nearest predecessor already holds its inclusive
    // prefix, and nothing needs folding (the fold below costs five shuffle
    // rounds, in FP64 for float carries)
    if (pmask & 1u) {
      const scl_C w = scl_shfl_idx(v, 0);
      return first_round ? w : (scl_C)SCL_FUNC_C(w, running SCL_OP_ARGS);
    }
    const int first_inc = pmask ? __ffs(pmask) - 1 : 31;  // nearest inclusive prefix
    if (lane > first_inc) v = cid;
    // ordered fold over lanes: higher lane = earlier tile
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      scl_C o = scl_shfl_down(v, off);
      if (lane + off < 32) v = (scl_C)SCL_FUNC_C(o, v SCL_OP_ARGS);
    }
    const scl_C window = scl_shfl_idx(v, 0);
    running = (scl_C)SCL_FUNC_C(window, running SCL_OP_ARGS);
    if (pmask) return running;
    pred -= 32;
    first_round = false;
  }
}

template <int R, int MINB>
__global__ void __launch_bounds__(SCL_SCAN_B, MINB)  // MINB resident tiles per SM at least
scl_scan_k(const scl_T* in, scl_T* out, scl_u64 n, unsigned int flags, int aligned,
           unsigned int* tile_counter, scl_scan_status st, scl_scan_clear clr,
           unsigned int spin_limit, unsigned int* err SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  constexpr int B = SCL_SCAN_B, W = SCL_SCAN_W;
  constexpr int V = scl_vec_width<sizeof(scl_T)>::value;
  constexpr int TILE = R * B * V;
  const bool inclusive = (flags & 1u) != 0, reverse = (flags & 2u) != 0;
  const scl_T ident = (scl_T)(SCL_IDENTITY);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  __shared__ unsigned int s_tile;
  __shared__ scl_T s_wsum[R * W];
  __shared__ scl_T s_carry;  // the tile's prefix, converted once to the element type
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
  scl_scan_clear_other(clr);
  __syncthreads();
  const unsigned int tile = s_tile;
  const scl_u64 base = (scl_u64)tile * TILE;

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
    for (int e = 1; e < V; ++e) x[r][e] = SCL_FUNC(x[r][e - 1], x[r][e] SCL_OP_ARGS);
    wincl[r] = scl_warp_incl(x[r][V - 1] SCL_EXTRA_ARGS);
    if (lane == 31) s_wsum[r * W + warp] = wincl[r];
  }
  __syncthreads();

  // ---- warp 0: exclusive prefixes of the R*W warp totals (row-major = tile
  //      order), the tile aggregate, then the look-back for the tile prefix
  if (warp == 0) {
    scl_T carry = ident;
#pragma unroll
    for (int c = 0; c < (R * W + 31) / 32; ++c) {
      const int q = c * 32 + lane;
      scl_T v = q < R * W ? s_wsum[q] : ident;
      scl_T vi = scl_warp_incl(v SCL_EXTRA_ARGS);
      scl_T ve = scl_shfl_up(vi, 1);
      if (lane == 0) ve = ident;
      if (q < R * W) s_wsum[q] = SCL_FUNC(carry, ve SCL_OP_ARGS);
      scl_T total = scl_shfl_idx(vi, 31);
      carry = SCL_FUNC(carry, total SCL_OP_ARGS);
    }
    const scl_C aggc = (scl_C)carry;
    scl_C prefix = (scl_C)ident;
    if (lane == 0) scl_publish(st, tile, tile == 0, aggc);
    if (tile != 0) {
      prefix = scl_lookback(st, (long long)tile, 0, spin_limit, err SCL_EXTRA_ARGS);
      if (lane == 0) scl_publish(st, tile, true, (scl_C)SCL_FUNC_C(prefix, aggc SCL_OP_ARGS));
    }
    if (lane == 0) s_carry = (scl_T)prefix;
  }
  __syncthreads();

  // ---- outputs (computed in place in x)
  const scl_T tile_carry = s_carry;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    scl_T lane_excl = scl_shfl_up(wincl[r], 1);
    if (lane == 0) lane_excl = ident;
    const scl_T pre = SCL_FUNC(SCL_FUNC(tile_carry, s_wsum[r * W + warp] SCL_OP_ARGS),
                               lane_excl SCL_OP_ARGS);
    if (inclusive) {
#pragma unroll
      for (int e = 0; e < V; ++e) x[r][e] = SCL_FUNC(pre, x[r][e] SCL_OP_ARGS);
    } else {
#pragma unroll
      for (int e = V - 1; e > 0; --e) x[r][e] = SCL_FUNC(pre, x[r][e - 1] SCL_OP_ARGS);
      x[r][0] = pre;
    }
  }
  if (full) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const scl_u64 q = (scl_u64)r * B + threadIdx.x;
      scl_pack<scl_T, V> p;
      if (!reverse) {
#pragma unroll
        for (int e = 0; e < V; ++e) p.v[e] = x[r][e];
        scl_store<scl_T, V>(out + base + q * V, p);
      } else {
#pragma unroll
        for (int e = 0; e < V; ++e) p.v[V - 1 - e] = x[r][e];
        scl_store<scl_T, V>(out + (n - base - (q + 1) * V), p);
      }
    }
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const scl_u64 i = base + ((scl_u64)r * B + threadIdx.x) * V + e;
        if (i < n) out[reverse ? n - 1 - i : i] = x[r][e];
      }
  }
}

// ---------------------------------------------------------------------------
// Shared-memory staged variant.  One elected thread brings the tile into
// shared memory with bulk asynchronous copies (completion counted on an
// mbarrier), threads scan it there, and only the R warp totals per thread stay
// in registers while warp 0 looks back: about 40 registers per thread, so the
// SM holds as many tiles as its shared memory allows (6 of 32 KB) instead of
// as many as the register file allows with the tile in registers (4).
// Reverse, ragged and unaligned tiles are staged with ordinary loads.
// ---------------------------------------------------------------------------

// Segmented scan of the segments of at most short_max elements: one warp per
// segment, warps striding over the segments (warp `wid` of `nw`); per round
// each lane scans U contiguous elements serially, a warp scan combines the
// lanes' totals, and rounds are chained through a carry in the element type
// (no block boundary is crossed, as inside one tile of the tiled kernel; FP64
// carries here would make the FP64 pipe the bound for tiny segments); longer
// segments (and empty ones, which have nothing to write) are left to the
// tiles.  Operand order and identity handling are those of the tiled kernel:
// f(earlier, later), the exclusive form starts from SCL_IDENTITY.
template <int U>
__device__ __forceinline__ void scl_scan_short_run(const scl_T* in, scl_O* out, const scl_u64* seg_off,
                                                   scl_u64 n_seg, unsigned int flags, scl_u64 short_max,
                                                   scl_u64 wid, scl_u64 nw SCL_USER_PARAMS) {
  const int lane = threadIdx.x & 31;
  const bool inclusive = (flags & 1u) != 0, reverse = (flags & 2u) != 0;
  const scl_T ident = (scl_T)(SCL_IDENTITY);
  // round b of a segment [lo, hi): lane l holds the logical elements
  // b + l*U .. b + l*U + U-1, which sit at lo + e, or at hi - 1 - e reversed
  // (identity past the end, and nothing loaded for segments left to tiles)
  auto load = [&](scl_T (&v)[U], scl_u64 lo, scl_u64 hi, scl_u64 b) {
    const scl_u64 len = hi - lo;
    const bool mine = len <= short_max;
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const scl_u64 e = b + (scl_u64)lane * U + k;
      v[k] = (mine && e < len) ? in[reverse ? hi - 1 - e : lo + e] : ident;
    }
  };
  auto bounds = [&](scl_u64 sg, scl_u64* lo, scl_u64* hi) {
    *lo = 0;
    *hi = 0;
    if (sg < n_seg) {
      *lo = seg_off[sg];
      const scl_u64 h = seg_off[sg + 1];
      *hi = h > *lo ? h : *lo;
    }
  };
  // software pipeline: the next segment's first round and the offsets of
  // the one after are loaded while this segment is scanned
  scl_u64 sg = wid;
  scl_u64 lo, hi, lo_n, hi_n;
  bounds(sg, &lo, &hi);
  bounds(sg + nw, &lo_n, &hi_n);
  scl_T v[U];
  load(v, lo, hi, 0);
  for (; sg < n_seg; sg += nw) {
    scl_u64 lo_nn, hi_nn;
    bounds(sg + 2 * nw, &lo_nn, &hi_nn);
    scl_T vn[U];
    load(vn, lo_n, hi_n, 0);
    const scl_u64 len = hi - lo;
    if (len > 0 && len <= short_max) {
      scl_T carry = ident;
      for (scl_u64 b = 0; b < len; b += 32 * U) {
        if (b > 0) load(v, lo, hi, b);
        const scl_u64 e0 = b + (scl_u64)lane * U;
#pragma unroll
        for (int k = 1; k < U; ++k) v[k] = SCL_FUNC(v[k - 1], v[k] SCL_OP_ARGS);
        const scl_T tot = scl_warp_incl(v[U - 1] SCL_EXTRA_ARGS);
        scl_T lane_excl = scl_shfl_up(tot, 1);
        if (lane == 0) lane_excl = ident;
        const scl_T pre = SCL_FUNC(carry, lane_excl SCL_OP_ARGS);
#pragma unroll
        for (int k = 0; k < U; ++k) {
          const scl_u64 e = e0 + k;
          if (e < len) {
            const scl_T r = inclusive ? SCL_FUNC(pre, v[k] SCL_OP_ARGS)
                                      : (k == 0 ? pre : SCL_FUNC(pre, v[k - 1] SCL_OP_ARGS));
            out[reverse ? hi - 1 - e : lo + e] = SCL_EPILOGUE(r);
          }
        }
        carry = SCL_FUNC(carry, scl_shfl_idx(tot, 31) SCL_OP_ARGS);
      }
    }
    lo = lo_n;
    hi = hi_n;
    lo_n = lo_nn;
    hi_n = hi_nn;
#pragma unroll
    for (int k = 0; k < U; ++k) v[k] = vn[k];
  }
}

// Window role of a planned segmented scan (the blocks past the tiles): block
// r takes window record r of the plan, {first vector, end vector, first
// element, elements}: consecutive vectors of at most short_max elements that
// start in one window of short_max elements (all but the last end inside
// it, so the record spans at most 2 * short_max = TILE elements, one staged
// tile).  The record's elements are brought into shared memory by bulk
// asynchronous copies (element e0 + p at ts[p + shift]; bounded wait) while
// each thread reads its first vector's offsets, and every vector is scanned
// in place there: one of at most SCL_WIN_THREAD elements by
// one thread, in element order; a longer one by a warp, in rounds of 32 x U
// logical elements (lane l holds U consecutive ones; a reverse scan reads the
// vector from its end), the lanes' totals scanned across the warp and rounds
// chained by a carry.  Then the block stores the record's elements in order
// (the vectors cover them).  f(earlier, later) throughout, in the element
// type; the exclusive form starts from SCL_IDENTITY (neutral, as for the
// tiles' padding).
template <int TILE>
__device__ __forceinline__ void scl_scan_window_run(const scl_T* in, scl_O* out, const scl_u64* seg_off,
                                                    const scl_u64* win_rec, scl_u64 r,
                                                    unsigned int flags, scl_T* ts, unsigned int bar_s,
                                                    unsigned int spin_limit,
                                                    unsigned int* err SCL_USER_PARAMS) {
  constexpr int B = SCL_SCAN_B, NW = B / 32, U = 4;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool inclusive = (flags & 1u) != 0, reverse = (flags & 2u) != 0;
  const scl_T ident = (scl_T)(SCL_IDENTITY);
  const scl_u64 lo = win_rec[4 * r], top = win_rec[4 * r + 1], e0 = win_rec[4 * r + 2];
  const scl_u64 ln = win_rec[4 * r + 3];
  const int len = (int)(ln < (scl_u64)TILE ? ln : (scl_u64)TILE);  // (more only for bad offsets)
  if (len == 0) return;  // (block-uniform) nothing to write for empty vectors
  __shared__ int s_ok;
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
  // short vectors: a thread each, in place
  for (; sg < top; sg += B) {
    const scl_u64 a = a_n, b = b_n;
    if (sg + B < top) {
      a_n = seg_off[sg + B];
      b_n = seg_off[sg + B + 1];
    }
    if (b <= a || b - a > SCL_WIN_THREAD || a < e0 || b > e0 + (scl_u64)len) continue;
    const int nv = (int)(b - a);
    scl_T* v = ts + (int)(a - e0) + shift;
    const int step = reverse ? -1 : 1;
    if (reverse) v += nv - 1;
    scl_T acc = v[0];
    if (!inclusive) v[0] = ident;
#pragma unroll 4
    for (int e = 1; e < nv; ++e) {
      const scl_T x = v[e * step];
      if (inclusive) {
        acc = SCL_FUNC(acc, x SCL_OP_ARGS);
        v[e * step] = acc;
      } else {
        v[e * step] = acc;
        acc = SCL_FUNC(acc, x SCL_OP_ARGS);
      }
    }
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
      const scl_u64 a = __shfl_sync(0xffffffffu, a_l, k), b = __shfl_sync(0xffffffffu, b_l, k);
      if (b <= a || b - a <= SCL_WIN_THREAD) continue;  // (empty, or a thread's above)
      if (a < e0 || b > e0 + (scl_u64)len) continue;  // (only for offsets changed since the plan)
      const int pa = (int)(a - e0) + shift, nv = (int)(b - a);
      // logical element e of the vector sits at ts[at(e)]
      auto at = [&](int e) { return reverse ? pa + nv - 1 - e : pa + e; };
      scl_T carry = ident;
      for (int b0 = 0; b0 < nv; b0 += 32 * U) {
        const int eb = b0 + lane * U;
        scl_T v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = eb + u < nv ? ts[at(eb + u)] : ident;
#pragma unroll
        for (int u = 1; u < U; ++u) v[u] = SCL_FUNC(v[u - 1], v[u] SCL_OP_ARGS);
        const scl_T tot = scl_warp_incl(v[U - 1] SCL_EXTRA_ARGS);
        scl_T lane_excl = scl_shfl_up(tot, 1);
        if (lane == 0) lane_excl = ident;
        const scl_T pre = SCL_FUNC(carry, lane_excl SCL_OP_ARGS);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (eb + u < nv)
            ts[at(eb + u)] = inclusive ? SCL_FUNC(pre, v[u] SCL_OP_ARGS)
                                       : (u == 0 ? pre : SCL_FUNC(pre, v[u - 1] SCL_OP_ARGS));
        }
        carry = SCL_FUNC(carry, scl_shfl_idx(tot, 31) SCL_OP_ARGS);
      }
    }
  }
  __syncthreads();
  for (int p = threadIdx.x; p < len; p += B) out[e0 + p] = SCL_EPILOGUE(ts[p + shift]);
}

// The warp-per-segment kernel on its own (segmented launches without a
// segment plan; with one, scl_scan_s<R, MINB, 2> runs the same code in the
// blocks past the tiles).
template <int U>
__global__ void __launch_bounds__(256)
scl_scan_short(const scl_T* in, scl_O* out, const scl_u64* seg_off, scl_u64 n_seg,
               unsigned int flags, scl_u64 short_max SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  scl_scan_short_run<U>(in, out, seg_off, n_seg, flags, short_max,
                        ((scl_u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                        ((scl_u64)gridDim.x * blockDim.x) >> 5 SCL_EXTRA_ARGS);
}
//
// Tiles lie on the 16-byte grid of `in`: with `a` the first element index on
// a 16-byte boundary, a (forward) sequence [lo, hi) starts its first tile at
// lo rounded down onto the grid, and a reverse sequence ends its first tile
// at hi rounded up; elements of a tile outside the sequence are masked with
// the identity (which must be neutral, as for the reference's padding).  So
// every tile's shared-memory image has position p <-> element tile_lo + p,
// 16-byte vector slots, and one bulk copy of the tile's elements, rounded
// out to 16 bytes, when that stays inside the vector.  Elements that cannot
// be aligned (sizes other than 4, 8, 16 bytes, or a misaligned pointer) use
// ordinary loads.  The host counts tiles with the same rule (scl_scan_tiles).
//
// SEG = 1: a segmented scan, one independent scan per segment
// [seg_off[s], seg_off[s+1]) of the flat vector.  Segment s owns the tiles
// tile_start[s] .. tile_start[s+1]-1 (at least one), and the look-back stops
// at the segment's first tile.  Blocks past the last tile (the grid is an
// upper bound) return at once.
// SEG = 2: the same (a segment plan numbered the tiles), and the blocks past
// the tiles scan the segments of at most short_max elements, one window of
// them per block (scl_scan_window_run): one launch for a whole segmented
// scan.
template <int R, int MINB, int SEG = 0>
__global__ void __launch_bounds__(SCL_SCAN_B, MINB)
scl_scan_s(const scl_T* in, scl_O* out, scl_u64 n, unsigned int flags, int aligned,
           unsigned int* tile_counter, scl_scan_status st, scl_scan_clear clr, unsigned int spin_limit,
           unsigned int* err, const scl_u64* seg_off, const unsigned int* tile_start,
           scl_u64 n_seg, scl_u64 short_max, const scl_u64* win_rec,
           const unsigned int* tile_seg, unsigned int n_tiles SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  (void)aligned;
  (void)short_max;
  (void)win_rec;
  (void)tile_seg;
  (void)tile_counter;
  // segmented: the tile count, from the host when a plan knows it (~0u:
  // read it from tile_start[n_seg])
  unsigned int nt = 0;
  if constexpr (SEG != 0) nt = n_tiles != ~0u ? n_tiles : tile_start[n_seg];
  (void)n_tiles;  // (the register kernel's ticket; the host passes both kernels the same arguments)
  constexpr int B = SCL_SCAN_B, W = SCL_SCAN_W;
  constexpr int V = scl_vec_width<sizeof(scl_T)>::value;
  constexpr int TILE = R * B * V;
  constexpr unsigned int ROW_BYTES = B * V * sizeof(scl_T);
  constexpr bool natural = sizeof(scl_T) == 4 || sizeof(scl_T) == 8 || sizeof(scl_T) == 16;
  const bool inclusive = (flags & 1u) != 0, reverse = (flags & 2u) != 0;
  const scl_T ident = (scl_T)(SCL_IDENTITY);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  scl_T* ts = reinterpret_cast<scl_T*>(scl_dyn_smem);  // position p <-> element tile_lo + p

  __shared__ __align__(8) unsigned long long bar;
  __shared__ unsigned int s_tile;
  __shared__ int s_ok;
  __shared__ scl_T s_wsum[R * W];
  __shared__ scl_T s_carry;  // the tile's prefix, converted once to the element type
  const unsigned int bar_s = (unsigned int)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    // the block index is the tile; segmented, the grid is an upper bound
    // and blocks at or past the tile count take no tile
    if constexpr (SEG == 0) {
      s_tile = blockIdx.x;
    } else {
      s_tile = blockIdx.x < nt ? blockIdx.x : 0xffffffffu;
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar_s));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  scl_scan_clear_other(clr);
  if constexpr (SEG == 2) {
    if (blockIdx.x >= nt) {  // (block-uniform: the whole block takes the window role)
      scl_scan_window_run<TILE>(in, out, seg_off, win_rec, blockIdx.x - nt, flags, ts, bar_s, spin_limit,
                                err SCL_EXTRA_ARGS);
      return;
    }
  }
  __syncthreads();
  const unsigned int tile = s_tile;
  unsigned int first = 0;  // number of the first tile of this tile's sequence
  long long lo = 0, hi = (long long)n;  // the sequence's elements
  if constexpr (SEG != 0) {
    __shared__ long long s_seg;
    if (threadIdx.x == 0) {
      long long sg = -1;
      if (tile < nt) {
        if (tile_seg) {  // (a segment plan's table)
          sg = (long long)tile_seg[tile];
        } else {
          scl_u64 l = 0, h = n_seg - 1;  // largest s with tile_start[s] <= tile
          while (l < h) {
            const scl_u64 mid = (l + h + 1) / 2;
            if (tile_start[mid] <= tile) l = mid; else h = mid - 1;
          }
          sg = (long long)l;
        }
      }
      s_seg = sg;
    }
    __syncthreads();
    if (s_seg < 0) return;
    const scl_u64 sg = (scl_u64)s_seg;
    first = tile_start[sg];
    lo = (long long)seg_off[sg];
    hi = (long long)seg_off[sg + 1];
    if (hi < lo) hi = lo;  // a decreasing offset (reported by the pre-pass)
    if (lo == hi) return;  // an empty segment's only tile: nobody looks back at it
  }
  const long long local = (long long)(tile - first);

  // ---- the tile's place on the grid, its valid elements [c_lo, c_hi)
  const bool grid = natural && ((scl_u64)in % sizeof(scl_T)) == 0;
  const long long vg = grid ? V : 1;
  const long long a = grid ? (long long)(((16u - ((scl_u64)in & 15u)) & 15u) / sizeof(scl_T)) : 0;
  long long tile_lo;
  if (!reverse) {
    const long long m = (((lo - a) % vg) + vg) % vg;
    tile_lo = lo - m + local * TILE;
  } else {
    const long long m = (((a - hi) % vg) + vg) % vg;
    tile_lo = hi + m - (local + 1) * TILE;
  }
  const long long c_lo = tile_lo > lo ? tile_lo : lo;
  const long long c_hi = tile_lo + TILE < hi ? tile_lo + TILE : hi;
  const bool full = c_lo == tile_lo && c_hi == tile_lo + TILE;

  // ---- stage: one bulk copy of [c_lo, c_hi) rounded out to 16 bytes, or loads
  const scl_u64 tbase = (scl_u64)in + (scl_u64)(tile_lo * (long long)sizeof(scl_T));
  const scl_u64 g0 = (scl_u64)in + (scl_u64)c_lo * sizeof(scl_T);
  const scl_u64 g1 = (scl_u64)in + (scl_u64)c_hi * sizeof(scl_T);
  const scl_u64 a0 = g0 & ~(scl_u64)15, a1 = (g1 + 15) & ~(scl_u64)15;
  const scl_u64 vlo = ((scl_u64)in + 15) & ~(scl_u64)15;
  const scl_u64 vhi = ((scl_u64)in + (scl_u64)n * sizeof(scl_T)) & ~(scl_u64)15;
  const bool bulk = grid && a0 >= vlo && a1 <= vhi;
  if (bulk) {
    if (threadIdx.x == 0) {
      const unsigned int bytes = (unsigned int)(a1 - a0);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                   :: "r"(bar_s), "r"(bytes) : "memory");
      const unsigned int dst = (unsigned int)__cvta_generic_to_shared(ts) + (unsigned int)(a0 - tbase);
      if (full) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
              :: "r"(dst + r * ROW_BYTES), "l"((const void*)(a0 + r * ROW_BYTES)), "r"(ROW_BYTES),
                 "r"(bar_s)
              : "memory");
      } else {
        for (unsigned int o = 0; o < bytes; o += ROW_BYTES) {
          const unsigned int sz = bytes - o < ROW_BYTES ? bytes - o : ROW_BYTES;
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
              :: "r"(dst + o), "l"((const void*)(a0 + o)), "r"(sz), "r"(bar_s)
              : "memory");
        }
      }
      const bool ok = scl_mbar_wait(bar_s, spin_limit);
      if (!ok) {
        scl_raise(err, SCL_DEV_ERR_TIMEOUT);
        // The copies may still land in this block's shared memory: the block
        // stays until they have (bounded by about 0.1 s, whatever the
        // caller's poll limit), and the tile is not used.
        scl_mbar_wait(bar_s, 1u << 21);
      }
      s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) return;  // successors time out too and see the error flag
  } else {
    for (int k = threadIdx.x; k < TILE; k += B) {
      const long long i = tile_lo + k;
      ts[k] = (i >= c_lo && i < c_hi) ? in[i] : ident;
    }
    __syncthreads();
  }
  const bool mask = bulk && !full;  // positions outside [c_lo, c_hi) hold other data

  // ---- in-thread inclusive scan of each logical vector (written back to its
  //      slot in logical order), warp scans of the vector totals.  Logical
  //      vector q sits at q*V, or at TILE-(q+1)*V reversed for a reverse scan.
  scl_T wincl[R];  // (unused with local prefixes)
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = r * B + threadIdx.x;
    const int pos = reverse ? TILE - (q + 1) * V : q * V;
    scl_pack<scl_T, V> p = scl_load<scl_T, V>(ts + pos);
    if (mask) {
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const long long i = tile_lo + pos + e;
        if (i < c_lo || i >= c_hi) p.v[e] = ident;
      }
    }
    if (reverse) {
#pragma unroll
      for (int e = 0; e < V / 2; ++e) {
        const scl_T t = p.v[e];
        p.v[e] = p.v[V - 1 - e];
        p.v[V - 1 - e] = t;
      }
    }
#pragma unroll
    for (int e = 1; e < V; ++e) p.v[e] = SCL_FUNC(p.v[e - 1], p.v[e] SCL_OP_ARGS);
    if constexpr (kLocalPrefix) {
      const scl_T tot = scl_warp_incl(p.v[V - 1] SCL_EXTRA_ARGS);
      scl_T lx = scl_shfl_up(tot, 1);
      if (lane == 0) lx = ident;
      if (lane == 31) s_wsum[r * W + warp] = tot;
#pragma unroll
      for (int e = 0; e < V; ++e) p.v[e] = SCL_FUNC(lx, p.v[e] SCL_OP_ARGS);
      scl_store<scl_T, V>(ts + pos, p);
    } else {
      scl_store<scl_T, V>(ts + pos, p);
      wincl[r] = scl_warp_incl(p.v[V - 1] SCL_EXTRA_ARGS);
      if (lane == 31) s_wsum[r * W + warp] = wincl[r];
    }
  }
  __syncthreads();

  // ---- warp 0: tile aggregate, publication and look-back (as scl_scan_k)
  if (warp == 0) {
    scl_T carry = ident;
#pragma unroll
    for (int c = 0; c < (R * W + 31) / 32; ++c) {
      const int q = c * 32 + lane;
      scl_T v = q < R * W ? s_wsum[q] : ident;
      scl_T vi = scl_warp_incl(v SCL_EXTRA_ARGS);
      scl_T ve = scl_shfl_up(vi, 1);
      if (lane == 0) ve = ident;
      if (q < R * W) s_wsum[q] = SCL_FUNC(carry, ve SCL_OP_ARGS);
      scl_T total = scl_shfl_idx(vi, 31);
      carry = SCL_FUNC(carry, total SCL_OP_ARGS);
    }
    const scl_C aggc = (scl_C)carry;
    scl_C prefix = (scl_C)ident;
    if (lane == 0) scl_publish(st, tile, tile == first, aggc);
    if (tile != first) {
      prefix = scl_lookback(st, (long long)tile, (long long)first, spin_limit, err SCL_EXTRA_ARGS);
      if (lane == 0) scl_publish(st, tile, true, (scl_C)SCL_FUNC_C(prefix, aggc SCL_OP_ARGS));
    }
    if (lane == 0) s_carry = (scl_T)prefix;
  }
  __syncthreads();

  // ---- outputs: 16-byte stores for whole slots when `out` shares the grid
  const scl_T tile_carry = s_carry;
  // (whole-slot stores need the output elements the size of the scanned ones)
  const bool ovec = sizeof(scl_O) == sizeof(scl_T) && full &&
                    (((scl_u64)out + (scl_u64)(tile_lo * (long long)sizeof(scl_O))) & 15u) == 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = r * B + threadIdx.x;
    const int pos = reverse ? TILE - (q + 1) * V : q * V;
    scl_pack<scl_T, V> p = scl_load<scl_T, V>(ts + pos);
    scl_pack<scl_T, V> o;  // logical order
    if constexpr (kLocalPrefix) {
      // the slot holds the warp-local inclusive values
      const scl_T pre = SCL_FUNC(tile_carry, s_wsum[r * W + warp] SCL_OP_ARGS);
      if (inclusive) {
#pragma unroll
        for (int e = 0; e < V; ++e) o.v[e] = SCL_FUNC(pre, p.v[e] SCL_OP_ARGS);
      } else {
        const scl_T lx = scl_shfl_up(p.v[V - 1], 1);  // the previous lane's last value
        o.v[0] = lane == 0 ? pre : SCL_FUNC(pre, lx SCL_OP_ARGS);
#pragma unroll
        for (int e = 1; e < V; ++e) o.v[e] = SCL_FUNC(pre, p.v[e - 1] SCL_OP_ARGS);
      }
    } else {
      scl_T lane_excl = scl_shfl_up(wincl[r], 1);
      if (lane == 0) lane_excl = ident;
      const scl_T pre = SCL_FUNC(SCL_FUNC(tile_carry, s_wsum[r * W + warp] SCL_OP_ARGS),
                                 lane_excl SCL_OP_ARGS);
      if (inclusive) {
#pragma unroll
        for (int e = 0; e < V; ++e) o.v[e] = SCL_FUNC(pre, p.v[e] SCL_OP_ARGS);
      } else {
        o.v[0] = pre;
#pragma unroll
        for (int e = 1; e < V; ++e) o.v[e] = SCL_FUNC(pre, p.v[e - 1] SCL_OP_ARGS);
      }
    }
    if (reverse) {  // back to physical order
#pragma unroll
      for (int e = 0; e < V / 2; ++e) {
        const scl_T t = o.v[e];
        o.v[e] = o.v[V - 1 - e];
        o.v[V - 1 - e] = t;
      }
    }
    scl_pack<scl_O, V> m;
#pragma unroll
    for (int e = 0; e < V; ++e) m.v[e] = SCL_EPILOGUE(o.v[e]);
    if (ovec) {
      scl_store<scl_O, V>(out + (tile_lo + pos), m);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const long long i = tile_lo + pos + e;
        if (i >= c_lo && i < c_hi) out[i] = m.v[e];
      }
    }
  }
}

#endif
