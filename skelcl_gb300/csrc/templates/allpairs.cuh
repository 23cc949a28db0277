// ---------------------------------------------------------------------------
// AllPairs for sm_103a on CUDA cores.
//
// SCL_KIND 12 (Reduce + Zip pair, include/SkelCL/detail/AllPairsKernel.cl:47-135):
//   P[i][j] = id (+) z(A[i][0],B[0][j]) (+) ... (+) z(A[i][K-1],B[K-1][j])
// folded strictly in k order (AllPairsKernel.cl:89-91); the right operand is
// K x N row-major (AllPairsKernel.cl:72).  Extra arguments: the Reduce's
// first, then the Zip's (AllPairsDef.h:265-269).
// Shape: 128 x 128 output tile per 256-thread block, 8 x 8 register
// accumulators per thread, k-tiles of 16 double-buffered in shared memory
// with the next tile prefetched into registers.  Unlike the reference, P is
// written once (the reference re-reads and re-writes P every 32-wide k
// segment, AllPairsKernel.cl:77-78,95-96).
//
// SCL_KIND 13 (user f(lmatrix_t*, rmatrix_t*, dim, ...),
// include/SkelCL/detail/AllPairsKernel2.cl:42-65): one output per thread in
// 16 x 16 blocks; when 16 rows of A and 16 columns of B fit in shared memory
// they are staged there and the accessors read the staged copies.
// ---------------------------------------------------------------------------
#if SCL_KIND == 12
#define SCL_AP_BM 128
#define SCL_AP_BN 128
// k-tile: 16 for 4-byte operands, 8 for wider ones (48 KB of static shared memory)
#define SCL_AP_BK ((sizeof(SCL_TYPE_0) <= 4 && sizeof(SCL_TYPE_1) <= 4) ? 16 : 8)
typedef SCL_TYPE_0 scl_L;
typedef SCL_TYPE_1 scl_Rt;
typedef SCL_TYPE_2 scl_O;

// Thread (tx, ty) of the 16 x 16 block owns rows {ty*4 .. +3, 64 + ty*4 .. +3}
// and columns {tx*4 .. +3, 64 + tx*4 .. +3} of the 128 x 128 tile: its
// shared-memory reads are 16-byte loads that a warp spreads over all banks.
// two blocks per SM when the accumulators are 4-byte values
extern "C" __global__ void __launch_bounds__(256, sizeof(SCL_TYPE_2) <= 4 ? 2 : 1)
scl_allpairs_simt(const scl_L* A, const scl_Rt* B, scl_O* P, unsigned int M, unsigned int N,
                  unsigned int K, int vec_a, int vec_b SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  __shared__ __align__(16) scl_L As[2][SCL_AP_BK][SCL_AP_BM];
  __shared__ __align__(16) scl_Rt Bs[2][SCL_AP_BK][SCL_AP_BN];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const unsigned int m0 = blockIdx.y * SCL_AP_BM, n0 = blockIdx.x * SCL_AP_BN;
  // global -> register mapping: A tile 128 rows x BK k (row = tid/2, AE
  // consecutive k per thread), B tile BK k x 128 cols (BE consecutive columns)
  constexpr int BK = SCL_AP_BK, AE = BK / 2, TPR = 256 / BK, BE = SCL_AP_BN / TPR;
  const int a_row = tid >> 1, a_k = (tid & 1) * AE;
  const int b_k = tid / TPR, b_col = (tid % TPR) * BE;
  scl_L ra[AE];
  scl_Rt rb[BE];
  auto load_tile = [&](unsigned int k0) {
    const unsigned int gm = m0 + a_row;
#pragma unroll
    for (int h = 0; h < AE / 4; ++h) {
      const unsigned int gk = k0 + a_k + h * 4;
      if (vec_a && gm < M && gk + 3 < K) {
        scl_pack<scl_L, 4> p = scl_load<scl_L, 4>(A + (scl_u64)gm * K + gk);
#pragma unroll
        for (int i = 0; i < 4; ++i) ra[h * 4 + i] = p.v[i];
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          ra[h * 4 + i] = (gm < M && gk + i < K) ? A[(scl_u64)gm * K + gk + i] : (scl_L)0;
      }
    }
    const unsigned int bk = k0 + b_k;
#pragma unroll
    for (int h = 0; h < BE / 4; ++h) {
      const unsigned int bn = n0 + b_col + h * 4;
      if (vec_b && bk < K && bn + 3 < N) {
        scl_pack<scl_Rt, 4> p = scl_load<scl_Rt, 4>(B + (scl_u64)bk * N + bn);
#pragma unroll
        for (int i = 0; i < 4; ++i) rb[h * 4 + i] = p.v[i];
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          rb[h * 4 + i] = (bk < K && bn + i < N) ? B[(scl_u64)bk * N + bn + i] : (scl_Rt)0;
      }
    }
  };
  auto store_tile = [&](int buf) {
#pragma unroll
    for (int i = 0; i < AE; ++i) As[buf][a_k + i][a_row] = ra[i];
#pragma unroll
    for (int i = 0; i < BE; ++i) Bs[buf][b_k][b_col + i] = rb[i];
  };
  auto step = [&](scl_O (&acc)[8][8], int cur, int kk) {
    scl_L a[8];
    scl_Rt b[8];
    const scl_pack<scl_L, 4> a0 = scl_load<scl_L, 4>(&As[cur][kk][ty * 4]);
    const scl_pack<scl_L, 4> a1 = scl_load<scl_L, 4>(&As[cur][kk][64 + ty * 4]);
    const scl_pack<scl_Rt, 4> b0 = scl_load<scl_Rt, 4>(&Bs[cur][kk][tx * 4]);
    const scl_pack<scl_Rt, 4> b1 = scl_load<scl_Rt, 4>(&Bs[cur][kk][64 + tx * 4]);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      a[i] = a0.v[i];
      a[4 + i] = a1.v[i];
      b[i] = b0.v[i];
      b[4 + i] = b1.v[i];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j)
        acc[i][j] = USR_REDUCE(acc[i][j], USR_ZIP(a[i], b[j] SCL_ZIP_ARGS) SCL_REDUCE_ARGS);
  };

  scl_O acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = (scl_O)(SCL_IDENTITY);

  const unsigned int ktiles = (K + SCL_AP_BK - 1) / SCL_AP_BK;
  load_tile(0);
  store_tile(0);
  __syncthreads();
  for (unsigned int kt = 0; kt < ktiles; ++kt) {
    const int cur = kt & 1;
    if (kt + 1 < ktiles) load_tile((kt + 1) * SCL_AP_BK);
    const unsigned int kmax = min((unsigned int)SCL_AP_BK, K - kt * SCL_AP_BK);
    if (kmax == SCL_AP_BK) {
#pragma unroll
      for (int kk = 0; kk < SCL_AP_BK; ++kk) step(acc, cur, kk);
    } else {
      for (unsigned int kk = 0; kk < kmax; ++kk) step(acc, cur, (int)kk);
    }
    if (kt + 1 < ktiles) store_tile(cur ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const unsigned int gm = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
    if (gm >= M) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const unsigned int gn = n0 + h * 64 + tx * 4;
      scl_O* dst = P + (scl_u64)gm * N + gn;
      if (sizeof(scl_O) == 4 && (N % 4u) == 0 && gn + 3 < N &&
          (((scl_u64)dst) & 15u) == 0) {
        scl_pack<scl_O, 4> o;
#pragma unroll
        for (int j = 0; j < 4; ++j) o.v[j] = acc[i][h * 4 + j];
        scl_store<scl_O, 4>(dst, o);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (gn + j < N) dst[j] = acc[i][h * 4 + j];
      }
    }
  }
}

#elif SCL_KIND == 13
extern "C" __global__ void __launch_bounds__(256)
scl_allpairs_generic(const SCL_TYPE_0* A, const SCL_TYPE_1* B, SCL_TYPE_2* P,
                     unsigned int dimension, unsigned int height, unsigned int width,
                     int staged SCL_EXTRA_PARAMS) {
  SCL_EXTRA_SETUP
  const unsigned int col = blockIdx.x * 16 + threadIdx.x;
  const unsigned int row = blockIdx.y * 16 + threadIdx.y;
  SCL_TYPE_0* As = reinterpret_cast<SCL_TYPE_0*>(scl_dyn_smem);
  SCL_TYPE_1* Bs = reinterpret_cast<SCL_TYPE_1*>(
      scl_dyn_smem + (((size_t)16 * dimension * sizeof(SCL_TYPE_0) + 15) & ~(size_t)15));
  lmatrix_t Mm;
  Mm.data = A;
  Mm.dimension = dimension;
  Mm.row = row;
  rmatrix_t Nm;
  Nm.data = B;
  Nm.width = width;
  Nm.column = col;
  if (staged) {
    const int t = threadIdx.y * 16 + threadIdx.x;
    const unsigned int r0 = blockIdx.y * 16, c0 = blockIdx.x * 16;
    for (unsigned int k = t; k < 16u * dimension; k += 256) {
      const unsigned int rr = k / dimension, kk = k % dimension;
      As[k] = (r0 + rr < height) ? A[(scl_u64)(r0 + rr) * dimension + kk] : (SCL_TYPE_0)0;
    }
    for (unsigned int k = t; k < 16u * dimension; k += 256) {
      const unsigned int kk = k / 16, cc = k % 16;
      Bs[k] = (c0 + cc < width) ? B[(scl_u64)kk * width + c0 + cc] : (SCL_TYPE_1)0;
    }
    __syncthreads();
    Mm.scl_row = As + (size_t)threadIdx.y * dimension;
    Nm.scl_col = Bs + threadIdx.x;
    Nm.scl_stride = 16;
  } else {
    Mm.scl_row = A + (scl_u64)row * dimension;
    Nm.scl_col = B + col;
    Nm.scl_stride = width;
  }
  if (row < height && col < width)
    P[(scl_u64)row * width + col] = USR_FUNC(&Mm, &Nm, dimension SCL_EXTRA_ARGS);
}
#endif
