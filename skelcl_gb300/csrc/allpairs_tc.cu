// AllPairs zip(x*y) / reduce(x+y) over float on the 5th-generation tensor
// cores: P = A (M x K) * B (K x N), both row-major, FP32 in and out.
//
// Precision: "3xBF16" (Henry, Tang & Heinecke, "Leveraging the bfloat16
// Artificial Intelligence Datatype for Higher-Precision Computations",
// ARITH 2019).  Each FP32 operand is split into bf16 parts
//   x = hi + mid + lo (+ O(2^-24 |x|)),  hi = bf16(x), mid = bf16(x - hi),
//   lo = bf16(x - hi - mid)
// and the products whose magnitude can reach FP32 precision are accumulated
// in FP32 in tensor memory, smallest terms first:
//   kind 6: lo*hi + hi*lo + mid*mid + mid*hi + hi*mid + hi*hi   (3 parts)
//   kind 3: mid*hi + hi*mid + hi*hi                              (2 parts)
// The reference's semantics (AllPairsKernel.cl:47-135: P = sum over k of
// A[i][k]*B[k][j], identity 0) are kept; only the order of the FP32 sums
// differs from the sequential fold of the CUDA-core kernel.
//
// Shape: 128 x 128 output tile per CTA.  Warp 0 (one thread) streams k-blocks
// of 64 with TMA (3D tensor maps over the split parts, SWIZZLE_128B, one
// mbarrier per stage); warp 1 allocates 2 x 128 TMEM columns and one thread
// issues tcgen05.mma.kind::f16 (M=128, N=128, K=16; both operands K-major in
// shared memory), committing each stage back to the producer.  Each k-block
// is accumulated into one of two TMEM accumulators (ping-pong) and drained
// by warps 2-5 with tcgen05.ld into FP32 registers, where the k-block
// partials are summed with round-to-nearest adds.  Measured on GB300: letting
// the tensor core chain all 1536 MMAs of K = 4096 into one accumulator gave
// a normwise error of 2.6e-5 against FP64, growing about linearly with K (the
// accumulator's additions are not round-to-nearest); draining per k-block
// keeps each chain at 24 MMAs.  Every mbarrier wait is bounded; a wait that
// gives up raises the device status word and the CTA still frees its tensor
// memory before it returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace scl {
namespace tc {

constexpr int BM = 128;
constexpr int NPAD = 256;                        // N padding: fits both tile widths
constexpr int KPAD = 64;                         // K padding: whole k-blocks of both shapes

// Tile shape by output-tile width BN_T: 128 x 128 tiles take k-blocks of 64
// (one 128-byte SWIZZLE_128B row of bf16) with 4 epilogue warps; 128 x 256
// tiles take k-blocks of 32 (one 64-byte SWIZZLE_64B row, so that three
// stages of six parts fit in shared memory) with 8 epilogue warps, and read
// each A tile for twice as many columns.
template <int BN_T>
struct Shape {
  static constexpr int BN = BN_T;
  static constexpr int BK = BN_T == 256 ? 32 : 64;
  static constexpr int A_TILE = BM * BK * 2;     // bytes of one A part per stage
  static constexpr int B_TILE = BN * BK * 2;     // bytes of one B part per stage
  static constexpr int EPI_WARPS = BN / 32;      // each drains 32 rows x 128 columns
  static constexpr int THREADS = 64 + 32 * EPI_WARPS;
  static constexpr uint32_t TMEM_COLS = 2 * BN;  // two FP32 accumulators (ping-pong)
  static constexpr uint32_t SBO = 8 * BK * 2;    // bytes between 8-row groups
  static constexpr uint64_t LAYOUT = BK == 64 ? 2u : 4u;  // SWIZZLE_128B : SWIZZLE_64B
  // Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
  // (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
  // 17-22, M >> 4 in bits 24-28.
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) |
                                    ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
};

// Shared-memory matrix descriptor for a K-major swizzled tile (rows of BK
// bf16, 8-row groups SBO bytes apart): start address >> 4 (bits 0-13),
// leading-byte offset 1 (unused for swizzled K-major), stride-byte offset >> 4
// (bits 32-45), descriptor version 1 (bits 46-47), layout (bits 61-63).
template <int BN_T>
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  using SH = Shape<BN_T>;
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)(SH::SBO >> 4) << 32;
  d |= (uint64_t)1u << 46;
  d |= SH::LAYOUT << 61;
  return d;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;"
      " selp.u32 %0, 1, 0, p; }"
      : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
  return ok != 0;
}

// Bounded wait; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
  uint32_t polls = 0;
  while (!mbar_test(bar, parity)) {
    if (++polls > limit) return false;
    if (polls > 64) __nanosleep(32);
  }
  return true;
}

__device__ __forceinline__ void raise(unsigned int* err) {
  if (err) atomicOr(err, 1u);
}

// The split parts live in one [part][row][Kp] bf16 array per operand; rows and
// Kp are padded to the tile sizes and zero-filled, so every TMA box is in
// bounds.  Each thread splits 8 consecutive elements of a row and writes
// each part's 8 bf16 with one 16-byte store.
__device__ __forceinline__ void split8(const float (&x)[8], int parts, __nv_bfloat16* o0,
                                       __nv_bfloat16* o1, __nv_bfloat16* o2) {
  __align__(16) __nv_bfloat16 h[8], m[8], l[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    h[e] = __float2bfloat16_rn(x[e]);
    const float r1 = x[e] - __bfloat162float(h[e]);
    m[e] = __float2bfloat16_rn(r1);
    l[e] = __float2bfloat16_rn(r1 - __bfloat162float(m[e]));
  }
  *reinterpret_cast<uint4*>(o0) = *reinterpret_cast<const uint4*>(h);
  *reinterpret_cast<uint4*>(o1) = *reinterpret_cast<const uint4*>(m);
  if (parts > 2) *reinterpret_cast<uint4*>(o2) = *reinterpret_cast<const uint4*>(l);
}

// X (R x C row-major) -> parts of X ([part][Rp][Cp]): rows over blockIdx.y
// (grid-stride), 8-element chunks of a row over x.  Cp is a multiple of 64.
__global__ void __launch_bounds__(256) split_rows_kernel(const float* __restrict__ X, uint32_t R,
                                                         uint32_t C, uint32_t Rp, uint32_t Cp, int parts,
                                                         __nv_bfloat16* __restrict__ out) {
  const uint64_t plane = (uint64_t)Rp * Cp;
  const uint32_t chunks = Cp / 8;
  const bool vec = (C % 4u) == 0 && (reinterpret_cast<uintptr_t>(X) & 15u) == 0;
  for (uint32_t r = blockIdx.y; r < Rp; r += gridDim.y) {
    for (uint32_t ch = blockIdx.x * blockDim.x + threadIdx.x; ch < chunks; ch += gridDim.x * blockDim.x) {
      const uint32_t c0 = ch * 8;
      float x[8];
      if (r < R && vec && c0 + 8 <= C) {
        const float4 a = *reinterpret_cast<const float4*>(X + (uint64_t)r * C + c0);
        const float4 b = *reinterpret_cast<const float4*>(X + (uint64_t)r * C + c0 + 4);
        x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
        x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = (r < R && c0 + e < C) ? X[(uint64_t)r * C + c0 + e] : 0.0f;
      }
      const uint64_t o = (uint64_t)r * Cp + c0;
      split8(x, parts, out + o, out + plane + o, out + 2 * plane + o);
    }
  }
}

// B (K x N row-major) -> parts of B^T ([part][Np][Kp]) through 64 x 64 tiles
// in shared memory: coalesced row reads of B (16 bytes at a time when rows
// allow it), 16-byte stores of 8 consecutive k per part.  Np and Kp are
// multiples of 64.
__global__ void __launch_bounds__(256) split_transpose_kernel(const float* __restrict__ B, uint32_t K,
                                                              uint32_t N, uint32_t Np, uint32_t Kp,
                                                              int parts, __nv_bfloat16* __restrict__ out) {
  __shared__ float tile[64][65];  // [k][n]
  const uint32_t k0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const uint64_t plane = (uint64_t)Np * Kp;
  if ((N % 4u) == 0 && (reinterpret_cast<uintptr_t>(B) & 15u) == 0) {
    // 16-byte loads, four rows per thread in flight (a full row of 64 is 16
    // loads; n0 and N are multiples of 4, so a load is wholly in or out)
    const uint32_t c4 = threadIdx.x % 16, r0 = threadIdx.x / 16;
    float4 q[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint32_t k = k0 + r0 + 16 * i, n = n0 + c4 * 4;
      q[i] = (k < K && n < N) ? *reinterpret_cast<const float4*>(B + (uint64_t)k * N + n)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float* t = &tile[r0 + 16 * i][c4 * 4];
      t[0] = q[i].x;
      t[1] = q[i].y;
      t[2] = q[i].z;
      t[3] = q[i].w;
    }
  } else {
    for (int i = threadIdx.x; i < 64 * 64; i += 256) {
      const uint32_t kk = (uint32_t)i / 64, nn = (uint32_t)i % 64;
      const uint32_t k = k0 + kk, n = n0 + nn;
      tile[kk][nn] = (k < K && n < N) ? B[(uint64_t)k * N + n] : 0.0f;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 64 * 8; i += 256) {
    const uint32_t nn = (uint32_t)i / 8, kc = ((uint32_t)i % 8) * 8;
    const uint32_t n = n0 + nn, k = k0 + kc;
    if (n >= Np || k >= Kp) continue;
    float x[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) x[e] = tile[kc + e][nn];
    const uint64_t o = (uint64_t)n * Kp + k;
    split8(x, parts, out + o, out + plane + o, out + 2 * plane + o);
  }
}

// G = k-blocks accumulated in tensor memory between two drains into the
// epilogue's FP32 registers (1: every k-block; larger G drains less often at
// a longer in-TMEM accumulation chain).
//
// Output tiles are numbered in groups of `group_m` tile rows: block b of the
// 1D grid takes tile row first + (b mod group) mod rows and tile column
// (b mod group) div rows of its group, so consecutive blocks share one
// column of B's parts while cycling over a few rows of A's.  A wave of one
// block per SM then reads about group_m rows of A and SMs / group_m columns
// of B, which stay in L2 for the whole wave (row-major order read every
// column of B in every wave: at 4096^3, 2.5x the parts' bytes from DRAM).
template <int PARTS, int STAGES, int G, int BN_T>
__global__ void __launch_bounds__(Shape<BN_T>::THREADS, 1)
gemm_3xbf16_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   float* __restrict__ P, uint32_t M, uint32_t N, uint32_t Kp, uint32_t spin_limit,
                   unsigned int* err, uint32_t tiles_n, uint32_t group_m) {
  using SH = Shape<BN_T>;
  constexpr int BN = SH::BN, BK = SH::BK;
  constexpr int STAGE_BYTES = PARTS * (SH::A_TILE + SH::B_TILE);
  constexpr uint32_t TMEM_COLS = SH::TMEM_COLS;
  constexpr uint32_t IDESC = SH::IDESC;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t acc_full[2];   // MMA -> epilogue: k-block partial ready
  __shared__ __align__(8) uint64_t acc_empty[2];  // epilogue -> MMA: accumulator drained
  __shared__ __align__(8) uint64_t drain_bar;     // all issued MMAs have finished
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;  // 1024-aligned stage ring
  uint32_t n0, m0;
  {
    const uint32_t tiles_m = gridDim.x / tiles_n, per_group = group_m * tiles_n;
    const uint32_t grp = blockIdx.x / per_group, r = blockIdx.x % per_group;
    const uint32_t first = grp * group_m;
    const uint32_t rows = tiles_m - first < group_m ? tiles_m - first : group_m;
    m0 = (first + r % rows) * BM;
    n0 = (r / rows) * BN;
  }
  const uint32_t nk = Kp / BK;

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < STAGES; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&full_bar[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&empty_bar[s])));
    }
    for (int a = 0; a < 2; ++a) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&acc_full[a])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
                   :: "r"(smem_u32(&acc_empty[a])), "r"(SH::EPI_WARPS));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&drain_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" :: "l"(&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" :: "l"(&tmB) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(&tmem_slot)), "r"(TMEM_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ---- TMA producer
    if (lane == 0) {
      for (uint32_t kb = 0; kb < nk; ++kb) {
        const int s = (int)(kb % STAGES);
        const uint32_t round = kb / STAGES;
        if (round > 0 && !mbar_wait(smem_u32(&empty_bar[s]), (round - 1) & 1u, spin_limit)) {
          raise(err);
          s_fail = 1;
          break;
        }
        const uint32_t fb = smem_u32(&full_bar[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                     :: "r"(fb), "r"((uint32_t)STAGE_BYTES) : "memory");
        const uint32_t stage = base + (uint32_t)s * STAGE_BYTES;
        const int kx = (int)(kb * BK);
#pragma unroll
        for (int p = 0; p < PARTS; ++p) {
          asm volatile(
              "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
              " [%0], [%1, {%2, %3, %4}], [%5];"
              :: "r"(stage + (uint32_t)p * SH::A_TILE), "l"(&tmA), "r"(kx), "r"((int)m0), "r"(p),
                 "r"(fb)
              : "memory");
          asm volatile(
              "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
              " [%0], [%1, {%2, %3, %4}], [%5];"
              :: "r"(stage + (uint32_t)(PARTS * SH::A_TILE + p * SH::B_TILE)), "l"(&tmB), "r"(kx),
                 "r"((int)n0), "r"(p), "r"(fb)
              : "memory");
        }
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer
    if (lane == 0) {
      // (a part, b part) products, smallest first
      constexpr int NPROD = PARTS == 3 ? 6 : 3;
      int prod_a[NPROD], prod_b[NPROD];
      if (PARTS == 3) {  // lo*hi, hi*lo, mid*mid, mid*hi, hi*mid, hi*hi
        const int pa[6] = {2, 0, 1, 1, 0, 0}, pb[6] = {0, 2, 1, 0, 1, 0};
        for (int q = 0; q < NPROD; ++q) { prod_a[q] = pa[q]; prod_b[q] = pb[q]; }
      } else {           // mid*hi, hi*mid, hi*hi
        const int pa[3] = {1, 0, 0}, pb[3] = {0, 1, 0};
        for (int q = 0; q < NPROD; ++q) { prod_a[q] = pa[q]; prod_b[q] = pb[q]; }
      }
      for (uint32_t kb = 0; kb < nk; ++kb) {
        const int s = (int)(kb % STAGES);
        const uint32_t grp = kb / G;          // drain group of this k-block
        const bool first_in_grp = kb % G == 0;
        const bool last_in_grp = kb % G == G - 1 || kb + 1 == nk;
        const int acc_i = (int)(grp & 1u);
        const uint32_t use = grp >> 1;  // how often this accumulator was used before
        if (first_in_grp && use > 0 &&
            !mbar_wait(smem_u32(&acc_empty[acc_i]), (use - 1) & 1u, spin_limit)) {
          raise(err);
          s_fail = 1;
          break;
        }
        if (!mbar_wait(smem_u32(&full_bar[s]), (kb / STAGES) & 1u, spin_limit)) {
          raise(err);
          s_fail = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t stage = base + (uint32_t)s * STAGE_BYTES;
        const uint32_t dtm = tmem + (uint32_t)(acc_i * BN);
#pragma unroll
        for (int q = 0; q < NPROD; ++q) {
          const uint64_t ad = smem_desc<BN_T>(stage + (uint32_t)prod_a[q] * SH::A_TILE);
          const uint64_t bd =
              smem_desc<BN_T>(stage + (uint32_t)(PARTS * SH::A_TILE + prod_b[q] * SH::B_TILE));
#pragma unroll
          for (int ks = 0; ks < BK / 16; ++ks) {
            // advance 16 bf16 = 32 bytes along K inside the swizzle row
            const uint64_t a = ad + (uint64_t)(ks * 2);
            const uint64_t b = bd + (uint64_t)(ks * 2);
            const uint32_t acc = (!first_in_grp || q > 0 || ks > 0) ? 1u : 0u;  // fresh per group
            asm volatile(
                "{ .reg .pred p; setp.ne.b32 p, %4, 0;"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }"
                :: "r"(dtm), "l"(a), "l"(b), "r"(IDESC), "r"(acc)
                : "memory");
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
            :: "r"(smem_u32(&empty_bar[s])) : "memory");
        if (last_in_grp)
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
              :: "r"(smem_u32(&acc_full[acc_i])) : "memory");
      }
      // no MMA may still run when the tensor memory is freed (also after a
      // failed wait above)
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
          :: "r"(smem_u32(&drain_bar)) : "memory");
      if (!mbar_wait(smem_u32(&drain_bar), 0, spin_limit)) raise(err);
    }
  } else {
    // ---- epilogue: warp w (2 .. 1 + EPI_WARPS) owns TMEM lanes 32*(w % 4) ..
    //      and columns 128*((w - 2) / 4) ..; each thread keeps its row's 128
    //      partial sums in registers
    constexpr int CW = 128;  // columns per epilogue warp
    const int q = warp & 3;
    const int h = (warp - 2) >> 2;
    float sum[CW];
#pragma unroll
    for (int j = 0; j < CW; ++j) sum[j] = 0.0f;
    bool ok = true;
    const uint32_t ngrp = (nk + G - 1) / G;
    for (uint32_t grp = 0; grp < ngrp; ++grp) {
      const int acc_i = (int)(grp & 1u);
      if (!mbar_wait(smem_u32(&acc_full[acc_i]), (grp >> 1) & 1u, spin_limit)) {
        if (lane == 0) raise(err);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c = 0; c < CW / 32; ++c) {
        uint32_t r[32];
        const uint32_t taddr =
            tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc_i * BN + h * CW + c * 32);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10,"
            " %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27,"
            " %28, %29, %30, %31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
              "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
              "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
              "=r"(r[31])
            : "r"(taddr)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; ++j) sum[c * 32 + j] += __uint_as_float(r[j]);
      }
      // accumulator drained: hand it back to the MMA issuer (one arrive per warp)
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];"
                     :: "r"(smem_u32(&acc_empty[acc_i])) : "memory");
    }
    if (ok) {
      const uint32_t row = m0 + (uint32_t)(q * 32 + lane);
      if (row < M) {
        const bool vec = (N % 4u) == 0u;
#pragma unroll
        for (int c = 0; c < CW / 32; ++c) {
          const uint32_t col0 = n0 + (uint32_t)(h * CW + c * 32);
          float* dst = P + (uint64_t)row * N + col0;
          if (vec && col0 + 32 <= N) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(dst + j) =
                  make_float4(sum[c * 32 + j], sum[c * 32 + j + 1], sum[c * 32 + j + 2],
                              sum[c * 32 + j + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (col0 + j < N) dst[j] = sum[c * 32 + j];
          }
        }
      }
    }
  }

  // ---- teardown: wait for the copies a failed pipeline may still have in
  //      flight (bounded), then free the tensor memory
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (s_fail && threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_wait(smem_u32(&full_bar[s]), 0, spin_limit);
      mbar_wait(smem_u32(&full_bar[s]), 1, spin_limit);
    }
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

inline uint32_t round_up(uint32_t v, uint32_t m) { return (v + m - 1) / m * m; }

}  // namespace tc

size_t allpairs_tc_scratch_bytes(uint32_t M, uint32_t N, uint32_t K, int parts) {
  const uint64_t Mp = tc::round_up(M, tc::BM), Np = tc::round_up(N, tc::NPAD),
                 Kp = tc::round_up(K, tc::KPAD);
  return (size_t)parts * (Mp + Np) * Kp * 2 + 1024;
}

bool allpairs_tc_supported(uint32_t M, uint32_t N, uint32_t K, const void*, const void*,
                           const void*) {
  // the split arrays' row pitch (Kp * 2 bytes) and plane sizes stay far below
  // the tensor-map limits for any 32-bit shape; tiny products are not worth
  // the split
  return (uint64_t)M * N >= 128ull * 128ull && K >= 16 && rt().cc_major == 10;
}

static int encode_parts(CUtensorMap* tm, void* base, uint64_t rows, uint64_t Kp, int parts,
                        uint32_t box_rows, uint32_t box_k) {
  cuuint64_t dims[3] = {Kp, rows, (cuuint64_t)parts};
  cuuint64_t strides[2] = {Kp * 2, rows * Kp * 2};
  cuuint32_t box[3] = {box_k, box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = rt().drv.cuTensorMapEncodeTiled(
      tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
      CU_TENSOR_MAP_INTERLEAVE_NONE,
      box_k == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cu_fail(r, "cuTensorMapEncodeTiled(3xbf16 parts)");
  return SCL_OK;
}

namespace {
template <int PARTS, int STAGES, int G, int BN_T>
cudaError_t launch_gemm(dim3 grid, cudaStream_t stream, const CUtensorMap& tmA, const CUtensorMap& tmB,
                        float* P, uint32_t M, uint32_t N, uint32_t Kp, uint32_t spin_limit,
                        unsigned int* err, uint32_t tiles_n, uint32_t group_m) {
  using SH = tc::Shape<BN_T>;
  const size_t smem = (size_t)STAGES * PARTS * (SH::A_TILE + SH::B_TILE) + 1024;
  auto kern = tc::gemm_3xbf16_kernel<PARTS, STAGES, G, BN_T>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, SH::THREADS, smem, stream>>>(tmA, tmB, P, M, N, Kp, spin_limit, err, tiles_n, group_m);
  return cudaGetLastError();
}
}  // namespace

// The split pass: both operands into `parts` bf16 planes, K-major ([row][k]
// and [col][k]), zero-padded to Mp / Np / Kp, in `scratch` (1024-aligned
// inside it).  A transposed operand (trans bit 0: A stored K x M, bit 1: B
// stored N x K) swaps which of the two split kernels produces it.
void split_operands(const float* A, const float* B, uint32_t M, uint32_t N, uint32_t K, int parts,
                    int trans, void* scratch, cudaStream_t stream, __nv_bfloat16** a_out,
                    __nv_bfloat16** b_out) {
  const uint32_t Mp = tc::round_up(M, tc::BM), Np = tc::round_up(N, tc::NPAD),
                 Kp = tc::round_up(K, tc::KPAD);
  uint8_t* s = reinterpret_cast<uint8_t*>(((uintptr_t)scratch + 1023) & ~(uintptr_t)1023);
  __nv_bfloat16* a_parts = reinterpret_cast<__nv_bfloat16*>(s);
  __nv_bfloat16* b_parts = a_parts + (size_t)parts * Mp * Kp;
  auto rows_grid = [](uint32_t Rp, uint32_t Cp) {
    return dim3((Cp / 8 + 255) / 256, Rp < 65535u ? Rp : 65535u);
  };
  if (trans & 1) {
    tc::split_transpose_kernel<<<dim3(Mp / 64, Kp / 64), 256, 0, stream>>>(A, K, M, Mp, Kp, parts, a_parts);
  } else {
    tc::split_rows_kernel<<<rows_grid(Mp, Kp), 256, 0, stream>>>(A, M, K, Mp, Kp, parts, a_parts);
  }
  if (trans & 2) {
    tc::split_rows_kernel<<<rows_grid(Np, Kp), 256, 0, stream>>>(B, N, K, Np, Kp, parts, b_parts);
  } else {
    tc::split_transpose_kernel<<<dim3(Np / 64, Kp / 64), 256, 0, stream>>>(B, K, N, Np, Kp, parts, b_parts);
  }
  rt().launches += 2;
  *a_out = a_parts;
  *b_out = b_parts;
}

int allpairs_tc_launch(const float* A, const float* B, float* P, uint32_t M, uint32_t N,
                       uint32_t K, int parts, int trans, int drain, int wide, uint32_t group_rows,
                       void* scratch, size_t scratch_bytes, cudaStream_t stream, uint32_t spin_limit,
                       unsigned int* err) {
  if (parts != 2 && parts != 3) return fail(SCL_ERR_ARG, "3xBF16: parts must be 2 or 3");
  const uint32_t Mp = tc::round_up(M, tc::BM), Np = tc::round_up(N, tc::NPAD),
                 Kp = tc::round_up(K, tc::KPAD);
  if (scratch_bytes < allpairs_tc_scratch_bytes(M, N, K, parts))
    return fail(SCL_ERR_ARG, "3xBF16: scratch too small");
  __nv_bfloat16 *a_parts = nullptr, *b_parts = nullptr;
  split_operands(A, B, M, N, K, parts, trans, scratch, stream, &a_parts, &b_parts);

  alignas(64) CUtensorMap tmA, tmB;
  const uint32_t bn = wide ? 256 : 128, bk = wide ? 32 : 64;
  if (int st = encode_parts(&tmA, a_parts, Mp, Kp, parts, tc::BM, bk)) return st;
  if (int st = encode_parts(&tmB, b_parts, Np, Kp, parts, bn, bk)) return st;

  // one 1D grid over the output tiles, grouped by `group_m` tile rows; the
  // default is a group whose rows of A and columns of B for one wave of one
  // block per SM fit in L2 together
  const uint64_t tiles_n = (N + bn - 1) / bn, tiles_m = Mp / tc::BM;
  if (tiles_n * tiles_m > 0x7fffffffull) return fail(SCL_ERR_ARG, "3xBF16: too many output tiles");
  uint32_t group_m = group_rows;
  if (group_m == 0) group_m = 16;
  if (group_m > tiles_m) group_m = (uint32_t)tiles_m;
  dim3 grid((unsigned)(tiles_n * tiles_m));
  const uint32_t tn = (uint32_t)tiles_n;
  cudaError_t e;
  if (wide) {
    // 128 x 256 tiles, k-blocks of 32: drains every 2 k-blocks (64 K, as the
    // narrow shape's default); parts 3: 3 stages of 72 KB; parts 2: 4 of 48 KB
    e = parts == 3 ? launch_gemm<3, 3, 2, 256>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m)
                   : launch_gemm<2, 4, 2, 256>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m);
  } else if (parts == 3) {
    // parts 3: 2 stages of 96 KB; parts 2: 3 stages of 64 KB
    e = drain >= 4 ? launch_gemm<3, 2, 4, 128>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m)
      : drain == 2 ? launch_gemm<3, 2, 2, 128>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m)
                   : launch_gemm<3, 2, 1, 128>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m);
  } else {
    e = drain >= 4 ? launch_gemm<2, 3, 4, 128>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m)
      : drain == 2 ? launch_gemm<2, 3, 2, 128>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m)
                   : launch_gemm<2, 3, 1, 128>(grid, stream, tmA, tmB, P, M, N, Kp, spin_limit, err, tn, group_m);
  }
  if (e != cudaSuccess) return cuda_fail(e, "3xBF16 launch");
  rt().launches += 1;
  return SCL_OK;
}

}  // namespace scl

using namespace scl;

extern "C" int scl_debug_allpairs_split(const float* A, const float* B, uint32_t M, uint32_t N,
                                        uint32_t K, int parts, int trans, void* scratch,
                                        size_t scratch_bytes, size_t* needed) {
  if (parts != 2 && parts != 3) return fail(SCL_ERR_ARG, "split: parts must be 2 or 3");
  const size_t need = allpairs_tc_scratch_bytes(M, N, K, parts);
  if (needed) *needed = need;
  if (!scratch) return SCL_OK;
  if (int st = require_init()) return st;
  if (!A || !B || scratch_bytes < need) return fail(SCL_ERR_ARG, "split: null operand or scratch too small");
  __nv_bfloat16 *a = nullptr, *b = nullptr;
  split_operands(A, B, M, N, K, parts, trans, scratch, rt().stream, &a, &b);
  SCL_CUDA(cudaGetLastError());
  return SCL_OK;
}
