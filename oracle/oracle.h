/*
 * CPU oracle for the SkelCL skeleton path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of what the reference's skeleton kernels compute,
 * used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as
 * the checker.  Nothing in the product (libskelcl_cuda.so, include/SkelCL)
 * calls it.  Each function names the reference code it restates.
 *
 * Pinned against the reference's own known answers (test/*.cpp of the
 * reference, collected in tests/golden/reference_kats.json).
 */
#ifndef SKELCL_ORACLE_H_
#define SKELCL_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- seeded generators (project-defined SplitMix64) ---------------------- */
uint64_t orc_splitmix64(uint64_t* state);
/* uniform [a, b): a + (b - a) * (u >> 11) * 2^-53, rounded to float */
void orc_fill_uniform_f32(float* out, size_t n, uint64_t seed, double a, double b);
/* integers u % modulus */
void orc_fill_mod_i32(int32_t* out, size_t n, uint64_t seed, uint32_t modulus);
/* N(0,1) by Box-Muller in double, rounded to float */
void orc_fill_normal_f32(float* out, size_t n, uint64_t seed);

/* ---- Zip / Map --------------------------------------------------------- */
void orc_zip_mul_f32(const float* x, const float* y, float* out, size_t n);
void orc_map_mod_i32(const int32_t* in, int32_t* out, size_t n, int32_t m, int nthreads);
void orc_map_sq1_f32(const float* in, float* out, size_t n); /* x*x+1 */

/* ---- Reduce ----------------------------------------------------------- */
double orc_sum_f64(const float* x, size_t n);
double orc_dot_f64(const float* x, const float* y, size_t n);
int32_t orc_sum_i32(const int32_t* x, size_t n); /* two's-complement wrap */
/* The reference's float summation order: SCL_REDUCE_1 with `global` work-items
 * folding x[j], x[j+global], ... then SCL_REDUCE_2 with `local` work-items and
 * the ceil-halving tree (include/SkelCL/detail/ReduceKernel.cl:51-128). */
float orc_sum_f32_reference_order(const float* x, size_t n, size_t global, size_t local);

/* ---- Scan -------------------------------------------------------------- */
/* exclusive scan seeded with `id`, wrapping int32 add
 * (include/SkelCL/detail/ScanKernel.cl:74-250) */
void orc_scan_excl_i32(const int32_t* in, int32_t* out, size_t n, int32_t id);
void orc_scan_incl_i32(const int32_t* in, int32_t* out, size_t n);
/* multithreaded inclusive int32 scan + map(x mod m) fused, the CPU baseline
 * for the integer scan workload */
void orc_scan_incl_mod_i32_mt(const int32_t* in, int32_t* out, size_t n, int32_t m, int nthreads);
void orc_scan_incl_i32_mt(const int32_t* in, int32_t* out, size_t n, int nthreads);
/* ordered scan of a non-commutative operator: affine-map composition on
 * uint32 pairs {a, b}, f(earlier, later), identity {1, 0} */
void orc_scan_affine_u32(const uint32_t* in, uint32_t* out, size_t n, int inclusive, int reverse);
/* double-precision scans of float input; reverse = from the last element */
void orc_scan_f64(const float* in, double* out, size_t n, int inclusive, int reverse);

/* ---- MapOverlap -------------------------------------------------------- */
/* out[y][x] = sum_{dy,dx in [-R,R]} w[(dy+R)*(2R+1)+(dx+R)] * in'[y+dy][x+dx]
 * in' = NEAREST clamp (padding 1) or constant `neutral` (padding 0)
 * (include/SkelCL/detail/MapOverlapKernel.cl:59-148 +
 *  OLDistributionDef.h:264-343), accumulated in double. */
void orc_stencil_f64(const float* in, size_t rows, size_t cols, int R, const float* w,
                     int padding, double neutral, double* out, int nthreads);
/* adjoint of the same stencil: g_in[q] = sum_p sum_o w[o] g_out[p] [in'(p+o) = q] */
void orc_stencil_adjoint_f64(const float* g_out, size_t rows, size_t cols, int R, const float* w,
                             int padding, double* g_in, int nthreads);

/* ---- AllPairs ---------------------------------------------------------- */
/* P = A (M x K) * B (K x N), row-major, accumulated in double */
void orc_gemm_f64(const float* A, const float* B, size_t M, size_t N, size_t K, double* P,
                  int nthreads);
/* P = A * B in float, k folded strictly in order (AllPairsKernel.cl:89-91) */
void orc_gemm_f32_seq(const float* A, const float* B, size_t M, size_t N, size_t K, float* P,
                      int nthreads);
/* P[i][j] = sum_k |A[i][k] - B[k][j]| in double */
void orc_manhattan_f64(const float* A, const float* B, size_t M, size_t N, size_t K, double* P,
                       int nthreads);

#ifdef __cplusplus
}
#endif

#endif /* SKELCL_ORACLE_H_ */
