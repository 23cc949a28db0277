/*
 * CPU oracle for the SkelCL skeleton path -- TEST INFRASTRUCTURE ONLY
 * (checker for tests/, __graft_entry__.smoke() and bench.py's cpu_baseline).
 * See oracle.h for what each function restates.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* generators                                                                */
/* ------------------------------------------------------------------------- */
uint64_t orc_splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static double u53(uint64_t* s) { return (double)(orc_splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

void orc_fill_uniform_f32(float* out, size_t n, uint64_t seed, double a, double b) {
  uint64_t s = seed;
  for (size_t i = 0; i < n; ++i) out[i] = (float)(a + (b - a) * u53(&s));
}

void orc_fill_mod_i32(int32_t* out, size_t n, uint64_t seed, uint32_t modulus) {
  uint64_t s = seed;
  for (size_t i = 0; i < n; ++i) out[i] = (int32_t)(orc_splitmix64(&s) % modulus);
}

void orc_fill_normal_f32(float* out, size_t n, uint64_t seed) {
  uint64_t s = seed;
  const double two_pi = 6.283185307179586476925286766559;
  for (size_t i = 0; i < n; i += 2) {
    double u1 = u53(&s), u2 = u53(&s);
    if (u1 < 1e-300) u1 = 1e-300;
    double r = sqrt(-2.0 * log(u1));
    out[i] = (float)(r * cos(two_pi * u2));
    if (i + 1 < n) out[i + 1] = (float)(r * sin(two_pi * u2));
  }
}

/* ------------------------------------------------------------------------- */
/* thread helper                                                             */
/* ------------------------------------------------------------------------- */
typedef void (*orc_range_fn)(void* ctx, size_t begin, size_t end, int tid);
typedef struct {
  orc_range_fn fn;
  void* ctx;
  size_t begin, end;
  int tid;
} orc_job;

static void* orc_job_run(void* p) {
  orc_job* j = (orc_job*)p;
  j->fn(j->ctx, j->begin, j->end, j->tid);
  return NULL;
}

static void orc_parallel(size_t n, int nthreads, orc_range_fn fn, void* ctx) {
  if (nthreads < 1) nthreads = 1;
  if ((size_t)nthreads > n) nthreads = n ? (int)n : 1;
  if (nthreads == 1) {
    fn(ctx, 0, n, 0);
    return;
  }
  pthread_t th[256];
  orc_job jobs[256];
  if (nthreads > 256) nthreads = 256;
  size_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    size_t b = (size_t)t * chunk, e = b + chunk;
    if (b > n) b = n;
    if (e > n) e = n;
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].begin = b;
    jobs[t].end = e;
    jobs[t].tid = t;
    pthread_create(&th[t], NULL, orc_job_run, &jobs[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------- */
/* Map / Zip (MapDef.h:187-195, ZipDef.h:197-206)                             */
/* ------------------------------------------------------------------------- */
void orc_zip_mul_f32(const float* x, const float* y, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) out[i] = x[i] * y[i];
}

typedef struct {
  const int32_t* in;
  int32_t* out;
  int32_t m;
} orc_mod_ctx;
static void orc_mod_range(void* c, size_t b, size_t e, int tid) {
  (void)tid;
  orc_mod_ctx* x = (orc_mod_ctx*)c;
  for (size_t i = b; i < e; ++i) x->out[i] = x->in[i] % x->m; /* C99 truncated modulo */
}
void orc_map_mod_i32(const int32_t* in, int32_t* out, size_t n, int32_t m, int nthreads) {
  orc_mod_ctx c = {in, out, m};
  orc_parallel(n, nthreads, orc_mod_range, &c);
}

void orc_map_sq1_f32(const float* in, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) out[i] = in[i] * in[i] + 1.0f;
}

/* ------------------------------------------------------------------------- */
/* Reduce (ReduceKernel.cl:51-128)                                           */
/* ------------------------------------------------------------------------- */
double orc_sum_f64(const float* x, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += (double)x[i];
  return s;
}

double orc_dot_f64(const float* x, const float* y, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += (double)x[i] * (double)y[i];
  return s;
}

int32_t orc_sum_i32(const int32_t* x, size_t n) {
  uint32_t s = 0;
  for (size_t i = 0; i < n; ++i) s += (uint32_t)x[i];
  return (int32_t)s;
}

float orc_sum_f32_reference_order(const float* x, size_t n, size_t global, size_t local) {
  if (n == 0) return 0.0f;
  size_t data = n < global ? n : global;
  float* tmp = (float*)malloc(data * sizeof(float));
  /* SCL_REDUCE_1: work-item p folds x[p], x[p+global], ... */
  for (size_t p = 0; p < data; ++p) {
    float r = x[p];
    for (size_t i = p + global; i < n; i += global) r = r + x[i];
    tmp[p] = r;
  }
  /* SCL_REDUCE_2: one work-group of min(data, local) items */
  size_t lsz = data < local ? data : local;
  float* buf = (float*)malloc(lsz * sizeof(float));
  for (size_t p = 0; p < lsz; ++p) {
    float r = tmp[p];
    for (size_t i = p + lsz; i < data; i += lsz) r = r + tmp[i];
    buf[p] = r;
  }
  size_t ds = lsz;
  while (ds > 1) {
    size_t modul = (ds + 1) / 2, active = ds / 2;
    for (size_t p = 0; p < active; ++p) buf[p] = buf[p] + buf[p + modul];
    ds = (ds + 1) / 2;
  }
  float r = buf[0];
  free(buf);
  free(tmp);
  return r;
}

/* ------------------------------------------------------------------------- */
/* Scan (ScanKernel.cl:74-250): exclusive, identity-seeded                   */
/* ------------------------------------------------------------------------- */
void orc_scan_excl_i32(const int32_t* in, int32_t* out, size_t n, int32_t id) {
  uint32_t acc = (uint32_t)id;
  for (size_t i = 0; i < n; ++i) {
    uint32_t v = (uint32_t)in[i];
    out[i] = (int32_t)acc;
    acc += v;
  }
}

void orc_scan_incl_i32(const int32_t* in, int32_t* out, size_t n) {
  uint32_t acc = 0;
  for (size_t i = 0; i < n; ++i) {
    acc += (uint32_t)in[i];
    out[i] = (int32_t)acc;
  }
}

typedef struct {
  const int32_t* in;
  int32_t* out;
  uint32_t* sums;
  size_t chunk;
  int32_t m;
  int pass;
} orc_scan_ctx;
static void orc_scan_range(void* c, size_t b, size_t e, int tid) {
  orc_scan_ctx* x = (orc_scan_ctx*)c;
  if (x->pass == 0) {
    uint32_t s = 0;
    for (size_t i = b; i < e; ++i) s += (uint32_t)x->in[i];
    x->sums[tid] = s;
  } else {
    uint32_t acc = x->sums[tid];
    if (x->m > 0) {
      for (size_t i = b; i < e; ++i) {
        acc += (uint32_t)x->in[i];
        x->out[i] = ((int32_t)acc) % x->m;
      }
    } else {
      for (size_t i = b; i < e; ++i) {
        acc += (uint32_t)x->in[i];
        x->out[i] = (int32_t)acc;
      }
    }
  }
}
static void orc_scan_mt(const int32_t* in, int32_t* out, size_t n, int32_t m, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  uint32_t sums[256];
  orc_scan_ctx c = {in, out, sums, 0, m, 0};
  orc_parallel(n, nthreads, orc_scan_range, &c);
  /* exclusive prefix of the chunk sums (same chunking as orc_parallel) */
  int used = (size_t)nthreads > n ? (n ? (int)n : 1) : nthreads;
  uint32_t run = 0;
  for (int t = 0; t < used; ++t) {
    uint32_t s = sums[t];
    sums[t] = run;
    run += s;
  }
  c.pass = 1;
  orc_parallel(n, nthreads, orc_scan_range, &c);
}
void orc_scan_incl_mod_i32_mt(const int32_t* in, int32_t* out, size_t n, int32_t m, int nthreads) {
  orc_scan_mt(in, out, n, m, nthreads);
}
void orc_scan_incl_i32_mt(const int32_t* in, int32_t* out, size_t n, int nthreads) {
  orc_scan_mt(in, out, n, 0, nthreads);
}

/* Scan with a non-commutative associative operator, folded strictly in
 * sequence order as f(earlier, later): composition of affine maps on
 * uint32 (wrapping), element i = the map x -> a_i*x + b_i stored as
 * {a_i, b_i}; f(p, q) = q after p = {q.a*p.a, q.a*p.b + q.b}; identity
 * {1, 0}.  Exclusive output i folds elements before i (identity first), as
 * ScanKernel.cl:74-196 seeds the exclusive scan with SCL_IDENTITY; with
 * `reverse`, "earlier" means a higher index.  The reference itself is only
 * well defined for commutative operators (ScanKernel.cl:135 and :243 call
 * f(later, earlier), :177 f(earlier, later)); this fixes the order the
 * GB300 kernels guarantee. */
void orc_scan_affine_u32(const uint32_t* in, uint32_t* out, size_t n, int inclusive, int reverse) {
  uint32_t a = 1u, b = 0u;
  for (size_t k = 0; k < n; ++k) {
    size_t i = reverse ? n - 1 - k : k;
    const uint32_t qa = in[2 * i], qb = in[2 * i + 1];
    if (!inclusive) {
      out[2 * i] = a;
      out[2 * i + 1] = b;
    }
    b = qa * b + qb;
    a = qa * a;
    if (inclusive) {
      out[2 * i] = a;
      out[2 * i + 1] = b;
    }
  }
}

void orc_scan_f64(const float* in, double* out, size_t n, int inclusive, int reverse) {
  double acc = 0.0;
  for (size_t k = 0; k < n; ++k) {
    size_t i = reverse ? n - 1 - k : k;
    if (inclusive) {
      acc += (double)in[i];
      out[i] = acc;
    } else {
      out[i] = acc;
      acc += (double)in[i];
    }
  }
}

/* ------------------------------------------------------------------------- */
/* MapOverlap (MapOverlapKernel.cl:59-148, OLDistributionDef.h:264-343)      */
/* ------------------------------------------------------------------------- */
typedef struct {
  const float* in;
  size_t rows, cols;
  int R;
  const float* w;
  int padding;
  double neutral;
  double* out;
} orc_st_ctx;

static long long orc_clampll(long long v, long long hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

static void orc_st_range(void* c, size_t b, size_t e, int tid) {
  (void)tid;
  orc_st_ctx* x = (orc_st_ctx*)c;
  const int R = x->R, W = 2 * R + 1;
  for (size_t y = b; y < e; ++y)
    for (size_t xx = 0; xx < x->cols; ++xx) {
      double s = 0.0;
      for (int dy = -R; dy <= R; ++dy)
        for (int dx = -R; dx <= R; ++dx) {
          long long gy = (long long)y + dy, gx = (long long)xx + dx;
          double v;
          if (gy >= 0 && gy < (long long)x->rows && gx >= 0 && gx < (long long)x->cols)
            v = x->in[(size_t)gy * x->cols + (size_t)gx];
          else if (x->padding == 1)
            v = x->in[(size_t)orc_clampll(gy, (long long)x->rows - 1) * x->cols +
                      (size_t)orc_clampll(gx, (long long)x->cols - 1)];
          else
            v = x->neutral;
          s += (double)x->w[(dy + R) * W + (dx + R)] * v;
        }
      x->out[y * x->cols + xx] = s;
    }
}
void orc_stencil_f64(const float* in, size_t rows, size_t cols, int R, const float* w,
                     int padding, double neutral, double* out, int nthreads) {
  orc_st_ctx c = {in, rows, cols, R, w, padding, neutral, out};
  orc_parallel(rows, nthreads, orc_st_range, &c);
}

/* positions p in [0,n) whose padded read at p+d lands on q: [*lo, *hi] (empty if lo > hi) */
static void orc_pre(long long q, long long d, long long n, int nearest, long long* lo, long long* hi) {
  if (!nearest) {
    long long p = q - d;
    *lo = p;
    *hi = p;
    if (p < 0 || p >= n) { *lo = 1; *hi = 0; }
    return;
  }
  if (n == 1) { *lo = 0; *hi = 0; return; }
  if (q == 0) {
    *lo = 0;
    *hi = -d < n - 1 ? -d : n - 1;
  } else if (q == n - 1) {
    *lo = n - 1 - d > 0 ? n - 1 - d : 0;
    *hi = n - 1;
  } else {
    long long p = q - d;
    *lo = p;
    *hi = p;
    if (p < 0 || p >= n) { *lo = 1; *hi = 0; }
  }
}

typedef struct {
  const float* g;
  size_t rows, cols;
  int R;
  const float* w;
  int padding;
  double* gin;
} orc_adj_ctx;
static void orc_adj_range(void* c, size_t b, size_t e, int tid) {
  (void)tid;
  orc_adj_ctx* x = (orc_adj_ctx*)c;
  const int R = x->R, W = 2 * R + 1;
  const int nearest = x->padding == 1;
  for (size_t qy = b; qy < e; ++qy)
    for (size_t qx = 0; qx < x->cols; ++qx) {
      double s = 0.0;
      for (int dy = -R; dy <= R; ++dy) {
        long long ylo, yhi;
        orc_pre((long long)qy, dy, (long long)x->rows, nearest, &ylo, &yhi);
        if (ylo > yhi) continue;
        for (int dx = -R; dx <= R; ++dx) {
          long long xlo, xhi;
          orc_pre((long long)qx, dx, (long long)x->cols, nearest, &xlo, &xhi);
          if (xlo > xhi) continue;
          double acc = 0.0;
          for (long long py = ylo; py <= yhi; ++py)
            for (long long px = xlo; px <= xhi; ++px) acc += (double)x->g[(size_t)py * x->cols + (size_t)px];
          s += (double)x->w[(dy + R) * W + (dx + R)] * acc;
        }
      }
      x->gin[qy * x->cols + qx] = s;
    }
}
void orc_stencil_adjoint_f64(const float* g_out, size_t rows, size_t cols, int R, const float* w,
                             int padding, double* g_in, int nthreads) {
  orc_adj_ctx c = {g_out, rows, cols, R, w, padding, g_in};
  orc_parallel(rows, nthreads, orc_adj_range, &c);
}

/* ------------------------------------------------------------------------- */
/* AllPairs (AllPairsKernel.cl:47-135, AllPairsKernel2.cl:42-65)              */
/* ------------------------------------------------------------------------- */
typedef struct {
  const float* A;
  const float* B;
  size_t M, N, K;
  double* Pd;
  float* Pf;
  int mode; /* 0 gemm f64, 1 gemm f32 sequential k, 2 manhattan f64 */
} orc_gemm_ctx;
static void orc_gemm_range(void* c, size_t b, size_t e, int tid) {
  (void)tid;
  orc_gemm_ctx* x = (orc_gemm_ctx*)c;
  const size_t N = x->N, K = x->K;
  if (x->mode == 1) {
    float* acc = (float*)malloc(N * sizeof(float));
    for (size_t i = b; i < e; ++i) {
      for (size_t j = 0; j < N; ++j) acc[j] = 0.0f;
      for (size_t k = 0; k < K; ++k) {
        const float a = x->A[i * K + k];
        const float* brow = x->B + k * N;
        for (size_t j = 0; j < N; ++j) acc[j] = acc[j] + a * brow[j];
      }
      memcpy(x->Pf + i * N, acc, N * sizeof(float));
    }
    free(acc);
    return;
  }
  double* acc = (double*)malloc(N * sizeof(double));
  for (size_t i = b; i < e; ++i) {
    for (size_t j = 0; j < N; ++j) acc[j] = 0.0;
    for (size_t k = 0; k < K; ++k) {
      const double a = x->A[i * K + k];
      const float* brow = x->B + k * N;
      if (x->mode == 0)
        for (size_t j = 0; j < N; ++j) acc[j] += a * (double)brow[j];
      else
        for (size_t j = 0; j < N; ++j) acc[j] += fabs(a - (double)brow[j]);
    }
    memcpy(x->Pd + i * N, acc, N * sizeof(double));
  }
  free(acc);
}
void orc_gemm_f64(const float* A, const float* B, size_t M, size_t N, size_t K, double* P,
                  int nthreads) {
  orc_gemm_ctx c = {A, B, M, N, K, P, NULL, 0};
  orc_parallel(M, nthreads, orc_gemm_range, &c);
}
void orc_gemm_f32_seq(const float* A, const float* B, size_t M, size_t N, size_t K, float* P,
                      int nthreads) {
  orc_gemm_ctx c = {A, B, M, N, K, NULL, P, 1};
  orc_parallel(M, nthreads, orc_gemm_range, &c);
}
void orc_manhattan_f64(const float* A, const float* B, size_t M, size_t N, size_t K, double* P,
                       int nthreads) {
  orc_gemm_ctx c = {A, B, M, N, K, P, NULL, 2};
  orc_parallel(M, nthreads, orc_gemm_range, &c);
}
