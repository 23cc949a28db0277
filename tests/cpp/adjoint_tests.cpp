// The reverse-mode tape (include/SkelCL/Adjoint.h) on the GB300.  Every
// gradient is checked two ways: against FP64 central finite differences of a
// plain CPU forward written here, and against the same gradient composed from
// forward skeletons (Map, Zip, MapOverlap, AllPairs) by hand.
#include <cmath>
#include <cstdint>
#include <vector>

#include <gtest/gtest.h>

#include <SkelCL/Adjoint.h>
#include <SkelCL/AllPairs.h>
#include <SkelCL/IndexVector.h>
#include <SkelCL/Map.h>
#include <SkelCL/MapOverlap.h>
#include <SkelCL/Matrix.h>
#include <SkelCL/Reduce.h>
#include <SkelCL/Segments.h>
#include <SkelCL/SkelCL.h>
#include <SkelCL/Vector.h>
#include <SkelCL/Zip.h>

namespace {

class AdjointTest : public ::testing::Test {
protected:
  AdjointTest() { skelcl::init(skelcl::nDevices(1)); }
  ~AdjointTest() override { skelcl::terminate(); }
};

// SplitMix64 uniform in [a, b)
std::vector<float> uniform(size_t n, uint64_t seed, float a, float b) {
  std::vector<float> v(n);
  uint64_t s = seed;
  for (size_t i = 0; i < n; ++i) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    v[i] = (float)(a + (b - a) * ((double)(z >> 11) * 0x1.0p-53));
  }
  return v;
}

template <typename F>
double centralDifference(F loss, std::vector<float> x, size_t j) {
  const double h = 1e-3 * std::max(1.0, std::fabs((double)x[j]));
  const float x0 = x[j];
  x[j] = (float)(x0 + h);
  const double up = (double)x[j];
  const double lp = loss(x);
  x[j] = (float)(x0 - h);
  const double lm = loss(x);
  return (lp - lm) / (up - (double)x[j]);
}

const char* kAdd = "float func(float x, float y){ return x + y; }";
const char* kMul = "float func(float x, float y){ return x * y; }";

}  // namespace

// L = sum(inclusive_scan(Zip(*)(x*x+1, x))): x feeds two skeletons, so its
// gradient is the sum of two adjoint contributions.
TEST_F(AdjointTest, ChainMapZipScanReduce) {
  const size_t n = 50000;
  std::vector<float> xh = uniform(n, 2, -1.0f, 1.0f);
  skelcl::Vector<float> xs(xh.begin(), xh.end());
  skelcl::ad::Tape tape;
  auto x = tape.variable(xs);
  skelcl::ad::Map<float(float)> sq("float func(float x){ return x*x + 1.0f; }",
                                   "float dfunc(float x, float g){ return 2.0f*x*g; }");
  skelcl::ad::Zip<float(float, float)> mul(kMul, "float dl(float x, float y, float g){ return y*g; }\n"
                                                 "float dr(float x, float y, float g){ return x*g; }");
  skelcl::ad::Scan<float> scan(kAdd);
  scan.setInclusive(true);
  skelcl::ad::Reduce<float> sum(kAdd);
  auto loss = sum(tape, scan(tape, mul(tape, sq(tape, x), x)));
  EXPECT_EQ(tape.size(), 4u);
  tape.backward(loss);
  ASSERT_TRUE(x.hasGrad());
  std::vector<float> grad(x.grad().begin(), x.grad().end());

  // the same gradient composed from forward skeletons: dL/dz_j = n - j, then
  // dz_j/dx_j = 3 x_j^2 + 1
  skelcl::Map<float(skelcl::Index)> count("float func(Index i, unsigned int n){ return (float)(n - i); }");
  skelcl::Vector<float> gz = count(skelcl::IndexVector(n), (unsigned int)n);
  skelcl::Zip<float(float, float)> chain("float func(float x, float g){ return g * (3.0f*x*x + 1.0f); }");
  skelcl::Vector<float> composed = chain(xs, gz);

  auto forward = [n](const std::vector<float>& v) {  // FP64 forward
    double acc = 0.0, l = 0.0;
    for (size_t i = 0; i < n; ++i) {
      const double a = v[i];
      acc += (a * a + 1.0) * a;
      l += acc;
    }
    return l;
  };
  for (size_t j = 0; j < n; j += 997) {
    const double want = (double)(n - j) * (3.0 * xh[j] * xh[j] + 1.0);
    EXPECT_NEAR(grad[j], want, 1e-5 * std::fabs(want) + 1e-4);
    EXPECT_NEAR(grad[j], composed[j], 1e-6 * std::fabs(want) + 1e-4);
    EXPECT_NEAR(centralDifference(forward, xh, j), grad[j], 1e-3 * std::fabs(want) + 1e-2);
  }

  // gradients of variables add up across backward() calls; intermediates restart
  tape.backward(loss);
  for (size_t j = 0; j < n; j += 4999) EXPECT_NEAR(x.grad()[j], 2.0f * grad[j], 1e-6 * std::fabs(grad[j]));
}

// Segmented pipeline: many uneven vectors back to back (some empty, and a
// tail outside every vector), L = sum_s gr[s] * Reduce_s(Scan_s(x*x+1)).
TEST_F(AdjointTest, SegmentedMapScanReduce) {
  const size_t nseg = 300;
  std::vector<float> u = uniform(nseg, 12, 0.0f, 11.0f);
  std::vector<size_t> lens(nseg);
  for (size_t s = 0; s < nseg; ++s) lens[s] = s % 37 == 5 ? 0 : (size_t)std::floor(std::exp2((double)u[s]));
  std::vector<uint64_t> off(nseg + 1, 0);
  for (size_t s = 0; s < nseg; ++s) off[s + 1] = off[s] + lens[s];
  const size_t total = off[nseg], n = total + 777;  // 777 elements in no vector
  std::vector<float> xh = uniform(n, 13, -1.0f, 1.0f), grh = uniform(nseg, 14, -1.0f, 1.0f);
  skelcl::Vector<float> xs(xh.begin(), xh.end()), gr(grh.begin(), grh.end());
  skelcl::Segments segs(lens);
  skelcl::ad::Tape tape;
  auto x = tape.variable(xs);
  skelcl::ad::Map<float(float)> sq("float func(float x){ return x*x + 1.0f; }",
                                   "float dfunc(float x, float g){ return 2.0f*x*g; }");
  skelcl::ad::Scan<float> scan(kAdd);
  scan.setInclusive(true);
  skelcl::ad::Reduce<float> sum(kAdd);
  auto per = sum.segmented(tape, scan.segmented(tape, sq(tape, x), segs), segs);
  ASSERT_EQ(per.value().size(), nseg);
  tape.backward(per, gr);
  std::vector<float> grad(x.grad().begin(), x.grad().end());

  // the same gradient from forward skeletons: element i of vector s gets
  // gr[s] * (off[s+1] - i) * 2 x_i, found by a Map over indices
  skelcl::Vector<uint64_t> offv(off.begin(), off.end());
  skelcl::Map<float(skelcl::Index)> weight(
      "float func(Index i, __global const ulong* off, unsigned int ns, __global const float* gr) {"
      "  if (i >= off[ns]) return 0.0f;"
      "  unsigned int lo = 0, hi = ns - 1;"
      "  while (lo < hi) { unsigned int mid = (lo + hi + 1) / 2; if (off[mid] <= i) lo = mid; else hi = mid - 1; }"
      "  while (off[lo + 1] <= i) ++lo;"
      "  return gr[lo] * (float)(off[lo + 1] - i); }");
  skelcl::Vector<float> gz = weight(skelcl::IndexVector(n), offv, (unsigned int)nseg, gr);
  skelcl::Zip<float(float, float)> chain("float func(float x, float g){ return 2.0f * x * g; }");
  skelcl::Vector<float> composed = chain(xs, gz);

  auto forward = [&](const std::vector<float>& v) {  // FP64 forward
    double l = 0.0;
    for (size_t s = 0; s < nseg; ++s) {
      double acc = 0.0, red = 0.0;
      for (uint64_t i = off[s]; i < off[s + 1]; ++i) {
        acc += (double)v[i] * v[i] + 1.0;
        red += acc;
      }
      l += (double)grh[s] * red;
    }
    return l;
  };
  size_t seg = 0;
  for (size_t j = 0; j < n; j += 613) {
    while (seg < nseg && off[seg + 1] <= j) ++seg;
    const double want = j < total ? 2.0 * xh[j] * grh[seg] * (double)(off[seg + 1] - j) : 0.0;
    EXPECT_NEAR(grad[j], want, 1e-5 * std::fabs(want) + 1e-5);
    EXPECT_NEAR(grad[j], composed[j], 1e-6 * std::fabs(want) + 1e-5);
    EXPECT_NEAR(centralDifference(forward, xh, j), grad[j], 1e-3 * std::fabs(want) + 1e-3);
  }
  for (size_t j = total; j < n; ++j) EXPECT_EQ(grad[j], 0.0f);
}

TEST_F(AdjointTest, ConstantsGetNoGradient) {
  std::vector<float> a = uniform(1000, 3, -1.0f, 1.0f), b = uniform(1000, 4, -1.0f, 1.0f);
  skelcl::Vector<float> av(a.begin(), a.end()), bv(b.begin(), b.end());
  skelcl::ad::Tape tape;
  auto x = tape.variable(av);
  auto c = tape.constant(bv);
  skelcl::ad::Zip<float(float, float)> mul(kMul, "float dl(float x, float y, float g){ return y*g; }", "func",
                                           "dl", "");
  skelcl::ad::Reduce<float> sum(kAdd);
  auto loss = sum(tape, mul(tape, x, c));
  tape.backward(loss);
  EXPECT_FALSE(c.hasGrad());
  for (size_t j = 0; j < 1000; ++j) EXPECT_EQ(x.grad()[j], b[j]);
}

// L = sum(seed * stencil(img)) for the radius-5 Gaussian, both paddings.
static void stencilCase(skelcl::detail::Padding padding) {
  const size_t rows = 61, cols = 83, R = 5, W = 2 * R + 1;
  std::vector<float> img = uniform(rows * cols, 5, 0.0f, 255.0f);
  std::vector<float> seed = uniform(rows * cols, 6, -1.0f, 1.0f);
  std::vector<float> w(W * W);
  double total = 0.0;
  for (size_t i = 0; i < W * W; ++i) {
    const double dy = (double)(i / W) - R, dx = (double)(i % W) - R;
    w[i] = (float)std::exp(-(dx * dx + dy * dy) / 8.0);
    total += w[i];
  }
  for (float& v : w) v = (float)(v / total);
  const char* src =
      "float func(input_matrix_t img, __global float* w) { float s = 0.0f;"
      " for (int dy = -5; dy <= 5; ++dy) for (int dx = -5; dx <= 5; ++dx)"
      "  s += getData(img, dx, dy) * w[(dy + 5) * 11 + (dx + 5)]; return s; }";
  const bool nearest = padding == skelcl::detail::Padding::NEAREST;

  skelcl::Matrix<float> m(img, cols);
  skelcl::Vector<float> wv(w.begin(), w.end());
  skelcl::Matrix<float> sm(seed, cols);
  skelcl::ad::Tape tape;
  auto x = tape.variable(m);
  skelcl::ad::MapOverlap<float(float)> blur(src, 5, padding, 0.0f);
  auto out = blur(tape, x, wv);
  tape.backward(out, sm);
  const skelcl::Matrix<float>& g = x.grad();

  auto at = [&](const std::vector<float>& v, long y, long xx) -> double {
    if (nearest) {
      y = std::min(std::max(y, 0L), (long)rows - 1);
      xx = std::min(std::max(xx, 0L), (long)cols - 1);
    } else if (y < 0 || y >= (long)rows || xx < 0 || xx >= (long)cols) {
      return 0.0;
    }
    return v[(size_t)y * cols + (size_t)xx];
  };
  auto forward = [&](const std::vector<float>& v) {
    double l = 0.0;
    for (long y = 0; y < (long)rows; ++y)
      for (long xx = 0; xx < (long)cols; ++xx) {
        double s = 0.0;
        for (long dy = -5; dy <= 5; ++dy)
          for (long dx = -5; dx <= 5; ++dx) s += at(v, y + dy, xx + dx) * w[(dy + 5) * 11 + (dx + 5)];
        l += s * seed[(size_t)y * cols + (size_t)xx];
      }
    return l;
  };
  std::vector<size_t> check = {0, cols - 1, (rows - 1) * cols, rows * cols - 1, cols * 7, 3};
  for (size_t j = 11; j < rows * cols; j += 389) check.push_back(j);
  for (size_t j : check) {
    const double gj = g[j / cols][j % cols];
    EXPECT_NEAR(centralDifference(forward, img, j), gj, 1e-3 * std::max(1.0, std::fabs(gj)));
  }
  if (!nearest) {
    // composed: the zero-padded stencil with the flipped weights
    std::vector<float> flipped(W * W);
    for (size_t i = 0; i < W * W; ++i) flipped[i] = w[W * W - 1 - i];
    skelcl::Vector<float> fv(flipped.begin(), flipped.end());
    skelcl::MapOverlap<float(float)> t(src, 5, skelcl::detail::Padding::NEUTRAL, 0.0f);
    skelcl::Matrix<float> composed = t(sm, fv);
    for (size_t y = 0; y < rows; ++y)
      for (size_t xx = 0; xx < cols; ++xx) EXPECT_NEAR(g[y][xx], composed[y][xx], 1e-5);
  }
}

TEST_F(AdjointTest, MapOverlapNeutral) { stencilCase(skelcl::detail::Padding::NEUTRAL); }
TEST_F(AdjointTest, MapOverlapNearest) { stencilCase(skelcl::detail::Padding::NEAREST); }

// L = sum(G * (A B)): dA = G B^T, dB = A^T G.
static void allPairsCase(bool precise) {
  const size_t M = 130, K = 72, N = 200;
  std::vector<float> a = uniform(M * K, 7, -1.0f, 1.0f), b = uniform(K * N, 8, -1.0f, 1.0f),
                     gs = uniform(M * N, 9, -1.0f, 1.0f);
  skelcl::Matrix<float> A(a, K), B(b, N), G(gs, N);
  skelcl::Reduce<float(float)> add(kAdd);
  skelcl::Zip<float(float, float)> mul(kMul);
  skelcl::ad::AllPairs<float(float, float)> mm(add, mul);
  mm.setPrecise(precise);
  skelcl::ad::Tape tape;
  auto x = tape.variable(A);
  auto y = tape.variable(B);
  auto p = mm(tape, x, y);
  tape.backward(p, G);
  const skelcl::Matrix<float>& dA = x.grad();
  const skelcl::Matrix<float>& dB = y.grad();

  // composed: two forward AllPairs on host-transposed operands
  std::vector<float> bt(N * K), at(K * M);
  for (size_t k = 0; k < K; ++k)
    for (size_t j = 0; j < N; ++j) bt[j * K + k] = b[k * N + j];
  for (size_t i = 0; i < M; ++i)
    for (size_t k = 0; k < K; ++k) at[k * M + i] = a[i * K + k];
  skelcl::Matrix<float> Bt(bt, K), At(at, M);
  skelcl::AllPairs<float(float, float)> fwd(add, mul);
  skelcl::Matrix<float> cA = fwd(G, Bt), cB = fwd(At, G);

  auto lossA = [&](const std::vector<float>& v) {
    double l = 0.0;
    for (size_t i = 0; i < M; ++i)
      for (size_t j = 0; j < N; ++j) {
        double s = 0.0;
        for (size_t k = 0; k < K; ++k) s += (double)v[i * K + k] * b[k * N + j];
        l += s * gs[i * N + j];
      }
    return l;
  };
  auto lossB = [&](const std::vector<float>& v) {
    double l = 0.0;
    for (size_t i = 0; i < M; ++i)
      for (size_t j = 0; j < N; ++j) {
        double s = 0.0;
        for (size_t k = 0; k < K; ++k) s += (double)a[i * K + k] * v[k * N + j];
        l += s * gs[i * N + j];
      }
    return l;
  };
  for (size_t j = 0; j < M * K; j += 613) {
    const double g = dA[j / K][j % K];
    EXPECT_NEAR(centralDifference(lossA, a, j), g, 1e-3 * std::max(1.0, std::fabs(g)));
  }
  for (size_t j = 0; j < K * N; j += 701) {
    const double g = dB[j / N][j % N];
    EXPECT_NEAR(centralDifference(lossB, b, j), g, 1e-3 * std::max(1.0, std::fabs(g)));
  }
  for (size_t i = 0; i < M; ++i)
    for (size_t k = 0; k < K; ++k) EXPECT_NEAR(dA[i][k], cA[i][k], 1e-4);
  for (size_t k = 0; k < K; ++k)
    for (size_t j = 0; j < N; ++j) EXPECT_NEAR(dB[k][j], cB[k][j], 1e-4);
}

TEST_F(AdjointTest, AllPairsTensorCores) { allPairsCase(false); }
TEST_F(AdjointTest, AllPairsCudaCores) { allPairsCase(true); }

int main(int argc, char** argv) {
  ::testing::InitGoogleTest(&argc, argv);
  return RUN_ALL_TESTS();
}
