// Matrix multiplication with AllPairs(Reduce(+), Zip(*)): on the tensor cores
// (3xBF16 split, FP32 accumulation) and, with --precise, on the CUDA cores.
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <random>
#include <vector>

#include <pvsutil/CLArgParser.h>
#include <pvsutil/Timer.h>

#include <SkelCL/AllPairs.h>
#include <SkelCL/Matrix.h>
#include <SkelCL/Reduce.h>
#include <SkelCL/SkelCL.h>
#include <SkelCL/Zip.h>

int main(int argc, char** argv) {
  using namespace pvsutil::cmdline;
  pvsutil::CLArgParser cmd(Description("C = A * B with AllPairs."));
  auto n = Arg<int>(Flags(Short('n'), Long("size")), Description("Rows of A = columns of B."), Default(1024));
  auto k = Arg<int>(Flags(Short('k'), Long("inner")), Description("Columns of A = rows of B."), Default(512));
  auto precise = Arg<bool>(Flags(Short('p'), Long("precise")), Description("CUDA cores only."), Default(false));
  auto check = Arg<bool>(Flags(Short('c'), Long("check")), Description("Compare with the host."), Default(false));
  cmd.add(n, k, precise, check).parse(argc, argv);

  skelcl::init(skelcl::nDevices(1));
  std::mt19937 rng(2);
  std::normal_distribution<float> g(0.0f, 1.0f);
  std::vector<float> a((size_t)n * k), b((size_t)k * n);
  for (float& v : a) v = g(rng);
  for (float& v : b) v = g(rng);
  skelcl::Matrix<float> A(a, (size_t)k), B(b, (size_t)n);
  skelcl::Reduce<float(float)> sum("float func(float x, float y){ return x + y; }", "0");
  skelcl::Zip<float(float, float)> mult("float func(float x, float y){ return x * y; }");
  skelcl::AllPairs<float(float, float)> mm(sum, mult);
  mm.setPrecise(precise);
  pvsutil::Timer t;
  skelcl::Matrix<float> C = mm(A, B);
  const float c00 = C[0][0];
  std::cout << "C[0][0] = " << c00 << ", " << t.stop() << " ms ("
            << (mm.lastVariant() == SCL_VARIANT_TC3XBF16 ? "tensor cores" : "CUDA cores") << ")\n";
  int rc = EXIT_SUCCESS;
  if (check) {
    double worst = 0.0, scale = 0.0;
    for (int i = 0; i < n; i += 37)
      for (int j = 0; j < n; j += 41) {
        double s = 0.0;
        for (int q = 0; q < k; ++q) s += (double)a[(size_t)i * k + q] * b[(size_t)q * n + j];
        worst = std::max(worst, std::fabs(s - C[i][j]));
        scale = std::max(scale, std::fabs(s));
      }
    const bool ok = worst <= 1e-5 * std::max(1.0, scale);
    std::cout << (ok ? "PASSED" : "FAILED") << " (normwise error " << worst / std::max(1.0, scale) << ")\n";
    rc = ok ? EXIT_SUCCESS : EXIT_FAILURE;
  }
  skelcl::terminate();
  return rc;
}
