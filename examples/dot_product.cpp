// Dot product of two random vectors: Zip(mult) then Reduce(add), and the
// fused ZipReduce, checked against a double-precision host loop.
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <random>

#include <pvsutil/CLArgParser.h>
#include <pvsutil/Logger.h>
#include <pvsutil/Timer.h>

#include <SkelCL/Fused.h>
#include <SkelCL/Reduce.h>
#include <SkelCL/SkelCL.h>
#include <SkelCL/Vector.h>
#include <SkelCL/Zip.h>

int main(int argc, char** argv) {
  using namespace pvsutil::cmdline;
  pvsutil::CLArgParser cmd(Description("Dot product of two random vectors."));
  auto size = Arg<int>(Flags(Short('n'), Long("size")), Description("Vector length."), Default(1 << 24));
  auto check = Arg<bool>(Flags(Short('c'), Long("check")), Description("Compare with the host."), Default(false));
  cmd.add(size, check).parse(argc, argv);

  skelcl::init(skelcl::nDevices(1));
  std::mt19937 rng(1);
  std::uniform_real_distribution<float> u(-1.0f, 1.0f);
  skelcl::Vector<float> x(size), y(size);
  for (int i = 0; i < size; ++i) {
    x[i] = u(rng);
    y[i] = u(rng);
  }
  skelcl::Zip<float(float, float)> mult("float func(float x, float y){ return x * y; }");
  skelcl::Reduce<float(float)> sum("float func(float x, float y){ return x + y; }", "0");
  skelcl::ZipReduce<float(float, float)> dot(sum, mult);

  pvsutil::Timer t;
  const float twoStep = sum(mult(x, y)).front();
  const float fused = dot(x, y).front();
  std::cout << "dot = " << twoStep << " (zip+reduce), " << fused << " (fused), " << t.stop() << " ms\n";
  int rc = EXIT_SUCCESS;
  if (check) {
    double want = 0.0;
    for (int i = 0; i < size; ++i) want += (double)x[i] * y[i];
    const double tol = 1e-5 * std::max(1.0, std::fabs(want));
    const bool ok = std::fabs(twoStep - want) <= tol && std::fabs(fused - want) <= tol;
    std::cout << (ok ? "PASSED" : "FAILED") << " (host " << want << ")\n";
    rc = ok ? EXIT_SUCCESS : EXIT_FAILURE;
  }
  skelcl::terminate();
  return rc;
}
