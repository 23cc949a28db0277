// y = a*x + y with Zip and a scalar extra argument.
#include <cstdlib>
#include <iostream>

#include <pvsutil/CLArgParser.h>

#include <SkelCL/SkelCL.h>
#include <SkelCL/Vector.h>
#include <SkelCL/Zip.h>

int main(int argc, char** argv) {
  using namespace pvsutil::cmdline;
  pvsutil::CLArgParser cmd(Description("SAXPY: y = a * x + y."));
  auto size = Arg<int>(Flags(Short('n'), Long("size")), Description("Vector length."), Default(1 << 22));
  auto a = Arg<float>(Flags(Short('a'), Long("alpha")), Description("The scalar a."), Default(2.5f));
  auto check = Arg<bool>(Flags(Short('c'), Long("check")), Description("Compare with the host."), Default(false));
  cmd.add(size, a, check).parse(argc, argv);

  skelcl::init(skelcl::nDevices(1));
  skelcl::Vector<float> x(size), y(size);
  for (int i = 0; i < size; ++i) {
    x[i] = (float)(i % 1000) * 0.25f;
    y[i] = (float)(i % 7);
  }
  skelcl::Zip<float(float, float)> saxpy("float func(float x, float y, float a){ return a * x + y; }");
  skelcl::Vector<float> r = saxpy(x, y, (float)a);
  std::cout << "r[0..2] = " << r[0] << " " << r[1] << " " << r[2] << "\n";
  int rc = EXIT_SUCCESS;
  if (check) {
    bool ok = true;
    for (int i = 0; i < size; ++i) ok = ok && r[i] == (float)a * x[i] + y[i];
    std::cout << (ok ? "PASSED" : "FAILED") << "\n";
    rc = ok ? EXIT_SUCCESS : EXIT_FAILURE;
  }
  skelcl::terminate();
  return rc;
}
