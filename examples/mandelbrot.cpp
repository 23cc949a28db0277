// Mandelbrot set with Map<IndexPoint> into an IndexMatrix; writes a PGM.
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include <pvsutil/CLArgParser.h>

#include <SkelCL/IndexMatrix.h>
#include <SkelCL/Map.h>
#include <SkelCL/SkelCL.h>

#include "pgm.h"

int main(int argc, char** argv) {
  using namespace pvsutil::cmdline;
  pvsutil::CLArgParser cmd(Description("Mandelbrot set, written as a PGM image."));
  auto width = Arg<int>(Flags(Short('w'), Long("width")), Description("Image width."), Default(1024));
  auto height = Arg<int>(Flags(Short('h'), Long("height")), Description("Image height."), Default(768));
  auto iters = Arg<int>(Flags(Short('i'), Long("iterations")), Description("Iteration limit."), Default(256));
  auto outFile = Arg<std::string>(Flags(Long("outFile")), Description("Output PGM."),
                                  Default(std::string("mandelbrot.pgm")));
  auto check = Arg<bool>(Flags(Short('c'), Long("check")), Description("Compare with the host."), Default(false));
  cmd.add(width, height, iters, outFile, check).parse(argc, argv);

  skelcl::init(skelcl::nDevices(1));
  skelcl::Map<float(skelcl::IndexPoint)> m(
      "float func(IndexPoint p, int w, int h, int limit) {"
      "  float cr = -2.0f + 3.0f * p.x / w, ci = -1.2f + 2.4f * p.y / h;"
      "  float zr = 0.0f, zi = 0.0f; int k = 0;"
      "  while (k < limit && zr * zr + zi * zi < 4.0f) {"
      "    float t = zr * zr - zi * zi + cr; zi = 2.0f * zr * zi + ci; zr = t; ++k; }"
      "  return 255.0f * k / limit; }");
  skelcl::IndexMatrix idx(skelcl::MatrixSize((size_t)(int)height, (size_t)(int)width));
  skelcl::Matrix<float> img = m(idx, (int)width, (int)height, (int)iters);
  std::vector<float> px(img.begin(), img.end());
  writePgm(outFile, width, height, px);
  std::cout << "wrote " << std::string(outFile) << "\n";
  int rc = EXIT_SUCCESS;
  if (check) {
    size_t bad = 0, checked = 0;
    for (int y = 0; y < height; y += 13)
      for (int x = 0; x < width; x += 11) {
        const float cr = -2.0f + 3.0f * x / width, ci = -1.2f + 2.4f * y / height;
        float zr = 0.0f, zi = 0.0f;
        int k = 0;
        while (k < iters && zr * zr + zi * zi < 4.0f) {
          const float t = zr * zr - zi * zi + cr;
          zi = 2.0f * zr * zi + ci;
          zr = t;
          ++k;
        }
        ++checked;
        // escape counts may differ by rounding near the boundary
        if (std::abs(px[(size_t)y * width + x] - 255.0f * k / iters) > 255.0f * 2 / iters) ++bad;
      }
    const bool ok = bad * 100 <= checked;
    std::cout << (ok ? "PASSED" : "FAILED") << " (" << bad << " of " << checked << " points differ)\n";
    rc = ok ? EXIT_SUCCESS : EXIT_FAILURE;
  }
  skelcl::terminate();
  return rc;
}
