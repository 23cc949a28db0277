// Gaussian blur of a PGM image with MapOverlap (NEAREST padding); without an
// input file a synthetic image is blurred.  Writes <out>.pgm.
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include <pvsutil/CLArgParser.h>

#include <SkelCL/MapOverlap.h>
#include <SkelCL/Matrix.h>
#include <SkelCL/SkelCL.h>
#include <SkelCL/Vector.h>

#include "pgm.h"

int main(int argc, char** argv) {
  using namespace pvsutil::cmdline;
  pvsutil::CLArgParser cmd(Description("Gaussian blur of a PGM image."));
  auto range = Arg<int>(Flags(Short('r'), Long("range")), Description("Overlap radius."), Default(5));
  auto inFile = Arg<std::string>(Flags(Long("inFile")), Description("Input PGM (empty: synthetic)."),
                                 Default(std::string()));
  auto outFile = Arg<std::string>(Flags(Long("outFile")), Description("Output PGM."),
                                  Default(std::string("gauss_out.pgm")));
  auto check = Arg<bool>(Flags(Short('c'), Long("check")), Description("Compare with the host."), Default(false));
  cmd.add(range, inFile, outFile, check).parse(argc, argv);

  Pgm img;
  if (!std::string(inFile).empty()) {
    if (!readPgm(inFile, &img)) {
      std::cerr << "cannot read " << std::string(inFile) << "\n";
      return EXIT_FAILURE;
    }
  } else {
    img.width = 640;
    img.height = 480;
    for (size_t y = 0; y < img.height; ++y)
      for (size_t x = 0; x < img.width; ++x)
        img.pixels.push_back(((x / 32 + y / 32) % 2) ? 230.0f : 20.0f);
  }
  const int R = range, W = 2 * R + 1;
  std::vector<float> w(W * W);
  double total = 0.0;
  for (int i = 0; i < W * W; ++i) {
    const double dy = i / W - R, dx = i % W - R, s = R / 2.0 > 0 ? R / 2.0 : 1.0;
    w[i] = (float)std::exp(-(dx * dx + dy * dy) / (2 * s * s));
    total += w[i];
  }
  for (float& v : w) v = (float)(v / total);

  skelcl::init(skelcl::nDevices(1));
  const std::string R_ = std::to_string(R), W_ = std::to_string(W);
  skelcl::MapOverlap<float(float)> blur(
      "float func(input_matrix_t img, __global float* w) { float s = 0.0f;"
      " for (int dy = -" + R_ + "; dy <= " + R_ + "; ++dy)"
      "  for (int dx = -" + R_ + "; dx <= " + R_ + "; ++dx)"
      "   s += getData(img, dx, dy) * w[(dy + " + R_ + ") * " + W_ + " + dx + " + R_ + "];"
      " return s; }",
      (unsigned)R, skelcl::detail::Padding::NEAREST, 0.0f);
  skelcl::Matrix<float> m(img.pixels, img.width);
  skelcl::Vector<float> wv(w.begin(), w.end());
  skelcl::Matrix<float> out = blur(m, wv);
  std::vector<float> res(out.begin(), out.end());
  writePgm(outFile, img.width, img.height, res);
  std::cout << "wrote " << std::string(outFile) << " (" << img.width << "x" << img.height << ")\n";
  int rc = EXIT_SUCCESS;
  if (check) {
    double worst = 0.0;
    const long H = (long)img.height, Wd = (long)img.width;
    for (long y = 0; y < H; y += 7)
      for (long x = 0; x < Wd; x += 5) {
        double s = 0.0;
        for (long dy = -R; dy <= R; ++dy)
          for (long dx = -R; dx <= R; ++dx) {
            const long yy = std::min(std::max(y + dy, 0L), H - 1), xx = std::min(std::max(x + dx, 0L), Wd - 1);
            s += (double)img.pixels[yy * Wd + xx] * w[(dy + R) * W + dx + R];
          }
        worst = std::max(worst, std::fabs(s - res[y * Wd + x]));
      }
    const bool ok = worst <= 2e-3;
    std::cout << (ok ? "PASSED" : "FAILED") << " (max error " << worst << ")\n";
    rc = ok ? EXIT_SUCCESS : EXIT_FAILURE;
  }
  skelcl::terminate();
  return rc;
}
