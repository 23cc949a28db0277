// Minimal binary PGM (P5, 8-bit) reading and writing for the examples.
#ifndef SKELCL_EXAMPLES_PGM_H_
#define SKELCL_EXAMPLES_PGM_H_

#include <cstdint>
#include <fstream>
#include <string>
#include <vector>

struct Pgm {
  size_t width = 0, height = 0;
  std::vector<float> pixels;  // row-major, 0..255
};

inline bool readPgm(const std::string& path, Pgm* img) {
  std::ifstream f(path, std::ios::binary);
  std::string magic;
  int maxval = 0;
  if (!(f >> magic) || magic != "P5") return false;
  auto skip = [&f] {
    f >> std::ws;
    while (f.peek() == '#') {
      std::string line;
      std::getline(f, line);
      f >> std::ws;
    }
  };
  skip();
  f >> img->width;
  skip();
  f >> img->height;
  skip();
  f >> maxval;
  f.get();
  if (!f || maxval <= 0 || maxval > 255) return false;
  std::vector<unsigned char> raw(img->width * img->height);
  f.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)raw.size());
  if (!f) return false;
  img->pixels.assign(raw.begin(), raw.end());
  return true;
}

inline bool writePgm(const std::string& path, size_t width, size_t height, const std::vector<float>& px) {
  std::ofstream f(path, std::ios::binary);
  f << "P5\n" << width << " " << height << "\n255\n";
  for (float v : px) {
    const float c = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
    f.put((char)(unsigned char)(c + 0.5f));
  }
  return (bool)f;
}

#endif  // SKELCL_EXAMPLES_PGM_H_
