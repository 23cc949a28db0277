// The extensions of the drop-in C++ API on the GB300: segmented Scan and
// Reduce over vectors stored back to back, CUDA-graph replay of a skeleton
// sequence, and autotuned launches -- each against plain host loops.
#include <cstdint>
#include <vector>

#include <gtest/gtest.h>

#include <SkelCL/Fused.h>
#include <SkelCL/Graph.h>
#include <SkelCL/Map.h>
#include <SkelCL/Reduce.h>
#include <SkelCL/Scan.h>
#include <SkelCL/Segments.h>
#include <SkelCL/SkelCL.h>
#include <SkelCL/Vector.h>
#include <SkelCL/Zip.h>

class ExtensionsTest : public ::testing::Test {
protected:
  ExtensionsTest() { skelcl::init(skelcl::nDevices(1)); }
  ~ExtensionsTest() override { skelcl::terminate(); }
};

static std::vector<size_t> lengths() {
  std::vector<size_t> l;
  uint64_t s = 12345;
  for (int i = 0; i < 700; ++i) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    l.push_back((size_t)((s >> 33) % 40000));  // 0 .. 39999 elements
  }
  return l;
}

TEST_F(ExtensionsTest, SegmentedScanAndReduce) {
  const std::vector<size_t> len = lengths();
  skelcl::Segments segs(len);
  std::vector<int> host(segs.total());
  for (size_t i = 0; i < host.size(); ++i) host[i] = (int)(i % 1001) - 500;
  skelcl::Vector<int> v(host.begin(), host.end());
  skelcl::Scan<int(int)> scan("int func(int x, int y){ return x + y; }");
  skelcl::Reduce<int(int)> sum("int func(int x, int y){ return x + y; }");
  skelcl::Vector<int> s = scan.segmented(v, segs);
  skelcl::Vector<int> r = sum.segmented(v, segs);
  ASSERT_EQ(r.size(), len.size());
  size_t off = 0;
  for (size_t k = 0; k < len.size(); ++k) {
    long long acc = 0;
    for (size_t i = 0; i < len[k]; ++i) {
      EXPECT_EQ(s[off + i], (int)acc);  // exclusive, restarting at every vector
      acc += host[off + i];
    }
    EXPECT_EQ(r[k], (int)acc);
    off += len[k];
  }
}

TEST_F(ExtensionsTest, GraphReplaysDotProduct) {
  const size_t n = 1 << 20;
  skelcl::Vector<float> x(n, 1.0f), y(n, 2.0f), z(n);
  skelcl::Vector<float> r(1);
  skelcl::Zip<float(float, float)> mul("float func(float x, float y){ return x * y; }");
  skelcl::Reduce<float(float)> sum("float func(float x, float y){ return x + y; }");
  skelcl::Graph g;
  g.capture([&] {
    mul(skelcl::out(z), x, y);
    sum(skelcl::out(r), z);
  });
  EXPECT_EQ(r[0], 2.0f * n);
  for (int rep = 1; rep <= 3; ++rep) {
    for (size_t i = 0; i < n; ++i) x[i] = (float)rep;  // new contents, same buffers
    x.dataOnHostModified();
    x.copyDataToDevices();
    g.launch();
    g.wait();
    r.dataOnDeviceModified();
    EXPECT_EQ(r[0], 2.0f * rep * n);
  }
}

TEST_F(ExtensionsTest, AutotunedMapGivesTheSameResult) {
  skelcl::setAutotune(true);
  const size_t n = (1 << 21) + 7;
  std::vector<int> host(n);
  for (size_t i = 0; i < n; ++i) host[i] = (int)(i * 7 % 1000);
  skelcl::Vector<int> v(host.begin(), host.end());
  skelcl::Map<int(int)> m("int func(int x){ return x * 3 + 1; }");
  skelcl::Vector<int> a = m(v);
  skelcl::Vector<int> b = m(v);  // from the tuning cache
  skelcl::setAutotune(false);
  for (size_t i = 0; i < n; i += 997) {
    EXPECT_EQ(a[i], host[i] * 3 + 1);
    EXPECT_EQ(b[i], host[i] * 3 + 1);
  }
}

TEST_F(ExtensionsTest, FusedPairsEqualUnfused) {
  const size_t n = (1 << 20) + 3;
  std::vector<int> a(n), b(n);
  for (size_t i = 0; i < n; ++i) {
    a[i] = (int)(i % 97) - 48;
    b[i] = (int)(i % 13) - 6;
  }
  skelcl::Vector<int> x(a.begin(), a.end()), y(b.begin(), b.end());
  skelcl::Reduce<int(int)> sum("int func(int x, int y){ return x + y; }");
  skelcl::Zip<int(int, int)> mul("int func(int x, int y){ return x * y; }");
  skelcl::ZipReduce<int(int, int)> dot(sum, mul);
  skelcl::Vector<int> d = dot(x, y);
  long long want = 0;
  for (size_t i = 0; i < n; ++i) want += (long long)a[i] * b[i];
  EXPECT_EQ(d[0], (int)want);

  skelcl::Scan<int(int)> scan("int func(int x, int y){ return x + y; }");
  scan.setInclusive(true);
  skelcl::Map<int(int)> mod("int func(int x){ return x % 7919; }");
  skelcl::ScanMap<int(int)> fused(scan, mod);
  skelcl::Vector<int> f = fused(x);
  skelcl::Vector<int> u = mod(scan(x));
  for (size_t i = 0; i < n; i += 101) EXPECT_EQ(f[i], u[i]);
}

int main(int argc, char** argv) {
  ::testing::InitGoogleTest(&argc, argv);
  return RUN_ALL_TESTS();
}
