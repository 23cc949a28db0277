// Known-answer tests of the SkelCL C++ API on the GB300, written against the
// drop-in headers in include/SkelCL.  The cases, user functions and expected
// values follow the reference's own gtest suites (test/MapTests.cpp,
// ZipTests.cpp, ReduceTests.cpp, ScanTests.cpp, MapOverlapTests.cpp,
// AllPairsTests.cpp, IndexVectorTests.cpp, IndexMatrixTests.cpp,
// SHA1Tests.cpp); each test names the case it restates.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include <gtest/gtest.h>

#include <SkelCL/AllPairs.h>
#include <SkelCL/Distributions.h>
#include <SkelCL/IndexMatrix.h>
#include <SkelCL/IndexVector.h>
#include <SkelCL/Map.h>
#include <SkelCL/MapOverlap.h>
#include <SkelCL/Matrix.h>
#include <SkelCL/Reduce.h>
#include <SkelCL/Scan.h>
#include <SkelCL/SkelCL.h>
#include <SkelCL/Vector.h>
#include <SkelCL/Zip.h>
#include <SkelCL/detail/Util.h>

class SkelCLTest : public ::testing::Test {
protected:
  SkelCLTest() { skelcl::init(skelcl::nDevices(1)); }
  ~SkelCLTest() override { skelcl::terminate(); }
};

// ---- Map (test/MapTests.cpp) ----------------------------------------------------
TEST_F(SkelCLTest, MapCreateWithFile) {  // MapTests.cpp:69-95
  const char* fn = "skelcl_test_function.cl";
  { std::ofstream f(fn, std::ios_base::trunc); f << "float func(float f) { return -f; }"; }
  skelcl::Map<float(float)> m{std::ifstream{fn}};
  std::remove(fn);
  skelcl::Vector<float> in(3, 2.0f);
  skelcl::Vector<float> out = m(in);
  EXPECT_EQ(-2.0f, out[2]);
}

TEST_F(SkelCLTest, SimpleMap) {  // MapTests.cpp:96-111
  skelcl::Map<float(float)> m{"float func(float f){ return -f; }"};
  skelcl::Vector<float> input(10);
  for (size_t i = 0; i < input.size(); ++i) input[i] = i * 2.5f;
  skelcl::Vector<float> output = m(input);
  EXPECT_EQ(10u, output.size());
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(-input[i], output[i]);
}

TEST_F(SkelCLTest, MapOutAndDeviceId) {  // MapTests.cpp:113-156 (one device)
  skelcl::Map<int(float)> m{"int func(float f) { return skelcl_get_device_id(); }"};
  skelcl::Vector<float> input(10);
  skelcl::Vector<int> output(input.size());
  m(skelcl::out(output), input);
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(0, output[i]);
  EXPECT_EQ(1u, skelcl::detail::globalDeviceList.size());
}

TEST_F(SkelCLTest, MapAddArgs) {  // MapTests.cpp:158-177
  skelcl::Map<float(float)> m{"float func(float f, float add, float add2) { return f+add+add2; }"};
  skelcl::Vector<float> input(10);
  for (size_t i = 0; i < input.size(); ++i) input[i] = i * 2.5f;
  float add = 5.25f, add2 = 7.75f;
  skelcl::Vector<float> output = m(input, add, add2);
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(input[i] + add + add2, output[i]);
}

TEST_F(SkelCLTest, MapVoid) {  // MapTests.cpp:179-195
  skelcl::Map<void(float)> m{"void func(float f, __global float* out) { out[get_global_id(0)] = f; }"};
  skelcl::Vector<float> input(10);
  for (size_t i = 0; i < input.size(); ++i) input[i] = i * 2.5f;
  skelcl::Vector<float> output(10);
  m(input, skelcl::out(output));
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(input[i], output[i]);
}

TEST_F(SkelCLTest, SimpleMap2D) {  // MapTests.cpp:225-246
  skelcl::Map<float(float)> m("float func(float f){ return -f; }");
  std::vector<float> vec(10);
  for (size_t i = 0; i < vec.size(); ++i) vec[i] = static_cast<float>(i);
  skelcl::Matrix<float> input(vec, 3);
  EXPECT_EQ(skelcl::Matrix<float>::size_type(4, 3), input.size());
  skelcl::Matrix<float> output = m(input);
  EXPECT_EQ(input.size(), output.size());
  for (size_t i = 0; i < output.rowCount(); ++i)
    for (size_t j = 0; j < output.columnCount(); ++j) {
      EXPECT_EQ(-input({i, j}), output({i, j}));
      EXPECT_EQ(-input[i][j], output[i][j]);
    }
}

TEST_F(SkelCLTest, MatrixAddArgsMatrix) {  // MapTests.cpp:274-321
  skelcl::Map<float(float)> m(R"(
float func( float f, float_matrix_t mat, float add2, int_matrix_t mat2 )
{
  return f + get(mat, 1, 1) + add2 + get(mat2, 1, 2);
}
)");
  std::vector<float> vec(10);
  for (size_t i = 0; i < 10; ++i) vec[i] = static_cast<float>(i * 2.5f);
  skelcl::Matrix<float> input(vec, 3);
  std::vector<float> vec2(10);
  for (size_t i = 0; i < 10; ++i) vec2[i] = static_cast<float>(i);
  skelcl::Matrix<float> mat(vec2, 3);
  skelcl::Matrix<int> mat2({2, 3});
  mat2[1][2] = 5;
  float add2 = 7.75f;
  skelcl::Matrix<float> output = m(input, mat, add2, mat2);
  for (size_t i = 0; i < output.rowCount(); ++i)
    for (size_t j = 0; j < output.columnCount(); ++j)
      EXPECT_EQ(input[i][j] + mat({1, 1}) + add2 + mat2[1][2], output[i][j]);
}

TEST_F(SkelCLTest, MapWithSingleDistribution) {  // MapTests.cpp:323-346
  skelcl::Map<int(int)> map{"int func(int i) { return -i; }"};
  skelcl::Vector<int> input(10, 3);
  skelcl::distribution::setSingle(input);
  skelcl::Vector<int> output = map(input);
  EXPECT_EQ(-3, output[9]);
}

TEST_F(SkelCLTest, MapWithLocalMemory) {  // MapTests.cpp:348-365
  skelcl::Map<int(int)> map{
      "int func(int i, __local int* lp) { lp[0] = i; barrier(CLK_LOCAL_MEM_FENCE); return -lp[0]; }"};
  map.setWorkGroupSize(16);
  skelcl::Vector<int> input(32);
  for (size_t i = 0; i < input.size(); ++i) input[i] = 5;
  skelcl::Vector<int> output = map(input, skelcl::Local(sizeof(int)));
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(-input[i], output[i]);
}

TEST_F(SkelCLTest, MapFloat4) {  // MapTests.cpp:367-388
  skelcl::Map<skelcl::float4(skelcl::float4)> m{"float4 func(float4 f) { return -f; }"};
  skelcl::Vector<skelcl::float4> input(10);
  for (size_t i = 0; i < input.size(); ++i) {
    input[i].s0 = 1.0f;
    input[i].s1 = 2.0f;
    input[i].s2 = 3.0f;
    input[i].s3 = 4.0f;
  }
  skelcl::Vector<skelcl::float4> output = m(input);
  for (size_t i = 0; i < output.size(); ++i) {
    EXPECT_EQ(-input[i].s0, output[i].s0);
    EXPECT_EQ(-input[i].s3, output[i].s3);
  }
}

TEST_F(SkelCLTest, MapDouble4) {  // MapTests.cpp:390-415
  skelcl::Map<skelcl::double4(skelcl::double4)> m{"double4 func(double4 f) { return -f; }"};
  skelcl::Vector<skelcl::double4> input(10);
  for (size_t i = 0; i < input.size(); ++i) {
    input[i].s0 = 1.0;
    input[i].s1 = 2.0;
    input[i].s2 = 3.0;
    input[i].s3 = 4.0;
  }
  skelcl::Vector<skelcl::double4> output = m(input);
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(-input[i].s2, output[i].s2);
}

// ---- Zip (test/ZipTests.cpp) ----------------------------------------------------
TEST_F(SkelCLTest, SimpleZip) {  // ZipTests.cpp:82-104
  skelcl::Zip<float(float, float)> z("float func(float x, float y){ return x+y; }");
  skelcl::Vector<float> left(10), right(10);
  for (size_t i = 0; i < 10; ++i) {
    left[i] = i * 2.5f;
    right[i] = i * 7.5f;
  }
  auto output = z(left, right);
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(left[i] + right[i], output[i]);
}

TEST_F(SkelCLTest, ZipAddArgs) {  // ZipTests.cpp:106-132
  skelcl::Zip<float(float, float)> z(
      "float func(float x, float y, float add, float add2) { return (x*y)+add+add2; }");
  skelcl::Vector<float> left(10), right(10);
  for (size_t i = 0; i < 10; ++i) {
    left[i] = i * 2.5f;
    right[i] = i * 4.5f;
  }
  float add = 5.25f, add2 = 7.75f;
  auto output = z(left, right, add, add2);
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ((left[i] * right[i]) + add + add2, output[i]);
}

TEST_F(SkelCLTest, ZipLeftID) {  // ZipTests.cpp:134-158: output aliases the left input
  skelcl::Zip<float(float, float)> z("float func(float x, float y) { return x; }");
  skelcl::Vector<float> left(10), right(10);
  left.setDistribution(skelcl::distribution::Block(left));
  right.setDistribution(skelcl::distribution::Block(right));
  for (size_t i = 0; i < 10; ++i) {
    left[i] = i * 2.5f;
    right[i] = i * 4.5f;
  }
  z(skelcl::out(left), left, right);
  for (size_t i = 0; i < left.size(); ++i) EXPECT_EQ(i * 2.5f, left[i]);
}

TEST_F(SkelCLTest, SimpleZip2D) {  // ZipTests.cpp:160-187
  skelcl::Zip<float(float, float)> z("float func(float mat1,float mat2){ return mat1 + mat2; }");
  std::vector<float> l(10), r(10);
  for (size_t i = 0; i < 10; ++i) {
    l[i] = i * 2.5f;
    r[i] = i * 7.5f;
  }
  skelcl::Matrix<float> ml(l, 3), mr(r, 3);
  auto output = z(ml, mr);
  EXPECT_EQ(ml.size(), output.size());
  for (size_t i = 0; i < output.rowCount(); ++i)
    for (size_t j = 0; j < output.columnCount(); ++j) EXPECT_EQ(ml[i][j] + mr[i][j], output[i][j]);
}

TEST_F(SkelCLTest, ZipVoidAddArgs) {  // ZipTests.cpp:189-214
  skelcl::Zip<void(float, float)> z(
      "void func(float x, float y, __global float* out) { out[get_global_id(0)] = x*y; }");
  skelcl::Vector<float> left(10), right(10), output(10);
  for (size_t i = 0; i < 10; ++i) {
    left[i] = i * 2.5f;
    right[i] = i * 4.5f;
  }
  z(left, right, skelcl::out(output));
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(left[i] * right[i], output[i]);
}

// ---- Reduce (test/ReduceTests.cpp) -------------------------------------------------
TEST_F(SkelCLTest, SimpleReduce) {  // ReduceTests.cpp:77-90
  skelcl::Reduce<float(float)> r("float func(float x, float y){ return x+y; }");
  skelcl::Vector<float> input(100);
  for (size_t i = 0; i < input.size(); ++i) input[i] = i;
  skelcl::Vector<float> output = r(input);
  EXPECT_LE(1u, output.size());
  EXPECT_EQ(4950, output[0]);
}

TEST_F(SkelCLTest, ReduceAdditionalArg) {  // ReduceTests.cpp:92-106
  skelcl::Reduce<float(float)> r("float func(float x, float y, float a){ return a*(x+y); }");
  skelcl::Vector<float> input(100);
  for (size_t i = 0; i < input.size(); ++i) input[i] = i;
  skelcl::Vector<float> output = r(input, 1.0f);
  EXPECT_EQ(4950, output[0]);
}

TEST_F(SkelCLTest, SimpleReduce2) {  // ReduceTests.cpp:108-121
  skelcl::Reduce<int(int)> r("int func(int x, int y){ return x+y; }");
  skelcl::Vector<int> input(1587);
  for (unsigned int i = 0; i < input.size(); ++i) input[i] = i;
  skelcl::Vector<int> output = r(input);
  EXPECT_EQ(1258491, output[0]);
}

TEST_F(SkelCLTest, LongReduce) {  // ReduceTests.cpp:123-136
  skelcl::Reduce<int(int)> r("int func(int x, int y){ return x+y; }");
  skelcl::Vector<int> input(100000000, 1);
  skelcl::Vector<int> output = r(input);
  EXPECT_EQ(100000000, output[0]);
}

TEST_F(SkelCLTest, ReduceSizes) {  // ReduceTests.cpp:138-170
  skelcl::Reduce<float(float)> r("float func(float x, float y){ return x+y; }");
  skelcl::Vector<float> input;
  skelcl::Vector<float> output;
  for (int i = 1; i < 256; ++i) {
    input.resize(i, 1);
    output = r(input);
    EXPECT_EQ(input.size(), output[0]);
  }
  for (int i = 8192; i < 8192 + 256; ++i) {
    input.resize(i, 1);
    output = r(input);
    EXPECT_EQ(input.size(), output[0]);
  }
}

// ---- Scan (test/ScanTests.cpp) --------------------------------------------------------
TEST_F(SkelCLTest, SimpleScan) {  // ScanTests.cpp:71-88
  skelcl::Scan<int(int)> s{"int func(int x, int y){ return x+y; }"};
  skelcl::Vector<int> input(1024);
  for (size_t i = 0; i < input.size(); ++i) input[i] = 1;
  skelcl::Vector<int> output = s(input);
  input.dataOnDeviceModified();
  EXPECT_EQ(1024u, output.size());
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(i, output[i]);
}

TEST_F(SkelCLTest, SmallScan) {  // ScanTests.cpp:90-105
  skelcl::Scan<int(int)> s{"int func(int x, int y){ return x+y; }"};
  skelcl::Vector<int> input(10);
  for (size_t i = 0; i < input.size(); ++i) input[i] = 1;
  skelcl::Vector<int> output = s(input);
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(i, output[i]);
}

TEST_F(SkelCLTest, FloatScanWithIdentity) {  // ScanTests.cpp:66-69
  skelcl::Scan<float(float)> s{"float func(float x, float y){ return x+y; }", "0.0f"};
  skelcl::Vector<float> input(5, 2.0f);
  skelcl::Vector<float> output = s(input);
  for (size_t i = 0; i < output.size(); ++i) EXPECT_EQ(2.0f * i, output[i]);
}

TEST_F(SkelCLTest, InclusiveAndReverseScan) {  // extension: inclusive / reverse forms
  skelcl::Scan<int(int)> s{"int func(int x, int y){ return x+y; }"};
  s.setInclusive(true);
  skelcl::Vector<int> input(100000, 1);
  skelcl::Vector<int> output = s(input);
  for (size_t i = 0; i < output.size(); i += 997) EXPECT_EQ(i + 1, output[i]);
  s.setReverse(true);
  output = s(input);
  for (size_t i = 0; i < output.size(); i += 997) EXPECT_EQ(input.size() - i, output[i]);
}

// ---- MapOverlap (test/MapOverlapTests.cpp) ---------------------------------------------
static void checkShift(int dx, int dy, unsigned range, size_t size, int fill) {
  char src[128];
  std::snprintf(src, sizeof(src), "int func(input_matrix_t f){ return getData(f, %d, %d); }", dx, dy);
  skelcl::MapOverlap<int(int)> m{src, range};
  skelcl::Matrix<int> input(skelcl::MatrixSize{size, size});
  for (size_t i = 0; i < size; ++i)
    for (size_t j = 0; j < size; ++j) input[i][j] = fill == 0 ? (int)(i * j + i) : (fill == 1 ? (int)j : (int)i);
  skelcl::Matrix<int> output = m(input);
  EXPECT_EQ(size, output.size().rowCount());
  EXPECT_EQ(size, output.size().columnCount());
  for (size_t i = 0; i < size; ++i)
    for (size_t j = 0; j < size; ++j) {
      long long y = (long long)i + dy, x = (long long)j + dx;
      y = y < 0 ? 0 : (y >= (long long)size ? (long long)size - 1 : y);
      x = x < 0 ? 0 : (x >= (long long)size ? (long long)size - 1 : x);
      EXPECT_EQ(input[y][x], output[i][j]);
    }
}

TEST_F(SkelCLTest, MapOverlapRightShift) { checkShift(-1, 0, 1, 1024, 0); }   // MapOverlapTests.cpp:187
TEST_F(SkelCLTest, MapOverlapTwoRightShift) { checkShift(-2, 0, 2, 100, 1); } // :218
TEST_F(SkelCLTest, MapOverlapLeftShift) { checkShift(1, 0, 1, 100, 1); }      // :251
TEST_F(SkelCLTest, MapOverlapTwoLeftShift) { checkShift(2, 0, 2, 100, 1); }   // :283
TEST_F(SkelCLTest, MapOverlapDownShift) { checkShift(0, -1, 1, 1024, 2); }    // :317
TEST_F(SkelCLTest, MapOverlapTwoDownShift) { checkShift(0, -2, 2, 100, 2); }  // :348
TEST_F(SkelCLTest, MapOverlapUpShift) { checkShift(0, 1, 1, 1024, 2); }       // :381
TEST_F(SkelCLTest, MapOverlapTwoUpShift) { checkShift(0, 2, 2, 100, 2); }     // :415

TEST_F(SkelCLTest, MapOverlapNeutralPadding) {  // NEUTRAL padding with a non-zero element
  skelcl::MapOverlap<float(float)> m{"float func(input_matrix_t f){ return getData(f, -1, -1); }", 1,
                                     skelcl::detail::Padding::NEUTRAL, 3.5f};
  skelcl::Matrix<float> input(skelcl::MatrixSize{10, 7}, 1.0f);
  skelcl::Matrix<float> output = m(input);
  EXPECT_EQ(3.5f, output[0][3]);
  EXPECT_EQ(3.5f, output[4][0]);
  EXPECT_EQ(1.0f, output[4][4]);
}

// ---- AllPairs (test/AllPairsTests.cpp) -----------------------------------------------------
static void testAllPairsWithMatrices(unsigned height, unsigned dim, unsigned width, bool precise) {
  skelcl::Zip<float(float, float)> zip("float func(float x, float y){ return x*y; }");
  skelcl::Reduce<float(float)> reduce("float func(float x, float y){ return x+y; }");
  skelcl::AllPairs<float(float, float)> allpairs(reduce, zip);
  allpairs.setPrecise(precise);
  std::vector<float> tl(height * dim), tr(dim * width);
  for (auto& v : tl) v = std::rand() % 100;
  for (auto& v : tr) v = std::rand() % 101;
  skelcl::Matrix<float> left(tl, dim), right(tr, width);
  EXPECT_EQ(height, left.rowCount());
  EXPECT_EQ(width, right.columnCount());
  skelcl::Matrix<float> output = allpairs(left, right);
  EXPECT_EQ(height, output.rowCount());
  EXPECT_EQ(width, output.columnCount());
  for (size_t i = 0; i < output.rowCount(); ++i)
    for (size_t j = 0; j < output.columnCount(); ++j) {
      float tmp = 0;
      for (size_t k = 0; k < left.columnCount(); ++k) tmp += left[i][k] * right[k][j];
      EXPECT_EQ(tmp, output[i][j]);
    }
}

TEST_F(SkelCLTest, AllPairsSquare64) {  // AllPairsTests.cpp:78-80
  std::srand(1);
  testAllPairsWithMatrices(64, 64, 64, false);
  testAllPairsWithMatrices(64, 64, 64, true);
}
TEST_F(SkelCLTest, AllPairs32x128) {  // AllPairsTests.cpp:83-85
  std::srand(1);
  testAllPairsWithMatrices(32, 128, 32, false);
  testAllPairsWithMatrices(32, 128, 32, true);
}
TEST_F(SkelCLTest, AllPairsArbitrary) {  // AllPairsTests.cpp:88-90
  std::srand(1);
  testAllPairsWithMatrices(100, 60, 11, false);
  testAllPairsWithMatrices(100, 60, 11, true);
}

TEST_F(SkelCLTest, AllPairsAdditionalArguments) {  // AllPairsTests.cpp:134-174
  std::srand(1);
  skelcl::Zip<float(float, float)> zip("float func(float x, float y, float a){ return x*y+a; }");
  skelcl::Reduce<float(float)> reduce("float func(float x, float y, float b){ return x+y+b; }");
  skelcl::AllPairs<float(float, float)> allpairs(reduce, zip);
  std::vector<float> tl(4096), tr(4096);
  for (auto& v : tl) v = std::rand() % 100;
  for (auto& v : tr) v = std::rand() % 101;
  skelcl::Matrix<float> left(tl, 64), right(tr, 64);
  float a = 5.0f, b = 6.0f;
  skelcl::Matrix<float> output = allpairs(left, right, b, a);  // the Reduce's argument first
  for (size_t i = 0; i < 64; ++i)
    for (size_t j = 0; j < 64; ++j) {
      float tmp = 0;
      for (size_t k = 0; k < 64; ++k) tmp += (left[i][k] * right[k][j] + a) + b;
      EXPECT_EQ(tmp, output[i][j]);
    }
}

TEST_F(SkelCLTest, AllPairsGeneric) {  // AllPairsTests.cpp:176-224
  std::srand(1);
  skelcl::AllPairs<float(float, float)> allpairs(
      "float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim) {"
      "float res = 0;"
      "for (int i = 0; i < dim; ++i) {"
      "  res += getElementFromRow(row, i) * getElementFromColumn(col, i); }"
      "return res; }");
  const unsigned height = 100, dim = 55, width = 23;
  std::vector<float> tl(height * dim), tr(dim * width);
  for (auto& v : tl) v = std::rand() % 99;
  for (auto& v : tr) v = std::rand() % 101;
  skelcl::Matrix<float> left(tl, dim), right(tr, width);
  skelcl::Matrix<float> output = allpairs(left, right);
  for (size_t i = 0; i < height; ++i)
    for (size_t j = 0; j < width; ++j) {
      float tmp = 0;
      for (size_t k = 0; k < dim; ++k) tmp += left[i][k] * right[k][j];
      EXPECT_EQ(tmp, output[i][j]);
    }
}

TEST_F(SkelCLTest, AllPairsGenericAddArguments) {  // AllPairsTests.cpp:226-270
  std::srand(1);
  skelcl::AllPairs<float(float, float)> allpairs(
      "float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim, int start) {"
      "float res = start;"
      "for (int i = 0; i < dim; ++i) {"
      "  res += getElementFromRow(row, i) * getElementFromColumn(col, i); }"
      "return res; }");
  const unsigned height = 10, dim = 55, width = 23;
  std::vector<float> tl(height * dim), tr(dim * width);
  for (auto& v : tl) v = std::rand() % 98;
  for (auto& v : tr) v = std::rand() % 107;
  skelcl::Matrix<float> left(tl, dim), right(tr, width);
  int start = 5;
  skelcl::Matrix<float> output = allpairs(left, right, start);
  for (size_t i = 0; i < height; ++i)
    for (size_t j = 0; j < width; ++j) {
      float tmp = start;
      for (size_t k = 0; k < dim; ++k) tmp += left[i][k] * right[k][j];
      EXPECT_EQ(tmp, output[i][j]);
    }
}

// ---- Index containers (test/IndexVectorTests.cpp, IndexMatrixTests.cpp) ----------------
TEST_F(SkelCLTest, IndexVector) {  // IndexVectorTests.cpp:61-95
  skelcl::Vector<skelcl::Index> vi(1024);
  EXPECT_EQ(1024u, vi.size());
  EXPECT_EQ(0u, vi.front());
  EXPECT_EQ(1023u, vi.back());
  skelcl::IndexVector index(1024);
  skelcl::Map<void(skelcl::Index)> mv("void func(Index i, __global int* out) { out[i] = i; }");
  skelcl::Vector<int> v(1024);
  mv(index, skelcl::out(v));
  for (size_t i = 0; i < v.size(); ++i) EXPECT_EQ(i, v[i]);
  skelcl::IndexVector index2(1023);
  skelcl::Map<int(skelcl::Index)> m("int func(Index i) { return i; }");
  auto w = m(index2);
  EXPECT_EQ(1023u, w.size());
  for (size_t i = 0; i < w.size(); ++i) EXPECT_EQ(i, w[i]);
}

TEST_F(SkelCLTest, IndexMatrix) {  // IndexMatrixTests.cpp:61-105
  skelcl::Matrix<skelcl::IndexPoint> mi({256, 32});
  EXPECT_EQ(256u * 32u, mi.size().elemCount());
  EXPECT_EQ(skelcl::IndexPoint(0, 0), mi.front());
  EXPECT_EQ(skelcl::IndexPoint(255, 31), mi.back());
  skelcl::IndexMatrix index({128, 32});
  skelcl::Map<void(skelcl::IndexPoint)> mv(
      "void func(IndexPoint ip, int_matrix_t out) { set(out, ip.y, ip.x, ip.y+ip.x); }");
  skelcl::Matrix<int> m({128, 32});
  mv(index, skelcl::out(m));
  for (size_t y = 0; y < 128; ++y)
    for (size_t x = 0; x < 32; ++x) EXPECT_EQ(y + x, m[y][x]);
  skelcl::Map<int(skelcl::IndexPoint)> mp("int func(IndexPoint i) { return i.y+i.x; }");
  skelcl::IndexMatrix index2({32, 128});
  skelcl::Matrix<int> o = mp(index2);
  EXPECT_EQ(32u, o.rowCount());
  EXPECT_EQ(128u, o.columnCount());
  for (size_t y = 0; y < 32; ++y)
    for (size_t x = 0; x < 128; ++x) EXPECT_EQ(y + x, o[y][x]);
}

// ---- SHA-1 (test/SHA1Tests.cpp) --------------------------------------------------------
TEST(SHA1, KnownAnswers) {  // SHA1Tests.cpp:58-77
  EXPECT_EQ(std::string("da39a3ee5e6b4b0d3255bfef95601890afd80709"), skelcl::detail::util::hash(""));
  EXPECT_EQ(std::string("2fd4e1c67a2d28fced849ee1bb76e7391b93eb12"),
            skelcl::detail::util::hash("The quick brown fox jumps over the lazy dog"));
  EXPECT_EQ(std::string("de9f2c7fd25e1b3afad3e85a0bd17d9b100db4b3"),
            skelcl::detail::util::hash("The quick brown fox jumps over the lazy cog"));
}

// ---- containers ----------------------------------------------------------------------------
TEST_F(SkelCLTest, VectorCoherence) {  // host writes after a device pass need dataOnHostModified
  skelcl::Map<int(int)> m("int func(int x) { return x + 1; }");
  skelcl::Vector<int> v(1000, 1);
  skelcl::Vector<int> w = m(v);
  EXPECT_EQ(2, w[999]);
  v[0] = 41;
  v.dataOnHostModified();
  w = m(v);
  EXPECT_EQ(42, w[0]);
  skelcl::Vector<int> copy(w);
  EXPECT_EQ(42, copy[0]);
}

// ---- further restated cases ---------------------------------------------------------
TEST_F(SkelCLTest, MapLargeHostFilledInput) {  // MapTests.cpp TempInputVector
  skelcl::Map<float(float)> neg("float func(float f) { return -f; }");
  skelcl::Vector<float> in(1024 * 1000);
  for (size_t i = 0; i < in.size(); ++i) in[i] = 2.5f * (float)i;
  skelcl::Vector<float> out;
  out = neg(in);
  ASSERT_EQ(in.size(), out.size());
  for (size_t i = 0; i < out.size(); i += 997) EXPECT_EQ(-in[i], out[i]);
  EXPECT_EQ(-in[in.size() - 1], out[out.size() - 1]);
}

TEST_F(SkelCLTest, MapMatrixScalarArgs) {  // MapTests.cpp MatrixAddArgs
  skelcl::Map<float(float)> m("float func(float v, float a, float b) { return v + a + b; }");
  std::vector<float> flat(10);
  for (size_t i = 0; i < flat.size(); ++i) flat[i] = 2.5f * (float)i;
  skelcl::Matrix<float> in(flat, 3);  // 4 rows of 3, the last row padded
  EXPECT_EQ(skelcl::Matrix<float>::size_type(4, 3), in.size());
  skelcl::Matrix<float> out = m(in, 5.25f, 7.75f);
  EXPECT_EQ(in.size(), out.size());
  for (size_t r = 0; r < out.rowCount(); ++r)
    for (size_t c = 0; c < out.columnCount(); ++c) EXPECT_EQ(in({r, c}) + 5.25f + 7.75f, out({r, c}));
}

TEST_F(SkelCLTest, TwoDeviceRequestRunsOnOne) {  // MapTests.cpp SimpleMultiDeviceMap2
  skelcl::terminate();
  skelcl::init(skelcl::nDevices(2));  // one GPU: every element on device 0
  skelcl::Map<int(float)> m("int func(float f) { return skelcl_get_device_id(); }");
  skelcl::Vector<float> in(10);
  skelcl::Vector<int> out = m(in);
  ASSERT_EQ(10u, out.size());
  for (size_t i = 0; i < out.size(); ++i) EXPECT_EQ(0, out[i]);
}

TEST_F(SkelCLTest, ReduceGrowingVector) {  // ReduceTests.cpp nSizesReduce2
  skelcl::Reduce<float(float)> sum("float func(float x, float y){ return x+y; }");
  skelcl::Vector<float> in;
  skelcl::Vector<float> out;
  for (int n = 8192; n < 8192 + 256; ++n) {
    in.resize(n, 1.0f);
    out = sum(in);
    EXPECT_EQ((float)in.size(), out[0]);
  }
}

TEST_F(SkelCLTest, VectorCopyIsDeep) {  // VectorTests.cpp Copy, CopyWithDataOnDevice
  skelcl::Vector<int> a(5);
  for (size_t i = 0; i < 5; ++i) a[i] = 5;
  skelcl::Vector<int> b(a);
  for (size_t i = 0; i < 5; ++i) a[i] = 0;
  for (size_t i = 0; i < 5; ++i) EXPECT_EQ(5, b[i]);
  // the same when the newest data is on the device
  skelcl::Vector<int> c(5);
  for (size_t i = 0; i < 5; ++i) c[i] = 5;
  c.setDistribution(skelcl::detail::SingleDistribution<skelcl::Vector<int>>());
  c.createDeviceBuffers();
  c.copyDataToDevices();
  c.dataOnDeviceModified();
  skelcl::Vector<int> d(c);
  for (size_t i = 0; i < 5; ++i) c[i] = 0;
  ASSERT_EQ(5u, d.size());
  for (size_t i = 0; i < 5; ++i) EXPECT_EQ(5, d[i]);
}

TEST_F(SkelCLTest, VectorResizeOperations) {  // VectorTests.cpp Resize
  skelcl::Vector<int> v;
  v.resize(10);
  EXPECT_EQ(10u, v.size());
  v.push_back(5);
  EXPECT_EQ(11u, v.size());
  v.pop_back();
  EXPECT_EQ(10u, v.size());
  v.insert(v.begin(), 5);
  EXPECT_EQ(11u, v.size());
  v.insert(v.begin(), 2, 5);
  EXPECT_EQ(13u, v.size());
  std::vector<int> two(2);
  v.insert(v.begin(), two.begin(), two.end());
  EXPECT_EQ(15u, v.size());
  v.erase(v.begin());
  EXPECT_EQ(14u, v.size());
  v.erase(v.begin(), v.begin() + 2);
  EXPECT_EQ(12u, v.size());
  v.clear();
  EXPECT_EQ(0u, v.size());
}

namespace {
struct GridPoint {  // a user struct stored in a Vector
  int x = 0, y = 0;
  GridPoint() = default;
  GridPoint(int x_, int y_) : x(x_), y(y_) {}
};
}  // namespace

TEST_F(SkelCLTest, VectorOfStructsFilledThroughIterators) {  // VectorTests.cpp CompleteInitialization
  skelcl::Vector<GridPoint> pts(1024 * 768);
  auto it = pts.begin();
  for (int x = 0; x < 1024; ++x)
    for (int y = 0; y < 768; ++y) *(it++) = GridPoint(x, y);
  EXPECT_EQ(1024u * 768u, pts.size());
  EXPECT_EQ(23, pts[23 * 768 + 42].x);
  EXPECT_EQ(42, pts[23 * 768 + 42].y);
}

TEST_F(SkelCLTest, MatrixFromNestedVectors) {  // MatrixTests.cpp CreateMatrixFrom2DVector
  std::vector<std::vector<int>> rows(10, std::vector<int>(10));
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) rows[i][j] = i * j;
  skelcl::Matrix<int> m = skelcl::Matrix<int>::from2DVector(rows);
  EXPECT_FALSE(m.empty());
  EXPECT_EQ(100u, m.size().elemCount());
  for (size_t i = 0; i < 10; ++i)
    for (size_t j = 0; j < 10; ++j) EXPECT_EQ((int)(i * j), m[i][j]);
}

namespace {
struct Tagged {  // a user struct with a non-zero default
  int a;
  explicit Tagged(int v = 7) : a(v) {}
};
}  // namespace

// VectorTests.cpp CreateEmptyVector, CreateVector; MatrixTests.cpp
// CreateEmptyMatrix, CreateMatrix; ZipTests.cpp CreateZipWithFile; the
// Create* cases of the skeleton suites (construction from strings and files)
TEST_F(SkelCLTest, ContainerAndSkeletonConstruction) {
  skelcl::Vector<int> empty;
  EXPECT_TRUE(empty.empty());
  EXPECT_EQ(0u, empty.size());
  skelcl::Vector<int> zeros(10);
  EXPECT_FALSE(zeros.empty());
  EXPECT_EQ(10u, zeros.size());
  for (size_t i = 0; i < zeros.size(); ++i) EXPECT_EQ(0, zeros[i]);
  skelcl::Vector<Tagged> tagged(5, Tagged(1));
  EXPECT_EQ(5u, tagged.size());
  EXPECT_EQ(1, tagged.begin()->a);
  skelcl::Matrix<int> emptyM;
  EXPECT_TRUE(emptyM.empty());
  skelcl::Matrix<double> md({10, 10});
  EXPECT_FALSE(md.empty());
  EXPECT_EQ(100u, md.size().elemCount());
  for (size_t i = 0; i < 10; ++i)
    for (size_t j = 0; j < 10; ++j) EXPECT_EQ(0.0, md({i, j}));

  const char* fn = "skelcl_zip_function.cl";
  { std::ofstream f(fn, std::ios_base::trunc); f << "float func(float x, float y) { return x+y; }"; }
  std::ifstream file(fn);
  skelcl::Zip<float(float, float)> add(file);
  std::remove(fn);
  skelcl::Vector<float> a(4, 1.5f), b(4, 2.0f);
  skelcl::Vector<float> c = add(a, b);
  for (size_t i = 0; i < 4; ++i) EXPECT_EQ(3.5f, c[i]);

  skelcl::Reduce<float(float)> r("float func(float x, float y){ return x+y; }");
  skelcl::Scan<int(int)> sc("int func(int x, int y){ return x+y; }");
  skelcl::MapOverlap<float(float)> mo("float func(input_matrix_t f) { return -getData(f, 0, 0); }", 1);
  skelcl::Reduce<float(float)> ar("float func(float x, float y){ return x+y; }");
  skelcl::Zip<float(float, float)> az("float func(float x, float y){ return x*y; }");
  skelcl::AllPairs<float(float, float)> ap(ar, az);
  EXPECT_EQ(std::string("func"), r.func());
}

// ---- distributions (test/DistributionTests.cpp): one GPU, every kind valid
//      and placed on the one device of the global list ----------------------------
template <typename C>
static void expectOnTheDevice(const C& c) {
  auto& dist = c.distribution();
  EXPECT_TRUE(dist.isValid());
  ASSERT_EQ(skelcl::detail::globalDeviceList.size(), dist.devices().size());
  EXPECT_EQ(1u, dist.devices().size());
  EXPECT_EQ(skelcl::detail::globalDeviceList[0].get(), dist.device(0).get());
}

TEST_F(SkelCLTest, DistributionKinds) {  // DistributionTests.cpp Default, Single*, Block*, Copy*
  EXPECT_FALSE((skelcl::detail::Distribution<skelcl::Vector<int>>().isValid()));
  skelcl::Vector<int> v1, v2, v3, v4, v5, v6;
  v1.setDistribution(skelcl::distribution::Single(v1));
  skelcl::distribution::setSingle(v2);
  v3.setDistribution(skelcl::distribution::Block(v3));
  skelcl::distribution::setBlock(v4);
  v5.setDistribution(skelcl::distribution::Copy(v5));
  skelcl::distribution::setCopy(v6);
  for (auto* v : {&v1, &v2, &v3, &v4, &v5, &v6}) expectOnTheDevice(*v);
  skelcl::Matrix<int> m1, m2, m3;
  m1.setDistribution(skelcl::distribution::Single(m1));
  skelcl::distribution::setBlock(m2);
  skelcl::distribution::setCopy(m3);
  for (auto* m : {&m1, &m2, &m3}) expectOnTheDevice(*m);
  skelcl::IndexVector iv(1024);
  skelcl::distribution::setSingle(iv);
  expectOnTheDevice(iv);
  // a skeleton still computes the whole container under each kind
  skelcl::Map<int(int)> neg("int func(int i) { return -i; }");
  for (int kind = 0; kind < 3; ++kind) {
    skelcl::Vector<int> in(1000);
    for (size_t i = 0; i < in.size(); ++i) in[i] = (int)i;
    if (kind == 0) skelcl::distribution::setSingle(in);
    if (kind == 1) skelcl::distribution::setBlock(in);
    if (kind == 2) skelcl::distribution::setCopy(in);
    skelcl::Vector<int> out = neg(in);
    ASSERT_EQ(in.size(), out.size());
    for (size_t i = 0; i < out.size(); ++i) EXPECT_EQ(-(int)i, out[i]);
  }
}

int main(int argc, char** argv) {
  ::testing::InitGoogleTest(&argc, argv);
  return RUN_ALL_TESTS();
}
