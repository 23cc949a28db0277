// A small GoogleTest-compatible harness (TEST, TEST_F, EXPECT_* / ASSERT_*)
// so that gtest-style SkelCL test programs build without GoogleTest, which
// this toolchain does not ship.  Failures print file:line and both values;
// RUN_ALL_TESTS() returns the number of failed tests.
#ifndef SKELCL_TEST_GTEST_MINI_H_
#define SKELCL_TEST_GTEST_MINI_H_

#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <iostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

namespace testing {

class Test {
public:
  virtual ~Test() = default;
  virtual void SetUp() {}
  virtual void TearDown() {}
  virtual void TestBody() = 0;
};

struct TestInfo {
  const char* suite;
  const char* name;
  std::function<Test*()> make;
};

inline std::vector<TestInfo>& registry() {
  static std::vector<TestInfo> r;
  return r;
}
inline bool& current_failed() {
  static bool f = false;
  return f;
}
inline int& failures_in_test() {
  static int n = 0;
  return n;
}

struct Registrar {
  Registrar(const char* s, const char* n, std::function<Test*()> m) {
    registry().push_back({s, n, std::move(m)});
  }
};

template <typename T, typename = void>
struct Printable : std::false_type {};
template <typename T>
struct Printable<T, decltype(void(std::declval<std::ostream&>() << std::declval<const T&>()))>
    : std::true_type {};

template <typename T>
std::string show(const T& v) {
  if constexpr (Printable<T>::value) {
    std::ostringstream s;
    s << v;
    return s.str();
  } else {
    return "<unprintable>";
  }
}

inline void report(const char* file, int line, const std::string& what) {
  current_failed() = true;
  if (++failures_in_test() <= 10) std::cout << file << ":" << line << ": Failure\n" << what << "\n";
}

template <typename A, typename B>
bool cmp_eq(const A& a, const B& b) {
  if constexpr (std::is_integral<A>::value && std::is_integral<B>::value &&
                std::is_signed<A>::value != std::is_signed<B>::value)
    return (long long)a == (long long)b;
  else
    return a == b;
}

inline int RunAllTests(const char* filter) {
  int failed = 0, run = 0;
  for (auto& t : registry()) {
    std::string full = std::string(t.suite) + "." + t.name;
    if (filter && *filter && full.find(filter) == std::string::npos) continue;
    ++run;
    current_failed() = false;
    failures_in_test() = 0;
    std::cout << "[ RUN      ] " << full << std::endl;
    Test* obj = t.make();
    obj->SetUp();
    obj->TestBody();
    obj->TearDown();
    delete obj;
    if (current_failed()) {
      ++failed;
      std::cout << "[  FAILED  ] " << full << std::endl;
    } else {
      std::cout << "[       OK ] " << full << std::endl;
    }
  }
  std::cout << "[==========] " << run << " tests ran, " << failed << " failed." << std::endl;
  return failed;
}

inline void InitGoogleTest(int*, char**) {}

}  // namespace testing

#define SCL_TEST_CLASS(suite, name) suite##_##name##_Test
#define TEST_F(fixture, name)                                                          \
  class SCL_TEST_CLASS(fixture, name) : public fixture {                               \
   public:                                                                             \
    void TestBody() override;                                                          \
  };                                                                                   \
  static ::testing::Registrar scl_reg_##fixture##_##name(                              \
      #fixture, #name, [] { return new SCL_TEST_CLASS(fixture, name)(); });             \
  void SCL_TEST_CLASS(fixture, name)::TestBody()
#define TEST(suite, name)                                                              \
  class SCL_TEST_CLASS(suite, name) : public ::testing::Test {                         \
   public:                                                                             \
    void TestBody() override;                                                          \
  };                                                                                   \
  static ::testing::Registrar scl_reg_##suite##_##name(                                \
      #suite, #name, [] { return new SCL_TEST_CLASS(suite, name)(); });                 \
  void SCL_TEST_CLASS(suite, name)::TestBody()

#define SCL_CHECK_BIN(op_ok, a, b, opname, fatal)                                        \
  do {                                                                                 \
    const auto& scl_a_ = (a);                                                          \
    const auto& scl_b_ = (b);                                                          \
    if (!(op_ok)) {                                                                    \
      ::testing::report(__FILE__, __LINE__,                                            \
                        std::string("  Expected: ") + #a + " " opname " " + #b +       \
                            "\n  Actual: " + ::testing::show(scl_a_) + " vs " +        \
                            ::testing::show(scl_b_));                                  \
      if (fatal) return;                                                               \
    }                                                                                  \
  } while (0)

#define EXPECT_EQ(a, b) SCL_CHECK_BIN(::testing::cmp_eq(scl_a_, scl_b_), a, b, "==", false)
#define EXPECT_NE(a, b) SCL_CHECK_BIN(!::testing::cmp_eq(scl_a_, scl_b_), a, b, "!=", false)
#define EXPECT_LE(a, b) SCL_CHECK_BIN(scl_a_ <= scl_b_, a, b, "<=", false)
#define EXPECT_LT(a, b) SCL_CHECK_BIN(scl_a_ < scl_b_, a, b, "<", false)
#define EXPECT_GE(a, b) SCL_CHECK_BIN(scl_a_ >= scl_b_, a, b, ">=", false)
#define EXPECT_GT(a, b) SCL_CHECK_BIN(scl_a_ > scl_b_, a, b, ">", false)
#define ASSERT_EQ(a, b) SCL_CHECK_BIN(::testing::cmp_eq(scl_a_, scl_b_), a, b, "==", true)
#define ASSERT_NE(a, b) SCL_CHECK_BIN(!::testing::cmp_eq(scl_a_, scl_b_), a, b, "!=", true)
#define ASSERT_LE(a, b) SCL_CHECK_BIN(scl_a_ <= scl_b_, a, b, "<=", true)
#define ASSERT_LT(a, b) SCL_CHECK_BIN(scl_a_ < scl_b_, a, b, "<", true)
#define ASSERT_GE(a, b) SCL_CHECK_BIN(scl_a_ >= scl_b_, a, b, ">=", true)
#define ASSERT_GT(a, b) SCL_CHECK_BIN(scl_a_ > scl_b_, a, b, ">", true)
#define EXPECT_TRUE(c) SCL_CHECK_BIN(bool(scl_a_), c, true, "is", false)
#define EXPECT_FALSE(c) SCL_CHECK_BIN(!bool(scl_a_), c, false, "is", false)
#define ASSERT_TRUE(c) SCL_CHECK_BIN(bool(scl_a_), c, true, "is", true)
#define ASSERT_FALSE(c) SCL_CHECK_BIN(!bool(scl_a_), c, false, "is", true)
#define EXPECT_FLOAT_EQ(a, b) \
  SCL_CHECK_BIN(std::fabs((double)scl_a_ - (double)scl_b_) <= 4 * 1.2e-7 * std::fabs((double)scl_b_), a, b, "~=", false)
#define EXPECT_NEAR(a, b, tol) \
  SCL_CHECK_BIN(std::fabs((double)scl_a_ - (double)scl_b_) <= (tol), a, b, "near", false)
#define RUN_ALL_TESTS() ::testing::RunAllTests(std::getenv("SKELCL_TEST_FILTER"))

#endif  // SKELCL_TEST_GTEST_MINI_H_
