// main() for gtest-style test files that bring none of their own (what
// GoogleTest's gtest_main library provides): runs every registered test and
// returns the number that failed.
#include "gtest/gtest.h"

int main(int argc, char** argv) {
  ::testing::InitGoogleTest(&argc, argv);
  return RUN_ALL_TESTS();
}
