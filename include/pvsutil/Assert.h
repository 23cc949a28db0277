// ASSERT / ASSERT_MESSAGE as in pvsutil (libraries/pvsutil/include/pvsutil/Assert.h:47-59):
// active unless NDEBUG; a failed assertion logs and aborts the program.
#ifndef PVSUTIL_ASSERT_H_
#define PVSUTIL_ASSERT_H_

#include <cstdlib>

#include "Logger.h"

#ifdef NDEBUG
#define ASSERT(e) ((void)0)
#define ASSERT_MESSAGE(e, ...) ((void)0)
#else
#define ASSERT(e)                                    \
  do {                                               \
    if (!(e)) {                                      \
      LOG_ERROR("Assertion `", #e, "' failed");      \
      std::abort();                                  \
    }                                                \
  } while (0)
#define ASSERT_MESSAGE(e, ...)                                     \
  do {                                                             \
    if (!(e)) {                                                    \
      LOG_ERROR("Assertion `", #e, "' failed: ", __VA_ARGS__);     \
      std::abort();                                                \
    }                                                              \
  } while (0)
#endif

#endif  // PVSUTIL_ASSERT_H_
