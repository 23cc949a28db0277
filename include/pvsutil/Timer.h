// Wall-clock timer with millisecond results, as pvsutil::Timer
// (libraries/pvsutil/include/pvsutil/Timer.h:49-64).
#ifndef PVSUTIL_TIMER_H_
#define PVSUTIL_TIMER_H_

#include <chrono>

namespace pvsutil {

class Timer {
public:
  typedef std::chrono::milliseconds::rep time_type;
  Timer() : _start(std::chrono::high_resolution_clock::now()) {}
  void restart() { _start = std::chrono::high_resolution_clock::now(); }
  time_type stop() { return time(); }
  time_type time() const {
    return std::chrono::duration_cast<std::chrono::milliseconds>(
               std::chrono::high_resolution_clock::now() - _start).count();
  }

private:
  std::chrono::high_resolution_clock::time_point _start;
};

}  // namespace pvsutil

#endif  // PVSUTIL_TIMER_H_
