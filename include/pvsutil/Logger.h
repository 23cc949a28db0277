// Minimal pvsutil logging shim with the names SkelCL programs and tests use
// (libraries/pvsutil/include/pvsutil/Logger.h:60-134 of the reference):
// Logger::Severity, defaultLogger.setLoggingLevel, LOG_* macros and
// ABORT_WITH_ERROR (exit, or throw when THROW_ON_FAILURE is defined).
#ifndef PVSUTIL_LOGGER_H_
#define PVSUTIL_LOGGER_H_

#include <cstdlib>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>

namespace pvsutil {

class Logger {
public:
  enum class Severity { LogAlways = 0, Error, Warning, Info, Debug, DebugInfo };

  Logger() : _level(Severity::Warning), _out(&std::clog) {}
  void setLoggingLevel(Severity s) { _level = s; }
  Severity loggingLevel() const { return _level; }
  void setOutput(std::ostream& os) { _out = &os; }

  template <typename... Args>
  void log(Severity s, const char* file, int line, Args&&... args) {
    if (static_cast<int>(s) > static_cast<int>(_level)) return;
    std::ostringstream msg;
    msg << "[skelcl " << name(s) << " " << file << ":" << line << "] ";
    int dummy[] = {0, ((void)(msg << std::forward<Args>(args)), 0)...};
    (void)dummy;
    (*_out) << msg.str() << std::endl;
  }

private:
  static const char* name(Severity s) {
    switch (s) {
      case Severity::LogAlways: return "LOG";
      case Severity::Error: return "ERROR";
      case Severity::Warning: return "WARNING";
      case Severity::Info: return "INFO";
      case Severity::Debug: return "DEBUG";
      default: return "DEBUG_INFO";
    }
  }
  Severity _level;
  std::ostream* _out;
};

inline Logger defaultLogger;

template <typename... Args>
std::string concat(Args&&... args) {
  std::ostringstream s;
  int dummy[] = {0, ((void)(s << std::forward<Args>(args)), 0)...};
  (void)dummy;
  return s.str();
}

}  // namespace pvsutil

#define LOG(severity, ...) \
  ::pvsutil::defaultLogger.log(severity, __FILE__, __LINE__, __VA_ARGS__)
#define LOG_ERROR(...) LOG(::pvsutil::Logger::Severity::Error, __VA_ARGS__)
#define LOG_WARNING(...) LOG(::pvsutil::Logger::Severity::Warning, __VA_ARGS__)
#define LOG_INFO(...) LOG(::pvsutil::Logger::Severity::Info, __VA_ARGS__)
#ifdef NDEBUG
#define LOG_DEBUG(...) ((void)0)
#define LOG_DEBUG_INFO(...) ((void)0)
#else
#define LOG_DEBUG(...) LOG(::pvsutil::Logger::Severity::Debug, __VA_ARGS__)
#define LOG_DEBUG_INFO(...) LOG(::pvsutil::Logger::Severity::DebugInfo, __VA_ARGS__)
#endif

#ifdef THROW_ON_FAILURE
#define ABORT_WITH_ERROR(err)                                             \
  do {                                                                    \
    LOG_ERROR(err);                                                       \
    throw std::runtime_error(::pvsutil::concat(err));                     \
  } while (0)
#else
#define ABORT_WITH_ERROR(err) \
  do {                        \
    LOG_ERROR(err);           \
    std::exit(EXIT_FAILURE);  \
  } while (0)
#endif

#endif  // PVSUTIL_LOGGER_H_
