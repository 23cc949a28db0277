// User source for a skeleton, from a string, a C string or a stream
// (include/SkelCL/Source.h:61-166, src/Source.cpp of the reference), and the
// process-wide CommonDefinitions prepended to every skeleton program.
#ifndef SKELCL_SOURCE_H_
#define SKELCL_SOURCE_H_

#include <istream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include <pvsutil/Assert.h>

namespace skelcl {

class Source {
public:
  Source() = default;
  Source(const char* source) : _source(source) {
    ASSERT_MESSAGE(!_source.empty(), "Tried to create source object with empty user source.");
  }
  Source(const std::string& source) : _source(source) {
    ASSERT_MESSAGE(!_source.empty(), "Tried to create source object with empty user source.");
  }
  Source(std::istream& is)
      : _source((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>()) {
    ASSERT_MESSAGE(!_source.empty(), "Tried to create source object with empty user source.");
  }
  Source(std::istream&& is)
      : _source((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>()) {
    ASSERT_MESSAGE(!_source.empty(), "Tried to create source object with empty user source.");
  }
  operator std::string() const { return _source; }
  void append(const std::string& source) { _source.append("\n" + source); }

private:
  std::string _source;
};

namespace detail {

class CommonDefinitions {
public:
  enum Level : unsigned int { PRAGMA, USER_DEFINITION, GENERATED_DEFINITION, SIZE };

  static CommonDefinitions& instance() {
    static CommonDefinitions inst;
    return inst;
  }
  static void append(const std::string& source, Level level) {
    std::string& s = instance()._sources[level];
    if (s.find(source) != std::string::npos) return;  // registered once per process
    s.append("\n" + source);
  }
  static Source getSource() {
    auto& inst = instance();
    std::string s;
    for (unsigned int i = 0; i < Level::SIZE; ++i) s.append(inst._sources[i]);
    return s.empty() ? Source() : Source(s);
  }
  static std::string getString() { return std::string(getSource()); }

private:
  CommonDefinitions() : _sources(Level::SIZE) {}
  std::vector<std::string> _sources;
};

class RegisterCommonDefinition {
public:
  RegisterCommonDefinition(const char* definition,
                           CommonDefinitions::Level level = CommonDefinitions::USER_DEFINITION) {
    CommonDefinitions::append(definition, level);
  }
};

class RegisterCommonMacroDefinition {
public:
  template <typename T>
  RegisterCommonMacroDefinition(const char* name, T&& value) {
    std::stringstream ss;
    ss << "#define " << name << " " << value;
    CommonDefinitions::append(ss.str(), CommonDefinitions::USER_DEFINITION);
  }
};

}  // namespace detail
}  // namespace skelcl

#endif  // SKELCL_SOURCE_H_
