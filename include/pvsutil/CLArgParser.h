// Command-line parsing for SkelCL programs: the pvsutil::CLArgParser interface
// the reference's examples use (libraries/pvsutil/include/pvsutil/CLArgParser.h
// and cmdline/{Arg,Flags,Default,Description,Version}.h), header-only.
//
//   using namespace pvsutil::cmdline;
//   pvsutil::CLArgParser cmd(Description("What the program does."));
//   auto size = Arg<int>(Flags(Short('n'), Long("size")), Description("..."), Default(1024));
//   cmd.add(size).parse(argc, argv);
//   int n = size;                       // or size.getValue()
//
// Accepted forms: --long value, --long=value, -s value, and bare --flag / -f
// for bool arguments.  --help prints the arguments and exits; an unknown
// flag, a missing mandatory argument or an unparsable value is reported
// (-h means --help unless an argument claims it)
// through the logger and exits with EXIT_FAILURE.
#ifndef PVSUTIL_CLARGPARSER_H_
#define PVSUTIL_CLARGPARSER_H_

#include <cstdlib>
#include <functional>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "Logger.h"

namespace pvsutil {
namespace cmdline {

class Short {
public:
  Short(char c) : _name(1, c) {}
  const std::string& getName() const { return _name; }
  bool operator<(const Short& o) const { return _name < o._name; }

private:
  std::string _name;
};

class Long {
public:
  Long(const char* name) : _name(name) {}
  Long(const std::string& name) : _name(name) {}
  const std::string& getName() const { return _name; }
  bool operator<(const Long& o) const { return _name < o._name; }

private:
  std::string _name;
};

class Flags {
public:
  template <typename... Rest>
  Flags(const Short& s, Rest... rest) {
    add(s, rest...);
  }
  template <typename... Rest>
  Flags(const Long& l, Rest... rest) {
    add(l, rest...);
  }
  const std::vector<Short>& getShortFlags() const { return _short; }
  const std::vector<Long>& getLongFlags() const { return _long; }

private:
  void add() {}
  template <typename... Rest>
  void add(const Short& s, Rest... rest) {
    _short.push_back(s);
    add(rest...);
  }
  template <typename... Rest>
  void add(const Long& l, Rest... rest) {
    _long.push_back(l);
    add(rest...);
  }
  std::vector<Short> _short;
  std::vector<Long> _long;
};

class Description {
public:
  Description(const std::string& text = std::string()) : _text(text) {}
  const std::string& getDescription() const { return _text; }

private:
  std::string _text;
};

class Version {
public:
  Version(const std::string& text = std::string()) : _text(text) {}
  const std::string& getVersion() const { return _text; }

private:
  std::string _text;
};

template <typename T>
class DefaultValue {
public:
  explicit DefaultValue(const T& v) : _v(v) {}
  const T& getValue() const { return _v; }

private:
  T _v;
};
template <typename T>
DefaultValue<T> Default(const T& v) {
  return DefaultValue<T>(v);
}
inline DefaultValue<std::string> Default(const char* v) { return DefaultValue<std::string>(v); }

class BaseArg {
public:
  virtual ~BaseArg() = default;
  const std::vector<Short>& shortFlags() const { return _flags.getShortFlags(); }
  const std::vector<Long>& longFlags() const { return _flags.getLongFlags(); }
  const std::string& description() const { return _description.getDescription(); }
  bool isMandatory() const { return _mandatory; }
  bool isSet() const { return _set; }
  std::string flagNames() const {
    std::string s;
    for (const Short& f : shortFlags()) s += (s.empty() ? "-" : ", -") + f.getName();
    for (const Long& f : longFlags()) s += (s.empty() ? "--" : ", --") + f.getName();
    return s;
  }
  virtual void parse(const std::string& value) = 0;
  virtual bool hasArgument() const = 0;  // false: a bool switch
  virtual void printValue(std::ostream& os) const = 0;

protected:
  BaseArg(const Flags& f, const Description& d, bool mandatory, bool set)
      : _flags(f), _description(d), _mandatory(mandatory), _set(set) {}
  Flags _flags;
  Description _description;
  bool _mandatory;
  bool _set;
};

template <typename T>
class ArgImpl : public BaseArg {
public:
  ArgImpl(const Flags& f, const Description& d) : BaseArg(f, d, true, false), _value() {}
  ArgImpl(const Flags& f, const Description& d, const DefaultValue<T>& v)
      : BaseArg(f, d, false, true), _value(v.getValue()) {}
  ArgImpl(const Flags& f, const Description& d, std::function<T(const std::string&)> parser)
      : BaseArg(f, d, true, false), _value(), _parser(parser) {}
  ArgImpl(const Flags& f, const Description& d, const DefaultValue<T>& v,
          std::function<T(const std::string&)> parser)
      : BaseArg(f, d, false, true), _value(v.getValue()), _parser(parser) {}

  void parse(const std::string& text) override {
    if (_parser) {
      _value = _parser(text);
    } else {
      std::istringstream is(text);
      if (!read(is, _value))
        throw std::invalid_argument("cannot read '" + text + "' for: " + description());
    }
    _set = true;
  }
  bool hasArgument() const override { return !std::is_same<T, bool>::value; }
  void printValue(std::ostream& os) const override { os << std::boolalpha << _value; }
  const T& getValue() const { return _value; }
  operator T() const { return _value; }

private:
  static bool read(std::istringstream& is, std::string& v) {
    v = is.str();
    return true;
  }
  template <typename U>
  static bool read(std::istringstream& is, U& v) {
    is >> std::boolalpha >> v;
    return !is.fail();
  }
  T _value;
  std::function<T(const std::string&)> _parser;
};

template <typename T>
ArgImpl<T> Arg(const Flags& f, const Description& d) {
  return ArgImpl<T>(f, d);
}
template <typename T, typename D>
ArgImpl<T> Arg(const Flags& f, const Description& d, const DefaultValue<D>& v) {
  return ArgImpl<T>(f, d, DefaultValue<T>(T(v.getValue())));
}
template <typename T>
ArgImpl<T> Arg(const Flags& f, const Description& d, std::function<T(const std::string&)> parser) {
  return ArgImpl<T>(f, d, parser);
}
template <typename T, typename D>
ArgImpl<T> Arg(const Flags& f, const Description& d, const DefaultValue<D>& v,
               std::function<T(const std::string&)> parser) {
  return ArgImpl<T>(f, d, DefaultValue<T>(T(v.getValue())), parser);
}

}  // namespace cmdline

class CLArgParser {
public:
  explicit CLArgParser(cmdline::Description&& d, cmdline::Version&& v = cmdline::Version(),
                       Logger& logger = defaultLogger)
      : _logger(logger), _description(d), _version(v) {}

  template <typename... Rest>
  CLArgParser& add(cmdline::BaseArg& arg, Rest&&... rest) {
    _args.push_back(&arg);
    for (const auto& s : arg.shortFlags()) _short[s.getName()] = &arg;
    for (const auto& l : arg.longFlags()) _long[l.getName()] = &arg;
    return add(std::forward<Rest>(rest)...);
  }
  CLArgParser& add() { return *this; }

  void parse(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
      std::string a = argv[i];
      if (a == "--help" || (a == "-h" && !_short.count("h"))) help(argv[0]);
      if (a == "--version" && !_version.getVersion().empty()) {
        std::cout << _version.getVersion() << std::endl;
        std::exit(EXIT_SUCCESS);
      }
      cmdline::BaseArg* arg = nullptr;
      std::string value;
      bool inline_value = false;
      if (a.rfind("--", 0) == 0) {
        std::string name = a.substr(2);
        const size_t eq = name.find('=');
        if (eq != std::string::npos) {
          value = name.substr(eq + 1);
          name = name.substr(0, eq);
          inline_value = true;
        }
        auto it = _long.find(name);
        if (it != _long.end()) arg = it->second;
      } else if (a.size() == 2 && a[0] == '-') {
        auto it = _short.find(a.substr(1));
        if (it != _short.end()) arg = it->second;
      }
      if (!arg) die("unknown argument '" + a + "' (--help lists them)");
      if (!inline_value) {
        if (arg->hasArgument()) {
          if (i + 1 >= argc) die("argument " + arg->flagNames() + " needs a value");
          value = argv[++i];
        } else {
          value = "true";
        }
      }
      try {
        arg->parse(value);
      } catch (const std::exception& e) {
        die(e.what());
      }
    }
    for (cmdline::BaseArg* arg : _args)
      if (arg->isMandatory() && !arg->isSet()) die("argument " + arg->flagNames() + " is required");
  }

private:
  [[noreturn]] void die(const std::string& msg) {
    _logger.log(Logger::Severity::Error, __FILE__, __LINE__, msg);
    std::exit(EXIT_FAILURE);
  }
  [[noreturn]] void help(const char* program) {
    std::cout << _description.getDescription() << "\n\nUsage: " << program << " [arguments]\n";
    for (cmdline::BaseArg* arg : _args) {
      std::cout << "  " << arg->flagNames() << "\n      " << arg->description();
      if (!arg->isMandatory()) {
        std::cout << " (default: ";
        arg->printValue(std::cout);
        std::cout << ")";
      }
      std::cout << "\n";
    }
    std::exit(EXIT_SUCCESS);
  }

  Logger& _logger;
  cmdline::Description _description;
  cmdline::Version _version;
  std::vector<cmdline::BaseArg*> _args;
  std::map<std::string, cmdline::BaseArg*> _short, _long;
};

}  // namespace pvsutil

#endif  // PVSUTIL_CLARGPARSER_H_
