// Source splicing: the behaviour of SkelCL's libclang-based `stooling`
// rewriter (libraries/stooling/src/SourceCode.cpp:98-263) re-done with a small
// C tokenizer, plus SHA-1 for the program-cache key (src/Util.cpp:149-180).
//
// stooling's operations and their counterparts here:
//   transferParameters(func, k, kernel)  -> parse_function() returns the
//        parameter list; the program builder appends params[k..] to the
//        generated kernel signature
//   transferArguments(func, k, call)     -> the builder forwards the same
//        names at the call site (SCL_EXTRA_ARGS)
//   renameFunction(from, to)             -> rename_identifier()
//   fixKernelParameter (T_matrix_t)      -> ParamKind::Matrix: the kernel takes
//        (T* data, uint cols) and rebuilds the struct before the call
//        (libraries/stooling/src/FixKernelParameterCallback.cpp:62-116)
#include <cctype>
#include <cstring>

#include "internal.h"

namespace scl {

// ---------------------------------------------------------------------------
// SHA-1 (FIPS 180-4).  Checked against the reference's three known answers
// (test/SHA1Tests.cpp:58-77).
// ---------------------------------------------------------------------------
namespace {
inline uint32_t rol(uint32_t x, int s) { return (x << s) | (x >> (32 - s)); }

void sha1_block(uint32_t h[5], const unsigned char* p) {
  uint32_t w[80];
  for (int i = 0; i < 16; ++i)
    w[i] = (uint32_t)p[4 * i] << 24 | (uint32_t)p[4 * i + 1] << 16 |
           (uint32_t)p[4 * i + 2] << 8 | (uint32_t)p[4 * i + 3];
  for (int i = 16; i < 80; ++i) w[i] = rol(w[i - 3] ^ w[i - 8] ^ w[i - 14] ^ w[i - 16], 1);
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4];
  for (int i = 0; i < 80; ++i) {
    uint32_t f, k;
    if (i < 20) { f = (b & c) | (~b & d); k = 0x5A827999u; }
    else if (i < 40) { f = b ^ c ^ d; k = 0x6ED9EBA1u; }
    else if (i < 60) { f = (b & c) | (b & d) | (c & d); k = 0x8F1BBCDCu; }
    else { f = b ^ c ^ d; k = 0xCA62C1D6u; }
    uint32_t t = rol(a, 5) + f + e + k + w[i];
    e = d; d = c; c = rol(b, 30); b = a; a = t;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e;
}
}  // namespace

std::string sha1_hex(const void* data, size_t n) {
  uint32_t h[5] = {0x67452301u, 0xEFCDAB89u, 0x98BADCFEu, 0x10325476u, 0xC3D2E1F0u};
  const unsigned char* p = static_cast<const unsigned char*>(data);
  size_t full = n / 64;
  for (size_t i = 0; i < full; ++i) sha1_block(h, p + 64 * i);
  unsigned char tail[128];
  size_t rem = n - full * 64;
  if (rem) std::memcpy(tail, p + full * 64, rem);
  tail[rem] = 0x80;
  size_t tail_len = (rem + 1 + 8 <= 64) ? 64 : 128;
  std::memset(tail + rem + 1, 0, tail_len - rem - 1);
  uint64_t bits = (uint64_t)n * 8;
  for (int i = 0; i < 8; ++i) tail[tail_len - 1 - i] = (unsigned char)(bits >> (8 * i));
  sha1_block(h, tail);
  if (tail_len == 128) sha1_block(h, tail + 64);
  static const char* hex = "0123456789abcdef";
  std::string out(40, '0');
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 4; ++j) {
      unsigned v = (h[i] >> (24 - 8 * j)) & 0xff;
      out[i * 8 + j * 2] = hex[v >> 4];
      out[i * 8 + j * 2 + 1] = hex[v & 15];
    }
  return out;
}

// ---------------------------------------------------------------------------
// Tokenizer: identifiers, numbers and punctuation; comments, string and char
// literals and preprocessor lines are skipped (they never hold the function
// definition or a renamable reference).
// ---------------------------------------------------------------------------
namespace {
struct Tok {
  enum Kind { Ident, Number, Punct } kind;
  size_t b, e;
};

std::vector<Tok> tokenize(const std::string& s) {
  std::vector<Tok> out;
  size_t i = 0, n = s.size();
  bool line_start = true;
  while (i < n) {
    char c = s[i];
    if (c == '\n') { line_start = true; ++i; continue; }
    if (std::isspace((unsigned char)c)) { ++i; continue; }
    if (line_start && c == '#') {  // preprocessor line, with continuations
      while (i < n && s[i] != '\n') {
        if (s[i] == '\\' && i + 1 < n && s[i + 1] == '\n') i += 2;
        else ++i;
      }
      continue;
    }
    line_start = false;
    if (c == '/' && i + 1 < n && s[i + 1] == '/') {
      while (i < n && s[i] != '\n') ++i;
      continue;
    }
    if (c == '/' && i + 1 < n && s[i + 1] == '*') {
      size_t e = s.find("*/", i + 2);
      i = (e == std::string::npos) ? n : e + 2;
      continue;
    }
    if (c == '"' || c == '\'') {
      char q = c;
      ++i;
      while (i < n && s[i] != q) {
        if (s[i] == '\\') ++i;
        ++i;
      }
      ++i;
      continue;
    }
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t b = i;
      while (i < n && (std::isalnum((unsigned char)s[i]) || s[i] == '_')) ++i;
      out.push_back({Tok::Ident, b, i});
      continue;
    }
    if (std::isdigit((unsigned char)c) || (c == '.' && i + 1 < n && std::isdigit((unsigned char)s[i + 1]))) {
      size_t b = i;
      while (i < n && (std::isalnum((unsigned char)s[i]) || s[i] == '.' || s[i] == '_' ||
                       ((s[i] == '+' || s[i] == '-') && (s[i - 1] == 'e' || s[i - 1] == 'E'))))
        ++i;
      out.push_back({Tok::Number, b, i});
      continue;
    }
    out.push_back({Tok::Punct, i, i + 1});
    ++i;
  }
  return out;
}

std::string text(const std::string& s, const Tok& t) { return s.substr(t.b, t.e - t.b); }

std::string trim(const std::string& s) {
  size_t b = 0, e = s.size();
  while (b < e && std::isspace((unsigned char)s[b])) ++b;
  while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
  return s.substr(b, e - b);
}

bool has_word(const std::string& s, const char* w) {
  std::vector<Tok> t = tokenize(s);
  for (auto& k : t)
    if (k.kind == Tok::Ident && text(s, k) == w) return true;
  return false;
}

// Classify one parameter declaration.
bool classify(const std::string& decl, Param* p, std::string* err) {
  std::vector<Tok> t = tokenize(decl);
  // name = last identifier not inside [...]
  int depth = 0;
  int name_idx = -1;
  for (size_t i = 0; i < t.size(); ++i) {
    std::string x = text(decl, t[i]);
    if (t[i].kind == Tok::Punct && x == "[") ++depth;
    else if (t[i].kind == Tok::Punct && x == "]") --depth;
    else if (t[i].kind == Tok::Ident && depth == 0) name_idx = (int)i;
  }
  if (name_idx < 0) {
    *err = "cannot find a parameter name in '" + decl + "'";
    return false;
  }
  p->name = text(decl, t[name_idx]);
  std::string type = decl.substr(0, t[name_idx].b) + decl.substr(t[name_idx].e);
  p->type = trim(type);
  if (p->type.empty()) {
    *err = "parameter '" + p->name + "' has no type";
    return false;
  }
  bool pointer = p->type.find('*') != std::string::npos || p->type.find('[') != std::string::npos;
  bool local = has_word(p->type, "__local") || has_word(p->type, "local");
  std::vector<Tok> tt = tokenize(p->type);
  std::string matrix_elem;
  for (auto& k : tt) {
    std::string x = text(p->type, k);
    const std::string suf = "_matrix_t";
    if (k.kind == Tok::Ident && x.size() > suf.size() &&
        x.compare(x.size() - suf.size(), suf.size(), suf) == 0)
      matrix_elem = x.substr(0, x.size() - suf.size());
  }
  if (local && pointer) {
    p->kind = ParamKind::Local;
    std::string pointee;
    for (auto& k : tt) {
      std::string x = text(p->type, k);
      if (k.kind == Tok::Ident && x != "__local" && x != "local" && x != "const" &&
          x != "volatile" && x != "restrict")
        pointee += (pointee.empty() ? "" : " ") + x;
    }
    p->elem = pointee;
  } else if (!matrix_elem.empty() && !pointer) {
    p->kind = ParamKind::Matrix;
    p->elem = matrix_elem;
  } else if (pointer) {
    p->kind = ParamKind::Buffer;
  } else {
    p->kind = ParamKind::Value;
  }
  return true;
}
}  // namespace

bool parse_function(const std::string& src, const std::string& name, FuncSig* sig,
                    std::string* err) {
  std::vector<Tok> t = tokenize(src);
  for (size_t i = 0; i + 1 < t.size(); ++i) {
    if (t[i].kind != Tok::Ident || text(src, t[i]) != name) continue;
    if (text(src, t[i + 1]) != "(") continue;
    // find the matching ')'
    size_t j = i + 1;
    int depth = 0;
    for (; j < t.size(); ++j) {
      std::string x = text(src, t[j]);
      if (x == "(") ++depth;
      else if (x == ")" && --depth == 0) break;
    }
    if (j >= t.size() || j + 1 >= t.size() || text(src, t[j + 1]) != "{") continue;  // call or prototype
    // return type: tokens back to the previous ';', '}' or start
    size_t k = i;
    while (k > 0) {
      std::string x = text(src, t[k - 1]);
      if (x == ";" || x == "}" || x == "{" || x == ")") break;
      --k;
    }
    sig->def_begin = (k < i) ? t[k].b : t[i].b;
    sig->ret = trim(src.substr(sig->def_begin, t[i].b - sig->def_begin));
    // body end
    size_t m = j + 1;
    depth = 0;
    for (; m < t.size(); ++m) {
      std::string x = text(src, t[m]);
      if (x == "{") ++depth;
      else if (x == "}" && --depth == 0) break;
    }
    if (m >= t.size()) {
      *err = "unterminated body of function '" + name + "'";
      return false;
    }
    sig->def_end = t[m].e;
    // split parameters at top-level commas
    sig->params.clear();
    std::string plist = src.substr(t[i + 1].e, t[j].b - t[i + 1].e);
    if (trim(plist).empty() || trim(plist) == "void") return true;
    std::vector<std::string> parts;
    int d = 0;
    size_t start = 0;
    for (size_t c = 0; c < plist.size(); ++c) {
      char ch = plist[c];
      if (ch == '(' || ch == '[' || ch == '<') ++d;
      else if (ch == ')' || ch == ']' || ch == '>') --d;
      else if (ch == ',' && d == 0) {
        parts.push_back(plist.substr(start, c - start));
        start = c + 1;
      }
    }
    parts.push_back(plist.substr(start));
    for (auto& part : parts) {
      Param p;
      if (!classify(trim(part), &p, err)) return false;
      sig->params.push_back(p);
    }
    return true;
  }
  *err = "no definition of function '" + name + "' found in the user source";
  return false;
}

std::string rename_identifier(const std::string& src, const std::string& from,
                              const std::string& to) {
  std::vector<Tok> t = tokenize(src);
  std::string out;
  size_t last = 0;
  for (auto& k : t) {
    if (k.kind == Tok::Ident && text(src, k) == from) {
      out.append(src, last, k.b - last);
      out += to;
      last = k.e;
    }
  }
  out.append(src, last, std::string::npos);
  return out;
}

std::string unroll_loops_in(const std::string& src, const std::string& name) {
  FuncSig sig;
  std::string err;
  if (!parse_function(src, name, &sig, &err)) return src;
  std::vector<Tok> t = tokenize(src);
  std::string out;
  size_t last = 0;
  for (auto& k : t) {
    if (k.b < sig.def_begin || k.e > sig.def_end) continue;
    if (k.kind == Tok::Ident && text(src, k) == "for") {
      out.append(src, last, k.b - last);
      out += "\n#pragma unroll\n";
      last = k.b;
    }
  }
  out.append(src, last, std::string::npos);
  return out;
}

bool source_uses_workitem(const std::string& src) {
  static const char* words[] = {"get_global_id", "get_local_id", "get_group_id",
                                "get_local_size", "get_num_groups", "get_global_size",
                                "barrier", "get_work_dim", "__local", "local"};
  std::vector<Tok> t = tokenize(src);
  for (auto& k : t) {
    if (k.kind != Tok::Ident) continue;
    std::string x = text(src, k);
    for (const char* w : words)
      if (x == w) return true;
  }
  return false;
}

}  // namespace scl
