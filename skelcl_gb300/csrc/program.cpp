// Program assembly and JIT compilation: the GB300 counterpart of
// detail::Program (src/Program.cpp:83-250) and the per-skeleton
// createAndBuildProgram() bodies (MapDef.h:170-212, ZipDef.h:177-224,
// ReduceDef.h:248-275, ScanDef.h:263-297, MapOverlapDef.h:181-248,
// AllPairsDef.h:213-344).
//
// The generated CUDA source is, in order:
//   prelude (OpenCL C vocabulary)          -- templates/prelude.cuh
//   SCL_TYPE_n typedefs, skeleton defines
//   definitions the user function sees    -- Index, IndexPoint, input_matrix_t,
//                                             lmatrix_t / rmatrix_t
//   common definitions (SKELCL_COMMON_DEFINITION, src/Source.cpp:118-126)
//   user source with the function renamed (stooling renameFunction)
//   extra-parameter plumbing macros (stooling transferParameters /
//                                    transferArguments / fixKernelParameter)
//   skeleton template                      -- templates/<skeleton>.cuh
// and is compiled by NVRTC for sm_103a into a cubin, loaded as a module.
// The cache key is the SHA-1 of the generated source + options, as the
// reference keys its binary cache by util::hash of the source
// (src/Program.cpp:62-75,136-175,252-281).  Environment switches kept from the
// reference: SKELCL_LOAD_BINARY=YES, SKELCL_SAVE_BINARY=YES,
// SKELCL_PRINT_BUILD_LOG=YES; SKELCL_CACHE_DIR picks the cache directory, and
// SKELCL_COMPILE_ALL=YES compiles every kernel variant at construction.
#include <nvrtc.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <sys/stat.h>
#include <unistd.h>

#include "internal.h"

// Template sources, embedded at build time (generated file).
extern const char* scl_tpl_prelude;
extern const char* scl_tpl_elementwise;
extern const char* scl_tpl_reduce;
extern const char* scl_tpl_scan;
extern const char* scl_tpl_mapoverlap_pre;
extern const char* scl_tpl_mapoverlap;
extern const char* scl_tpl_allpairs_pre;
extern const char* scl_tpl_allpairs;

namespace scl {
namespace {

std::string env(const char* name) {
  const char* v = std::getenv(name);
  return v ? std::string(v) : std::string();
}

bool env_yes(const char* name) {
  std::string v = env(name);
  return v == "YES" || v == "yes" || v == "1" || v == "ON" || v == "on";
}

std::string strip_opencl_pragmas(const std::string& s) {
  std::istringstream in(s);
  std::string line, out;
  while (std::getline(in, line)) {
    size_t p = line.find_first_not_of(" \t");
    if (p != std::string::npos && line.compare(p, 7, "#pragma") == 0 &&
        line.find("OPENCL") != std::string::npos)
      continue;
    out += line;
    out += '\n';
  }
  return out;
}

// Number of leading parameters the skeleton itself supplies.
int skeleton_arity(int kind) {
  switch (kind) {
    case SCL_KIND_ZIP:
    case SCL_KIND_ZIP_VOID:
    case SCL_KIND_REDUCE:
    case SCL_KIND_SCAN:
      return 2;
    case SCL_KIND_ALLPAIRS_GENERIC:
      return 3;
    case SCL_KIND_MAP_ADJOINT:
      return 2;  // x, g
    case SCL_KIND_ZIP_ADJOINT:
      return 3;  // x, y, g
    case SCL_KIND_ALLPAIRS:
      return 2;  // both the Reduce and the Zip take two
    default:
      return 1;
  }
}

struct ExtraMacros {
  std::string params, user, setup, args;
};

void append_extra(const std::vector<Param>& ps, size_t first_index, ExtraMacros* m,
                  std::string* args_only) {
  for (size_t i = 0; i < ps.size(); ++i) {
    const Param& p = ps[i];
    std::string nm = "scl_x" + std::to_string(first_index + i);
    switch (p.kind) {
      case ParamKind::Value:
      case ParamKind::Buffer:
        m->params += ", " + p.type + " " + nm;
        m->user += ", " + p.type + " " + nm;
        break;
      case ParamKind::Matrix:
        m->params += ", " + p.elem + "* " + nm + "_d, unsigned int " + nm + "_c";
        m->setup += p.elem + "_matrix_t " + nm + "; " + nm + ".data = " + nm + "_d; " + nm +
                    ".col_count = " + nm + "_c; ";
        m->user += ", " + p.elem + "_matrix_t " + nm;
        break;
      case ParamKind::Local:
        m->params += ", unsigned int " + nm + "_o";
        m->setup += p.type + " " + nm + " = (" + p.type + ")(scl_dyn_smem + " + nm + "_o); ";
        m->user += ", " + p.type + " " + nm;
        break;
    }
    m->args += ", " + nm;
    if (args_only) *args_only += ", " + nm;
  }
}

bool neutral_is_zero(const std::string& s) {
  if (s.empty()) return true;
  char* end = nullptr;
  double v = std::strtod(s.c_str(), &end);
  while (end && *end && (std::isspace((unsigned char)*end) || *end == 'f' || *end == 'F' ||
                         *end == 'u' || *end == 'U' || *end == 'l' || *end == 'L'))
    ++end;
  return end && *end == '\0' && v == 0.0;
}

// Float folds (Reduce, Scan and their fused forms) carry across blocks in FP64.
bool wants_f64_carry(const scl_program_desc* d) {
  if (d->flags & SCL_PROG_NO_F64_CARRY) return false;
  int t = -1;  // the folded type
  if (d->kind == SCL_KIND_REDUCE || d->kind == SCL_KIND_SCAN || d->kind == SCL_KIND_SCAN_MAP) t = 0;
  if (d->kind == SCL_KIND_ZIP_REDUCE) t = 2;
  return t >= 0 && d->n_types > t && d->type_names[t] && std::string(d->type_names[t]) == "float";
}

bool folds(int kind) {
  return kind == SCL_KIND_REDUCE || kind == SCL_KIND_SCAN || kind == SCL_KIND_ZIP_REDUCE ||
         kind == SCL_KIND_SCAN_MAP;
}

struct Assembly {
  std::string source;
  std::vector<std::string> kernels;  // name expressions compiled at construction
  std::vector<std::string> lazy;     // further variants, compiled on first use
};

int assemble(const scl_program_desc* d, scl_program* p, bool want_f64, Assembly* out,
             std::string* err) {
  const int kind = d->kind;
  const std::string func = d->func ? d->func : "func";
  const std::string src = strip_opencl_pragmas(d->source ? d->source : "");
  if (src.find_first_not_of(" \t\r\n") == std::string::npos) {
    *err = "empty user source";
    return SCL_ERR_ARG;
  }
  std::ostringstream s;
  s << "// generated by libskelcl_cuda\n#define SCL_KIND " << kind << "\n";
  const bool point = kind == SCL_KIND_MAP_POINT || kind == SCL_KIND_MAP_POINT_VOID;
  if (point) s << "#define SCL_WI_SWAP 1\n#define SCL_WORK_DIM 2\n";
  if (kind == SCL_KIND_MAPOVERLAP) s << "#define SCL_WORK_DIM 2\n";
  s << scl_tpl_prelude << "\n";
  for (int i = 0; i < d->n_types; ++i)
    s << "typedef " << d->type_names[i] << " SCL_TYPE_" << i << ";\n";
  if (kind == SCL_KIND_MAP_INDEX || kind == SCL_KIND_MAP_INDEX_VOID)
    s << "typedef size_t Index;\n";
  if (point) s << "typedef struct { size_t x; size_t y; } IndexPoint;\n";
  if (folds(kind) || kind == SCL_KIND_ALLPAIRS)
    s << "#define SCL_IDENTITY (" << (d->identity && *d->identity ? d->identity : "0") << ")\n";
  if (kind == SCL_KIND_MAPOVERLAP) {
    std::string neutral = d->neutral && *d->neutral ? d->neutral : "0";
    p->stencil_px = (d->flags & SCL_PROG_STENCIL_COLS1) ? 1 : ((d->flags & SCL_PROG_STENCIL_COLS2) ? 2 : 4);
    s << "#define SCL_PX " << p->stencil_px << "\n"
      << "#define SCL_OVERLAP_RANGE " << d->overlap_range << "\n"
      << "#define SCL_PADDING " << (d->padding == SCL_PAD_NEAREST ? 1 : 0) << "\n"
      << "#define SCL_NEUTRAL (" << neutral << ")\n"
      << "#define SCL_NEUTRAL_IS_ZERO " << (neutral_is_zero(neutral) ? 1 : 0) << "\n"
      << scl_tpl_mapoverlap_pre << "\n";
  }
  if (kind == SCL_KIND_ALLPAIRS_GENERIC) s << scl_tpl_allpairs_pre << "\n";
  if (d->common_source && *d->common_source)
    s << "// ---- common definitions\n" << strip_opencl_pragmas(d->common_source) << "\n";

  ExtraMacros em;
  p->extra.clear();
  p->n_reduce_extra = 0;
  std::string zip_args, reduce_args;
  if (kind == SCL_KIND_ZIP_REDUCE || kind == SCL_KIND_SCAN_MAP) {
    // the folding function becomes SCL_FUNC (with its FP64 twin), the second
    // USR_ZIP / USR_MAP; extras: the fold's, then the second function's
    const std::string func2 = d->func2 ? d->func2 : "func";
    const std::string src2 = strip_opencl_pragmas(d->source2 ? d->source2 : "");
    const char* second = kind == SCL_KIND_ZIP_REDUCE ? "USR_ZIP" : "USR_MAP";
    const size_t arity2 = kind == SCL_KIND_ZIP_REDUCE ? 2 : 1;
    FuncSig fs, ss;
    if (!parse_function(src, func, &fs, err)) { *err = "fold source: " + *err; return SCL_ERR_COMPILE; }
    if (!parse_function(src2, func2, &ss, err)) { *err = "second source: " + *err; return SCL_ERR_COMPILE; }
    if (fs.params.size() < 2 || ss.params.size() < arity2) {
      *err = "fused skeleton: the fold takes two parameters, the second function " + std::to_string(arity2);
      return SCL_ERR_COMPILE;
    }
    std::vector<Param> fx(fs.params.begin() + 2, fs.params.end());
    std::vector<Param> sx(ss.params.begin() + arity2, ss.params.end());
    const std::string renamed = rename_identifier(src, func, "SCL_FUNC");
    s << "// ---- fold user source\n" << renamed << "\n";
    s << "// ---- second user source\n" << rename_identifier(src2, func2, second) << "\n";
    if (want_f64) {
      FuncSig rsig;
      std::string e2;
      if (parse_function(renamed, "SCL_FUNC", &rsig, &e2)) {
        std::string def = renamed.substr(rsig.def_begin, rsig.def_end - rsig.def_begin);
        def = rename_identifier(def, "float", "double");
        def = rename_identifier(def, "SCL_FUNC", "SCL_FUNC_C");
        s << "// ---- FP64 twin for carries\n" << def << "\n";
      }
    }
    append_extra(fx, 0, &em, &reduce_args);
    append_extra(sx, fx.size(), &em, &zip_args);
    p->extra = fx;
    p->extra.insert(p->extra.end(), sx.begin(), sx.end());
    p->n_reduce_extra = fx.size();
    p->uses_workitem = false;
  } else if (kind == SCL_KIND_ALLPAIRS) {
    const std::string func2 = d->func2 ? d->func2 : "func";
    const std::string src2 = strip_opencl_pragmas(d->source2 ? d->source2 : "");
    FuncSig rs, zs;
    if (!parse_function(src, func, &rs, err)) { *err = "Reduce source: " + *err; return SCL_ERR_COMPILE; }
    if (!parse_function(src2, func2, &zs, err)) { *err = "Zip source: " + *err; return SCL_ERR_COMPILE; }
    if (rs.params.size() < 2 || zs.params.size() < 2) {
      *err = "AllPairs: the Reduce and Zip functions need two parameters each";
      return SCL_ERR_COMPILE;
    }
    std::vector<Param> rx(rs.params.begin() + 2, rs.params.end());
    std::vector<Param> zx(zs.params.begin() + 2, zs.params.end());
    s << "// ---- reduce user source\n" << rename_identifier(src, func, "USR_REDUCE") << "\n";
    s << "// ---- zip user source\n" << rename_identifier(src2, func2, "USR_ZIP") << "\n";
    append_extra(rx, 0, &em, &reduce_args);
    append_extra(zx, rx.size(), &em, &zip_args);
    p->extra = rx;
    p->extra.insert(p->extra.end(), zx.begin(), zx.end());
    p->n_reduce_extra = rx.size();
    p->uses_workitem = false;
    // tensor-core eligibility: zip x*y, reduce x+y, identity 0, all float, no extras
    auto body_is = [](const std::string& text, const FuncSig& sg, const char* op) {
      std::string body = text.substr(sg.def_begin, sg.def_end - sg.def_begin);
      size_t b = body.find('{');
      std::string inner;
      for (char c : body.substr(b)) if (!std::isspace((unsigned char)c)) inner += c;
      const std::string a = sg.params[0].name, bb = sg.params[1].name;
      return inner == std::string("{return") + a + op + bb + ";}" ||
             inner == std::string("{return") + bb + op + a + ";}" ||
             inner == std::string("{return(") + a + op + bb + ");}";
    };
    std::string id = d->identity && *d->identity ? d->identity : "0";
    bool all_float = d->n_types == 3;
    for (int i = 0; i < d->n_types && all_float; ++i) all_float = std::string(d->type_names[i]) == "float";
    p->tc_eligible = all_float && rx.empty() && zx.empty() && neutral_is_zero(id) &&
                     body_is(src, rs, "+") && body_is(src2, zs, "*");
  } else {
    FuncSig sig;
    if (!parse_function(src, func, &sig, err)) return SCL_ERR_COMPILE;
    const int k = skeleton_arity(kind);
    if ((int)sig.params.size() < k) {
      *err = "function '" + func + "' takes " + std::to_string(sig.params.size()) +
             " parameters; the skeleton passes " + std::to_string(k);
      return SCL_ERR_COMPILE;
    }
    std::vector<Param> ex(sig.params.begin() + k, sig.params.end());
    const char* target = (kind == SCL_KIND_MAPOVERLAP || kind == SCL_KIND_ALLPAIRS_GENERIC)
                             ? "USR_FUNC" : "SCL_FUNC";
    std::string renamed = rename_identifier(src, func, target);
    // Stencil taps: unrolled loops let the compiler read each staged input and
    // each weight once per thread across the rows it computes.
    if (kind == SCL_KIND_MAPOVERLAP) renamed = unroll_loops_in(renamed, target);
    std::string second;  // Zip adjoint: the right operand's derivative
    if (kind == SCL_KIND_ZIP_ADJOINT && d->func2 && *d->func2) {
      const std::string func2 = d->func2;
      const bool own = d->source2 && *d->source2;
      const std::string src2 = own ? strip_opencl_pragmas(d->source2) : renamed;
      FuncSig sig2;
      if (!parse_function(src2, func2, &sig2, err)) { *err = "right derivative: " + *err; return SCL_ERR_COMPILE; }
      if (sig2.params.size() != sig.params.size()) {
        *err = "the two derivative functions must take the same parameters (x, y, g, extra...)";
        return SCL_ERR_COMPILE;
      }
      if (own) second = rename_identifier(src2, func2, "SCL_FUNC2");
      else renamed = rename_identifier(renamed, func2, "SCL_FUNC2");
      s << "#define SCL_HAS_FUNC2 1\n";
    }
    s << "// ---- user source\n" << renamed << "\n";
    if (!second.empty()) s << "// ---- right derivative source\n" << second << "\n";
    p->uses_workitem = source_uses_workitem(src);
    if (want_f64) {
      // FP64 twin of the user function for cross-block carries
      FuncSig rsig;
      std::string e2;
      if (parse_function(renamed, target, &rsig, &e2)) {
        std::string def = renamed.substr(rsig.def_begin, rsig.def_end - rsig.def_begin);
        def = rename_identifier(def, "float", "double");
        def = rename_identifier(def, target, "SCL_FUNC_C");
        s << "// ---- FP64 twin for carries\n" << def << "\n";
      }
    }
    append_extra(ex, 0, &em, nullptr);
    p->extra = ex;
  }
  s << "#define SCL_EXTRA_PARAMS " << em.params << "\n"
    << "#define SCL_USER_PARAMS " << em.user << "\n"
    << "#define SCL_EXTRA_SETUP SCL_GRID_DEPENDENCY_WAIT " << em.setup << "\n"
    << "#define SCL_EXTRA_ARGS " << em.args << "\n"
    << "#define SCL_REDUCE_ARGS " << reduce_args << "\n"
    << "#define SCL_ZIP_ARGS " << zip_args << "\n";
  // the fold's own extra arguments, and the second function's (fused kinds)
  if (kind == SCL_KIND_ZIP_REDUCE || kind == SCL_KIND_SCAN_MAP)
    s << "#define SCL_OP_ARGS SCL_REDUCE_ARGS\n#define SCL_SECOND_ARGS SCL_ZIP_ARGS\n";
  else
    s << "#define SCL_OP_ARGS SCL_EXTRA_ARGS\n#define SCL_SECOND_ARGS\n";
  if (folds(kind)) {
    if (want_f64) s << "typedef double SCL_CARRY_T;\n";
    else s << "typedef SCL_TYPE_" << (kind == SCL_KIND_ZIP_REDUCE ? 2 : 0)
           << " SCL_CARRY_T;\n#define SCL_FUNC_C SCL_FUNC\n";
  }
  s << "// ---- skeleton template\n";
  switch (kind) {
    case SCL_KIND_MAP: case SCL_KIND_MAP_VOID: case SCL_KIND_MAP_INDEX:
    case SCL_KIND_MAP_INDEX_VOID: case SCL_KIND_MAP_POINT: case SCL_KIND_MAP_POINT_VOID:
    case SCL_KIND_ZIP: case SCL_KIND_ZIP_VOID:
    case SCL_KIND_MAP_ADJOINT: case SCL_KIND_ZIP_ADJOINT:
      s << scl_tpl_elementwise;
      out->kernels = {"scl_map_k<1>", "scl_map_k<2>", "scl_map_k<4>", "scl_map_simple"};
      break;
    case SCL_KIND_REDUCE:
      s << scl_tpl_reduce;
      out->kernels = {"scl_reduce_k<8>", "scl_reduce_k<4>"};
      out->lazy = {"scl_reduce_k<1>", "scl_reduce_k<2>", "scl_reduce_seg<32>", "scl_reduce_seg<8>",
                   "scl_reduce_seg<32, 1>", "scl_reduce_seg<8, 1>",
                   "scl_reduce_short<8>"};
      break;
    case SCL_KIND_SCAN:
      s << scl_tpl_reduce << "\n" << scl_tpl_scan;
      out->kernels = {"scl_scan_s<8, 6>", "scl_scan_k<8, 4>"};
      out->lazy = {"scl_scan_k<8, 3>", "scl_scan_k<8, 2>", "scl_scan_k<4, 4>", "scl_scan_k<4, 6>",
                   "scl_scan_k<2, 8>", "scl_scan_k<16, 2>", "scl_scan_k<16, 1>",
                   "scl_scan_s<8, 5>", "scl_scan_s<8, 4>", "scl_scan_s<4, 8>", "scl_scan_s<6, 8>",
                   "scl_scan_s<16, 3>", "scl_scan_s<8, 6, 1>", "scl_scan_s<16, 3, 1>",
                   "scl_scan_s<8, 6, 2>", "scl_scan_s<16, 3, 2>", "scl_scan_short<8>"};
      break;
    case SCL_KIND_ZIP_REDUCE:
      s << scl_tpl_reduce;
      out->kernels = {"scl_zipreduce_k<1>", "scl_zipreduce_k<2>", "scl_zipreduce_k<4>"};
      break;
    case SCL_KIND_SCAN_MAP:
      s << scl_tpl_reduce << "\n" << scl_tpl_scan;
      out->kernels = {"scl_scan_s<8, 6>"};
      out->lazy = {"scl_scan_s<8, 5>", "scl_scan_s<8, 4>", "scl_scan_s<4, 8>", "scl_scan_s<6, 8>",
                   "scl_scan_s<16, 3>", "scl_scan_s<8, 6, 1>", "scl_scan_s<16, 3, 1>",
                   "scl_scan_s<8, 6, 2>", "scl_scan_s<16, 3, 2>", "scl_scan_short<8>"};
      break;
    case SCL_KIND_MAPOVERLAP:
      s << scl_tpl_mapoverlap;
      // the default rows per thread: 4 with four columns, else 8
      if (p->stencil_px == 4) {
        out->kernels = {"scl_mapoverlap_tma<4>"};
        out->lazy = {"scl_mapoverlap_ldst<4>", "scl_mapoverlap_tma<8>", "scl_mapoverlap_ldst<8>",
                     "scl_mapoverlap_tma<16>"};
      } else {
        out->kernels = {"scl_mapoverlap_tma<8>"};
        out->lazy = {"scl_mapoverlap_ldst<4>", "scl_mapoverlap_tma<4>", "scl_mapoverlap_ldst<8>",
                     "scl_mapoverlap_tma<16>"};
      }
      break;
    case SCL_KIND_ALLPAIRS:
      s << scl_tpl_allpairs;
      out->kernels = {"scl_allpairs_simt"};
      break;
    case SCL_KIND_ALLPAIRS_GENERIC:
      s << scl_tpl_allpairs;
      out->kernels = {"scl_allpairs_generic"};
      break;
    default:
      *err = "unknown skeleton kind " + std::to_string(kind);
      return SCL_ERR_ARG;
  }
  // element / carry sizes, read back by the host after the module loads
  s << "\nextern \"C\" __device__ const unsigned int scl_type_sizes[5] = {";
  for (int i = 0; i < 3; ++i)
    s << (i < d->n_types ? "(unsigned int)sizeof(SCL_TYPE_" + std::to_string(i) + ")" : std::string("0u")) << ", ";
  s << (folds(kind) ? "(unsigned int)sizeof(SCL_CARRY_T)" : "0u")
    << ", " << ((kind == SCL_KIND_SCAN || kind == SCL_KIND_SCAN_MAP)
                    ? "(unsigned int)scl_status_mode<SCL_CARRY_T>::value" : "0u")
    << "};\n";
  out->source = s.str();
  return SCL_OK;
}

const char* kNvrtcOpts[] = {"-arch=sm_103a", "-std=c++17", "-default-device",
                            "-diag-suppress=177,550,174,1835", "-lineinfo"};
const int kNvrtcOptCount = 5;

std::mutex g_cache_mu;
std::map<std::string, std::pair<std::string, std::map<std::string, std::string>>> g_mem_cache;

std::string cache_dir() {
  std::string d = env("SKELCL_CACHE_DIR");
  if (!d.empty()) return d;
  std::string home = env("HOME");
  return (home.empty() ? std::string("/tmp") : home) + "/.cache/skelcl_gb300";
}

// Counters of the compile cache (scl_cache_stats).
std::atomic<uint64_t> g_nvrtc_compiles{0}, g_disk_loads{0}, g_disk_rejects{0}, g_disk_saves{0};

std::string cache_file(const std::string& key) { return cache_dir() + "/" + key + ".sm_103a.skelcl"; }

// Serialised cache entry (text header, then the cubin):
//   SCLBIN2 \n key \n n_names \n (name \n lowered name \n)* cubin_bytes sha1(cubin) \n cubin
// A file that is not exactly this -- another format or key, a name list
// that does not parse, fewer or more cubin bytes than recorded, a cubin whose
// SHA-1 differs or that is not an ELF image -- is rejected and the program is
// compiled instead (SKELCL_SAVE_BINARY then replaces the file).
bool load_disk(const std::string& key, std::string* cubin,
               std::map<std::string, std::string>* names) {
  std::ifstream f(cache_file(key), std::ios::binary);
  if (!f) return false;  // no entry: not a reject
  auto reject = [&]() {
    g_disk_rejects++;
    names->clear();
    cubin->clear();
    return false;
  };
  std::string magic, k, line;
  if (!std::getline(f, magic) || magic != "SCLBIN2") return reject();
  if (!std::getline(f, k) || k != key) return reject();
  if (!std::getline(f, line)) return reject();
  char* end = nullptr;
  const long n = std::strtol(line.c_str(), &end, 10);
  if (end == line.c_str() || *end != '\0' || n < 1 || n > 4096) return reject();
  std::map<std::string, std::string> got;
  for (long i = 0; i < n; ++i) {
    std::string a, b;
    if (!std::getline(f, a) || !std::getline(f, b) || a.empty() || b.empty()) return reject();
    got[a] = b;
  }
  if (!std::getline(f, line)) return reject();
  const size_t sp = line.find(' ');
  if (sp == std::string::npos) return reject();
  const unsigned long long bytes = std::strtoull(line.substr(0, sp).c_str(), &end, 10);
  const std::string digest = line.substr(sp + 1);
  if (bytes < 4 || bytes > (1ull << 31)) return reject();
  std::string bin((size_t)bytes, '\0');
  f.read(&bin[0], (std::streamsize)bytes);
  if ((unsigned long long)f.gcount() != bytes) return reject();  // truncated
  if (f.peek() != std::char_traits<char>::eof()) return reject();  // trailing bytes
  if (bin.compare(0, 4, "\x7f" "ELF") != 0) return reject();
  if (sha1_hex(bin.data(), bin.size()) != digest) return reject();
  *cubin = std::move(bin);
  *names = std::move(got);
  g_disk_loads++;
  return true;
}

void save_disk(const std::string& key, const std::string& cubin,
               const std::map<std::string, std::string>& names) {
  std::string dir = cache_dir();
  std::string acc;
  for (size_t i = 0; i <= dir.size(); ++i) {
    if (i == dir.size() || dir[i] == '/') {
      if (!acc.empty()) mkdir(acc.c_str(), 0755);
    }
    if (i < dir.size()) acc += dir[i];
  }
  std::string tmp = dir + "/" + key + ".tmp" + std::to_string((unsigned long)getpid());
  {
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return;
    f << "SCLBIN2\n" << key << "\n" << names.size() << "\n";
    for (auto& kv : names) f << kv.first << "\n" << kv.second << "\n";
    f << cubin.size() << " " << sha1_hex(cubin.data(), cubin.size()) << "\n";
    f.write(cubin.data(), (std::streamsize)cubin.size());
    if (!f) {
      f.close();
      std::remove(tmp.c_str());
      return;
    }
  }
  if (std::rename(tmp.c_str(), cache_file(key).c_str()) == 0) g_disk_saves++;
  else std::remove(tmp.c_str());
}

int nvrtc_compile(const Assembly& a, std::string* cubin,
                  std::map<std::string, std::string>* lowered, std::string* log) {
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, a.source.c_str(), "skelcl_program.cu", 0, nullptr, nullptr);
  if (r != NVRTC_SUCCESS) {
    *log = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r);
    return SCL_ERR_COMPILE;
  }
  for (auto& k : a.kernels)
    if (k.find('<') != std::string::npos) nvrtcAddNameExpression(prog, k.c_str());
  r = nvrtcCompileProgram(prog, kNvrtcOptCount, kNvrtcOpts);
  g_nvrtc_compiles++;
  size_t ls = 0;
  nvrtcGetProgramLogSize(prog, &ls);
  std::string lg(ls, '\0');
  if (ls) nvrtcGetProgramLog(prog, &lg[0]);
  while (!lg.empty() && lg.back() == '\0') lg.pop_back();
  *log = lg;
  if (r != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return SCL_ERR_COMPILE;
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin->assign(n, '\0');
  nvrtcGetCUBIN(prog, &(*cubin)[0]);
  for (auto& k : a.kernels) {
    if (k.find('<') != std::string::npos) {
      const char* low = nullptr;
      if (nvrtcGetLoweredName(prog, k.c_str(), &low) == NVRTC_SUCCESS && low) (*lowered)[k] = low;
    } else {
      (*lowered)[k] = k;
    }
  }
  nvrtcDestroyProgram(&prog);
  return SCL_OK;
}

void copy_log(const std::string& s, char* log, size_t cap) {
  if (!log || cap == 0) return;
  size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
  std::memcpy(log, s.data(), n);
  log[n] = '\0';
}

// Everything a cached cubin depends on besides the source and the kernel
// names: the NVRTC options (target sm_103a), NVRTC's version, the ABI
// version of this library and, once a device is open, its compute
// capability and driver version.  The reference names its binaries by
// source hash and device (src/Program.cpp:62-75).
std::string cache_context() {
  std::string k;
  for (int i = 0; i < kNvrtcOptCount; ++i) k += std::string("\n") + kNvrtcOpts[i];
  int major = 0, minor = 0;
  nvrtcVersion(&major, &minor);
  k += "\n#nvrtc " + std::to_string(major) + "." + std::to_string(minor);
  k += "\n#abi " + std::to_string(SCL_ABI_VERSION);
  if (rt().initialized) {
    int drv = 0;
    cudaDriverGetVersion(&drv);
    k += "\n#device cc" + std::to_string(rt().cc_major) + "." + std::to_string(rt().cc_minor) +
         " driver " + std::to_string(drv);
  } else {
    k += "\n#device none";
  }
  return k;
}

// Compile `names` out of `source` (or take them from the in-process / on-disk
// cache).  The cache key covers the source, the names and cache_context().
int compile_cached(const std::string& source, const std::vector<std::string>& names,
                   std::string* cubin, std::map<std::string, std::string>* lowered,
                   std::string* nvlog, std::string* hash) {
  std::string k = source + cache_context();
  for (auto& n : names) k += "\n#name " + n;
  const std::string key = sha1_hex(k.data(), k.size());
  if (hash) *hash = sha1_hex(source.data(), source.size());
  {
    std::lock_guard<std::mutex> g(g_cache_mu);
    auto it = g_mem_cache.find(key);
    if (it != g_mem_cache.end()) {
      *cubin = it->second.first;
      *lowered = it->second.second;
      return SCL_OK;
    }
  }
  if (env_yes("SKELCL_LOAD_BINARY") && load_disk(key, cubin, lowered)) {
    std::lock_guard<std::mutex> g(g_cache_mu);
    g_mem_cache[key] = {*cubin, *lowered};
    return SCL_OK;
  }
  Assembly a;
  a.source = source;
  a.kernels = names;
  lowered->clear();
  int st = nvrtc_compile(a, cubin, lowered, nvlog);
  if (env_yes("SKELCL_PRINT_BUILD_LOG") && !nvlog->empty())
    std::fprintf(stderr, "[skelcl] NVRTC build log:\n%s\n", nvlog->c_str());
  if (st != SCL_OK) return st;
  std::lock_guard<std::mutex> g(g_cache_mu);
  g_mem_cache[key] = {*cubin, *lowered};
  if (env_yes("SKELCL_SAVE_BINARY")) save_disk(key, *cubin, *lowered);
  return SCL_OK;
}

int load_module(scl_program* p, const std::string& cubin,
                const std::map<std::string, std::string>& lowered) {
  Driver& drv = rt().drv;
  CUmodule mod = nullptr;
  CUresult r = drv.cuModuleLoadData(&mod, cubin.data());
  rt().module_loads++;
  if (r != CUDA_SUCCESS) return cu_fail(r, "cuModuleLoadData");
  p->modules.push_back(mod);
  for (auto& kv : lowered) {
    CUfunction fn = nullptr;
    r = drv.cuModuleGetFunction(&fn, mod, kv.second.c_str());
    if (r != CUDA_SUCCESS) return cu_fail(r, ("cuModuleGetFunction " + kv.first).c_str());
    p->kernels[kv.first] = Kernel{fn, kv.second};
  }
  return SCL_OK;
}

}  // namespace

CUfunction find_kernel(scl_program* p, const std::string& name) {
  auto it = p->kernels.find(name);
  if (it != p->kernels.end()) return it->second.fn;
  if (!p->lazy.count(name)) return nullptr;
  // variant compiled on first use (same generated source, one instantiation)
  std::string cubin, nvlog, hash;
  std::map<std::string, std::string> lowered;
  if (compile_cached(p->source, {name}, &cubin, &lowered, &nvlog, &hash) != SCL_OK) {
    fail(SCL_ERR_COMPILE, "NVRTC compilation of " + name + " failed:\n" + nvlog);
    return nullptr;
  }
  if (load_module(p, cubin, lowered) != SCL_OK) return nullptr;
  it = p->kernels.find(name);
  return it == p->kernels.end() ? nullptr : it->second.fn;
}

int ensure_workspace(scl_program* p, size_t bytes, bool fresh) {
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  SCL_CUDA(cudaStreamIsCapturing(rt().stream, &capture));
  const bool capturing = capture != cudaStreamCaptureStatusNone;
  if (p->ws.bytes >= bytes && !fresh) {
    if (capturing) p->ws.recorded = true;
    return SCL_OK;
  }
  if (capturing)
    return fail(SCL_ERR_ARG, "the program's workspace would grow inside a stream capture; make the "
                             "same call once before capturing");
  if (p->ws.ptr) {
    cudaStreamSynchronize(rt().stream);
    if (p->ws.recorded) p->ws.retired.push_back(p->ws.ptr);  // a graph may still use it
    else cudaFree(p->ws.ptr);
    p->ws.ptr = nullptr;
    p->ws.bytes = 0;
    p->ws.recorded = false;
  }
  size_t sz = bytes < 4096 ? 4096 : bytes;
  cudaError_t e = cudaMalloc(&p->ws.ptr, sz);
  rt().device_allocs++;
  if (e != cudaSuccess) return fail(SCL_ERR_OOM, "workspace allocation of " + std::to_string(sz) + " bytes failed");
  // zeroed once: reduce tickets rely on it and reset themselves afterwards
  e = cudaMemset(p->ws.ptr, 0, sz);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(workspace)");
  p->ws.bytes = sz;
  return SCL_OK;
}

}  // namespace scl

using namespace scl;

namespace {
// Builds the program's source and compiles its kernels (every variant when
// `all`, else the eager ones): with FP64 carries when the element type asks
// for them and the eager kernels compile that way, else with carries in the
// element type.  The eager kernels alone decide the carry type, so a lazy
// variant that fails to compile is reported as the error it is instead of
// silently changing the carries of the default kernels.
int compile_program(const scl_program_desc* desc, scl_program* p, bool all, Assembly* a,
                    std::string* cubin, std::map<std::string, std::string>* lowered,
                    std::string* nvlog, std::string* err, bool* f64_used, std::string* hash) {
  const bool want_f64 = wants_f64_carry(desc);
  for (int attempt = 0; attempt < 2; ++attempt) {
    const bool f64 = want_f64 && attempt == 0;
    *a = Assembly();
    int st = assemble(desc, p, f64, a, err);
    if (st != SCL_OK) return st;
    const std::vector<std::string> eager = a->kernels;
    if (all) {
      a->kernels.insert(a->kernels.end(), a->lazy.begin(), a->lazy.end());
      a->lazy.clear();
    }
    lowered->clear();
    st = compile_cached(a->source, a->kernels, cubin, lowered, nvlog, hash);
    if (st == SCL_OK) {
      *f64_used = f64;
      return SCL_OK;
    }
    if (f64 && all) {
      std::string c2, l2;
      std::map<std::string, std::string> w2;
      if (compile_cached(a->source, eager, &c2, &w2, &l2, nullptr) == SCL_OK) {
        *err = "NVRTC compilation of a kernel variant failed:\n" + *nvlog;
        return SCL_ERR_COMPILE;
      }
    }
    if (!f64) break;
  }
  *err = "NVRTC compilation failed:\n" + *nvlog;
  return SCL_ERR_COMPILE;
}

bool compile_all_requested(const scl_program_desc* desc) {
  return (desc->flags & SCL_PROG_COMPILE_ALL) || env_yes("SKELCL_COMPILE_ALL");
}
}  // namespace

extern "C" int scl_sha1_hex(const void* data, size_t bytes, char* out41) {
  if (!out41 || (!data && bytes)) return fail(SCL_ERR_ARG, "scl_sha1_hex: null pointer");
  std::string h = sha1_hex(data, bytes);
  std::memcpy(out41, h.c_str(), 41);
  return SCL_OK;
}

extern "C" int scl_cache_stats(uint64_t* nvrtc_compiles, uint64_t* disk_loads,
                               uint64_t* disk_rejects, uint64_t* disk_saves) {
  if (nvrtc_compiles) *nvrtc_compiles = g_nvrtc_compiles.load();
  if (disk_loads) *disk_loads = g_disk_loads.load();
  if (disk_rejects) *disk_rejects = g_disk_rejects.load();
  if (disk_saves) *disk_saves = g_disk_saves.load();
  return SCL_OK;
}

extern "C" int scl_program_source(const scl_program_desc* desc, char* out, size_t cap,
                                  size_t* needed) {
  if (!desc) return fail(SCL_ERR_ARG, "scl_program_source: null desc");
  scl_program tmp;
  tmp.kind = desc->kind;
  Assembly a;
  std::string err;
  bool f64 = (desc->kind == SCL_KIND_REDUCE || desc->kind == SCL_KIND_SCAN) &&
             desc->n_types >= 1 && desc->type_names[0] &&
             std::string(desc->type_names[0]) == "float" &&
             !(desc->flags & SCL_PROG_NO_F64_CARRY);
  int st = assemble(desc, &tmp, f64, &a, &err);
  if (st != SCL_OK) return fail(st, err);
  if (needed) *needed = a.source.size() + 1;
  if (out && cap) copy_log(a.source, out, cap);
  return SCL_OK;
}

extern "C" int scl_program_build(const scl_program_desc* desc, scl_program** out, char* log,
                                 size_t log_cap) {
  if (!desc || !out) return fail(SCL_ERR_ARG, "scl_program_build: null argument");
  *out = nullptr;
  if (desc->n_types < 0 || desc->n_types > 3) return fail(SCL_ERR_ARG, "n_types out of range");
  for (int i = 0; i < desc->n_types; ++i)
    if (!desc->type_names[i] || !*desc->type_names[i])
      return fail(SCL_ERR_ARG, "missing type name " + std::to_string(i));
  if (desc->kind == SCL_KIND_MAPOVERLAP && (desc->overlap_range < 0 || desc->overlap_range > 64))
    return fail(SCL_ERR_ARG, "overlap range must be in [0, 64]");
  std::unique_ptr<scl_program> p(new scl_program);
  p->kind = desc->kind;
  p->overlap_range = desc->overlap_range;
  p->padding = desc->padding;
  for (int i = 0; i < desc->n_types; ++i) p->type_names.push_back(desc->type_names[i]);

  std::string cubin, nvlog, err;
  std::map<std::string, std::string> lowered;
  Assembly a;
  bool f64 = false;
  // every variant now, none on first use (flag, or SKELCL_COMPILE_ALL=YES)
  if (int st = compile_program(desc, p.get(), compile_all_requested(desc), &a, &cubin, &lowered,
                               &nvlog, &err, &f64, &p->hash)) {
    copy_log(err, log, log_cap);
    return fail(st, err);
  }
  p->f64_carry = f64;
  p->source = a.source;
  for (auto& k : a.lazy) p->lazy.insert(k);
  if (int st = require_init()) {
    copy_log("scl_init() has not been called", log, log_cap);
    return st;
  }
  if (int st = load_module(p.get(), cubin, lowered)) {
    copy_log(scl_last_error_string(), log, log_cap);
    return st;
  }
  {
    CUdeviceptr gp = 0;
    size_t gsz = 0;
    CUresult r = rt().drv.cuModuleGetGlobal(&gp, &gsz, p->modules.front(), "scl_type_sizes");
    if (r != CUDA_SUCCESS) return cu_fail(r, "cuModuleGetGlobal(scl_type_sizes)");
    unsigned int sz[5] = {0, 0, 0, 0, 0};
    cudaError_t e = cudaMemcpy(sz, (const void*)gp, sizeof(sz), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(scl_type_sizes)");
    for (int i = 0; i < desc->n_types; ++i) p->type_sizes.push_back(sz[i]);
    p->carry_size = sz[3];
    p->status_mode = (int)sz[4];
  }
  if (log && log_cap) copy_log(nvlog, log, log_cap);
  *out = p.release();
  return SCL_OK;
}

extern "C" int scl_program_compile(const scl_program_desc* desc, char* log, size_t log_cap) {
  if (!desc) return fail(SCL_ERR_ARG, "scl_program_compile: null desc");
  scl_program tmp;
  tmp.kind = desc->kind;
  std::string err, nvlog, cubin;
  std::map<std::string, std::string> lowered;
  Assembly a;
  bool f64 = false;
  if (int st = compile_program(desc, &tmp, compile_all_requested(desc), &a, &cubin, &lowered, &nvlog,
                               &err, &f64, nullptr)) {
    copy_log(err, log, log_cap);
    return fail(st, err);
  }
  copy_log(nvlog, log, log_cap);
  return SCL_OK;
}

extern "C" int scl_program_release(scl_program* p) {
  if (!p) return SCL_OK;
  if (rt().initialized) {
    cudaStreamSynchronize(rt().stream);
    if (p->ws.ptr) cudaFree(p->ws.ptr);
    for (void* r : p->ws.retired) cudaFree(r);
    for (CUmodule m : p->modules) rt().drv.cuModuleUnload(m);
  }
  delete p;
  return SCL_OK;
}

extern "C" int scl_program_extra_count(const scl_program* p, int* count) {
  if (!p || !count) return fail(SCL_ERR_ARG, "null argument");
  *count = (int)p->extra.size();
  return SCL_OK;
}

extern "C" int scl_program_hash(const scl_program* p, char* out41) {
  if (!p || !out41) return fail(SCL_ERR_ARG, "null argument");
  std::memcpy(out41, p->hash.c_str(), 41);
  return SCL_OK;
}

extern "C" int scl_program_last_variant(const scl_program* p, uint32_t* variant) {
  if (!p || !variant) return fail(SCL_ERR_ARG, "null argument");
  *variant = p->last_variant;
  return SCL_OK;
}
