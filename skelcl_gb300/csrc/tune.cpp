// Launch autotuner (no counterpart in the reference; the reference takes the
// work-group size from Skeleton::setWorkGroupSize only).
//
// When tuning is on (SKELCL_AUTOTUNE=1 in the environment, or
// scl_autotune_set(1)), a launch that passes no tuning of its own, is
// idempotent (its outputs overlap none of its inputs and its extra arguments
// are values only) and is not being captured into a graph is timed once per
// (device, program, skeleton, log2 of the size) over a small set of
// candidate shapes -- block size and items per thread for Map/Zip/Reduce,
// tile shape and variant for Scan, rows per thread and staging for
// MapOverlap -- with CUDA events on the library stream.  The fastest is kept
// in memory and appended to <cache dir>/autotune.tsv, which later processes
// read back.  Every candidate computes the same result.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <sys/stat.h>

#include "internal.h"

namespace scl {
namespace {

std::mutex g_tune_mu;
int g_mode = -1;  // -1: not read from the environment yet
bool g_loaded = false;
std::map<std::string, scl_tuning> g_cache;

std::string tune_file() {
  const char* d = std::getenv("SKELCL_CACHE_DIR");
  std::string dir = d && *d ? d : "";
  if (dir.empty()) {
    const char* h = std::getenv("HOME");
    dir = std::string(h && *h ? h : "/tmp") + "/.cache/skelcl_gb300";
  }
  return dir + "/autotune.tsv";
}

void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  std::ifstream f(tune_file());
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ls(line);
    std::string key;
    scl_tuning t{};
    if (std::getline(ls, key, '\t') && (ls >> t.workgroup >> t.items >> t.tile_w >> t.tile_h >> t.variant))
      g_cache[key] = t;
  }
}

void append_locked(const std::string& key, const scl_tuning& t) {
  const std::string path = tune_file();
  const std::string dir = path.substr(0, path.rfind('/'));
  for (size_t i = 1; i <= dir.size(); ++i)  // create the directory chain
    if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
  std::ofstream f(path, std::ios::app);
  if (f) f << key << '\t' << t.workgroup << ' ' << t.items << ' ' << t.tile_w << ' ' << t.tile_h << ' '
           << t.variant << '\n';
}

}  // namespace

bool autotune_enabled() {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (g_mode < 0) {
    const char* e = std::getenv("SKELCL_AUTOTUNE");
    const std::string v = e ? e : "";
    g_mode = (v == "1" || v == "YES" || v == "yes" || v == "ON" || v == "on") ? 1 : 0;
  }
  return g_mode == 1;
}

bool tune_lookup(const std::string& key, scl_tuning* out) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  load_locked();
  auto it = g_cache.find(key);
  if (it == g_cache.end()) return false;
  *out = it->second;
  return true;
}

void tune_store(const std::string& key, const scl_tuning& t) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  load_locked();
  g_cache[key] = t;
  append_locked(key, t);
}

bool untuned(const scl_tuning* t) {
  return !t || (t->workgroup == 0 && t->items == 0 && t->tile_w == 0 && t->tile_h == 0 && t->variant == 0);
}

int tuned_launch(scl_program* p, const char* skel, uint64_t size, const scl_tuning* tu, bool safe,
                 const std::vector<scl_tuning>& cands,
                 const std::function<int(const scl_tuning*)>& run) {
  if (!p || cands.empty() || !untuned(tu) || !autotune_enabled()) return run(tu);
  int bucket = 0;
  while (bucket < 63 && (1ull << (bucket + 1)) <= size) ++bucket;
  const std::string key = rt().name + "|" + p->hash + "|" + skel + "|" + std::to_string(bucket);
  const uint32_t spin = tu ? tu->spin_limit : 0;
  scl_tuning best{};
  if (tune_lookup(key, &best)) {
    best.spin_limit = spin;
    return run(&best);
  }
  if (!safe || rt().capturing) return run(tu);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return run(tu);
  }
  float best_ms = 0.0f;
  bool found = false;
  for (scl_tuning c : cands) {
    c.spin_limit = spin;
    if (run(&c) != SCL_OK) continue;  // warm-up (compiles a lazy variant); skip unusable shapes
    cudaEventRecord(e0, rt().stream);
    int st = SCL_OK;
    for (int k = 0; k < 3 && st == SCL_OK; ++k) st = run(&c);
    cudaEventRecord(e1, rt().stream);
    if (st != SCL_OK || cudaEventSynchronize(e1) != cudaSuccess) continue;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (!found || ms < best_ms) {
      best_ms = ms;
      best = c;
      found = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!found) return run(tu);
  best.spin_limit = 0;
  tune_store(key, best);
  best.spin_limit = spin;
  return run(&best);
}

}  // namespace scl

using namespace scl;

extern "C" int scl_autotune_set(int mode) {
  autotune_enabled();  // reads the environment once
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_mode = mode ? 1 : 0;
  return SCL_OK;
}

extern "C" int scl_autotune_get(int* mode) {
  if (!mode) return fail(SCL_ERR_ARG, "null pointer");
  *mode = autotune_enabled() ? 1 : 0;
  return SCL_OK;
}
