// Internal declarations shared by the libskelcl_cuda.so translation units.
#ifndef SKELCL_GB300_INTERNAL_H_
#define SKELCL_GB300_INTERNAL_H_

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "skelcl_cuda.h"

namespace scl {

// ---- error reporting ------------------------------------------------------
int fail(int status, const std::string& msg);  // records msg, returns status
int cuda_fail(cudaError_t e, const char* what);
int cu_fail(CUresult r, const char* what);

#define SCL_CUDA(call)                                  \
  do {                                                  \
    cudaError_t scl_e_ = (call);                        \
    if (scl_e_ != cudaSuccess) return ::scl::cuda_fail(scl_e_, #call); \
  } while (0)
#define SCL_CU(call)                                    \
  do {                                                  \
    CUresult scl_r_ = (call);                           \
    if (scl_r_ != CUDA_SUCCESS) return ::scl::cu_fail(scl_r_, #call); \
  } while (0)

// ---- driver entry points (resolved through the runtime, no -lcuda) --------
struct Driver {
  CUresult (*cuModuleLoadData)(CUmodule*, const void*) = nullptr;
  CUresult (*cuModuleUnload)(CUmodule) = nullptr;
  CUresult (*cuModuleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*cuModuleGetGlobal)(CUdeviceptr*, size_t*, CUmodule, const char*) = nullptr;
  CUresult (*cuFuncSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
  CUresult (*cuFuncGetAttribute)(int*, CUfunction_attribute, CUfunction) = nullptr;
  CUresult (*cuLaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned,
                             unsigned, unsigned, unsigned, CUstream, void**,
                             void**) = nullptr;
  CUresult (*cuLaunchKernelEx)(const CUlaunchConfig*, CUfunction, void**, void**) = nullptr;
  CUresult (*cuOccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int,
                                                          size_t) = nullptr;
  CUresult (*cuFuncGetParamInfo)(CUfunction, size_t, size_t*, size_t*) = nullptr;
  CUresult (*cuTensorMapEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t,
                                     void*, const cuuint64_t*, const cuuint64_t*,
                                     const cuuint32_t*, const cuuint32_t*,
                                     CUtensorMapInterleave, CUtensorMapSwizzle,
                                     CUtensorMapL2promotion,
                                     CUtensorMapFloatOOBfill) = nullptr;
  CUresult (*cuGetErrorString)(CUresult, const char**) = nullptr;
};

// ---- global runtime state -------------------------------------------------
struct Runtime {
  bool initialized = false;
  int device = 0;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
  size_t global_mem = 0;
  std::string name;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_streams[2] = {nullptr, nullptr};  // transfers that overlap launches
  unsigned int* dev_err = nullptr;   // device-side status word
  unsigned int* host_err = nullptr;  // pinned mirror
  uint64_t launches = 0;
  // Template kernels are launched with programmatic stream serialization: a
  // kernel's blocks may be scheduled while the previous kernel in the stream
  // drains, and each waits (griddepcontrol.wait, its first statement) until
  // that kernel has completed.  Off with SKELCL_PDL=0 or scl_pdl_set(0).
  bool pdl = true;
  uint64_t pdl_launches = 0;
  uint64_t device_allocs = 0;  // device allocations made by the library (scl_alloc included)
  uint64_t module_loads = 0;   // cubins loaded
  bool capturing = false;
  Driver drv;
};
Runtime& rt();
int require_init();

// ---- splicer ----------------------------------------------------------------
enum class ParamKind { Value, Buffer, Matrix, Local };
struct Param {
  std::string type;   // declared type text (qualifiers kept)
  std::string name;   // parameter name
  ParamKind kind = ParamKind::Value;
  std::string elem;   // Matrix: element type spelling; Local: pointee type
};
struct FuncSig {
  std::string ret;
  std::vector<Param> params;
  size_t def_begin = 0;  // offset of the return type in the source
  size_t def_end = 0;    // one past the closing brace of the body
};
bool parse_function(const std::string& src, const std::string& name, FuncSig* sig,
                    std::string* err);
std::string rename_identifier(const std::string& src, const std::string& from,
                              const std::string& to);
bool source_uses_workitem(const std::string& src);
// Adds `#pragma unroll` before every for-loop of function `name` (a hint
// only: the loops keep their meaning).
std::string unroll_loops_in(const std::string& src, const std::string& name);
std::string sha1_hex(const void* data, size_t n);

// ---- programs -----------------------------------------------------------------
struct Kernel {
  CUfunction fn = nullptr;
  std::string name;
};

struct Workspace {  // per-program scratch (reduce partials, scan tile status)
  void* ptr = nullptr;
  size_t bytes = 0;
  // A launch recorded into a CUDA graph keeps this allocation's address: when
  // it must grow (or change layout) afterwards it is retired, not freed, so
  // the graph stays valid; retired allocations are freed with the program.
  bool recorded = false;
  std::vector<void*> retired;
  // Scan status (scan.cuh): tiles per region, the allocation that layout
  // was cleared in, launches made since, and the slots the last launch in
  // each of the two alternating regions may have written
  uint64_t scan_cap = 0;
  void* scan_layout = nullptr;
  uint64_t scan_epoch = 0;
  uint64_t scan_used[2] = {0, 0};
};

// Scan status layout (scan.cuh): three regions of `cap` tiles, each a
// 128-byte ticket line followed by one 128-byte line per tile (modes 1, 2)
// or [flags | aggregates | inclusive prefixes] (mode 0).  Eager launches
// alternate between regions 0 and 1, each clearing the other for the next
// launch; a launch recorded into a graph uses region 2, which the graph
// clears before the kernel.  Zeroed once per layout.
size_t scan_region_bytes(int status_mode, size_t carry, uint64_t cap);
size_t scan_status_bytes(int status_mode, size_t carry, uint64_t cap);
// Bytes at the start of a region that must be zero before a launch of
// `tiles` tiles uses it (ticket line and status words / flags).
size_t scan_region_clear_bytes(int status_mode, uint64_t tiles);
// Kernel arguments (scan.cuh's scl_scan_status and scl_scan_clear).
struct ScanStatusArgs {
  void* slots;
  void* flags;
  void* agg;
  void* incl;
};
struct ScanClearArgs {
  void* slots;
  void* flags;
  void* ticket;
  uint64_t n;
};
// Region `r` of a layout at `base`: its ticket word and status pointers.
ScanStatusArgs scan_region(void* base, int status_mode, size_t carry, uint64_t cap, int r,
                           void** ticket);
// Tiles of `tile` elements a scan of n elements at `in` launches (the staged
// kernel lays them on the 16-byte grid of `in`: scan_grid gives the grid).
void scan_grid(const void* in, size_t tsz, bool staged, uint64_t* vg, uint64_t* a);
uint64_t scan_tiles(const void* in, size_t tsz, uint64_t n, uint64_t tile, bool staged, bool reverse);

}  // namespace scl

struct scl_program {
  int kind = 0;
  std::string hash;
  std::string source;                       // generated CUDA source
  std::vector<scl::Param> extra;            // user extra params (Reduce's then Zip's for AllPairs)
  size_t n_reduce_extra = 0;                // AllPairs: how many of `extra` belong to the Reduce
  std::vector<size_t> type_sizes;           // sizeof SCL_TYPE_n (read from the module)
  size_t carry_size = 0;                    // sizeof SCL_CARRY_T (Reduce / Scan)
  int status_mode = 0;                      // Scan tile-status encoding (see scan.cuh)
  std::vector<std::string> type_names;
  bool uses_workitem = false;
  bool f64_carry = false;
  bool tc_eligible = false;                 // AllPairs: zip == x*y, reduce == x+y, id 0, float
  int overlap_range = 0;
  int padding = 0;
  int stencil_px = 1;                       // MapOverlap: output columns per thread
  std::vector<CUmodule> modules;            // the first holds scl_type_sizes
  std::map<std::string, scl::Kernel> kernels;  // by template name expression
  std::set<std::string> lazy;               // variants compiled on first use
  scl::Workspace ws;
  uint32_t last_variant = 0;
};

namespace scl {
CUfunction find_kernel(scl_program* p, const std::string& name);
// At least `bytes` of workspace (a new, zeroed allocation when it grows, or
// when `fresh`).  Inside a stream capture it only notes that a graph now
// uses the allocation; growing there is refused.
int ensure_workspace(scl_program* p, size_t bytes, bool fresh = false);

// Kernel parameters of one launch (launch.cpp)
struct ArgPack {
  std::vector<void*> ptrs;
  uint32_t vals[64];  // storage for values built here (Local offsets)
  int nvals = 0;
  size_t local_bytes = 0;
};
// Appends the user function's extra arguments from the ABI blob to `pack`,
// checking them against the program's parameters; `fixed` = skeleton
// parameters already in `pack`.
int pack_extra(scl_program* p, CUfunction fn, size_t fixed, const unsigned char* blob,
               size_t bytes, ArgPack* pack);
// cuLaunchKernel on the library stream.
int launch(CUfunction fn, dim3 grid, dim3 block, size_t smem, ArgPack& pack);

// Device status word bits (bit 0: a bounded wait gave up, set by the
// generated kernels).
constexpr unsigned int kDevErrSegments = 2u;  // segment offsets decreasing or past the end
// Pre-pass of segmented launches (segments.cu): clamped offsets (segment s
// is read as [off[s], max(off[s], off[s+1]))) and the first tile of every
// segment longer than short_max (tile_start[n_seg] = tile count; shorter ones
// get none); tiles of `tile` elements laid on the grid {a + k*vg} (vg = 1:
// from the segment start).  `scratch` holds segments_prepare_scratch(n_seg)
// bytes.
constexpr uint64_t kSegShort = 4096;  // longest segment one warp handles
size_t segments_prepare_scratch(uint64_t n_seg);
int segments_prepare(const uint64_t* seg_offsets, uint64_t n_seg, uint64_t n_total, uint64_t tile,
                     uint64_t vg, uint64_t a, int reverse, uint64_t short_max, uint64_t* off_out,
                     unsigned int* tile_start, uint64_t* scratch, cudaStream_t stream);
// Segment plans (segments.cu, scl_segplan_create): the clamped offsets of
// one segmented vector, the segmented Reduce's per-segment tickets (zero
// between launches: the last tile of a segment resets its ticket), and per
// tile shape the tile numbering with its exact tile count and the window
// records of the short segments.
struct SegPlanCfg {
  uint64_t tile = 0, vg = 1, a = 0, short_max = 0;
  int reverse = 0;
  unsigned int* tile_start = nullptr;  // device, n_seg + 1
  uint64_t tiles = 0;                  // tile_start[n_seg]
  unsigned int* tile_seg = nullptr;    // device, `tiles` entries: each tile's segment
  // window records of the short segments (device, 4 words each: first
  // segment, end segment, first element, elements), one block each
  uint64_t n_rec = 0;
  uint64_t* win_rec = nullptr;
};
struct SegPlan {
  uint32_t id = 0;
  uint64_t n_seg = 0, n_total = 0;
  uint64_t* off = nullptr;
  unsigned int* tickets = nullptr;
  uint64_t* scratch = nullptr;
  std::deque<SegPlanCfg> cfgs;  // (stable addresses)
};
// The window records a segment plan makes of its short segments (four words
// each: first segment, end segment, first element, elements).
void segplan_window_records(const uint64_t* off, uint64_t n_seg, uint64_t short_max,
                            std::vector<uint64_t>* rec);

SegPlan* segplan_find(uint32_t id);
// The plan's tile numbering for one tile shape, built on first use (three
// small launches and a read-back of the tile count; refused inside a stream
// capture).
int segplan_config(SegPlan* p, uint64_t tile, uint64_t vg, uint64_t a, int reverse, uint64_t short_max,
                   const SegPlanCfg** out);
// Autotuner (tune.cpp): lookup/store of the (device, program, skeleton, size
// bucket) cache, and the launch wrapper that times `cands` on a miss.
bool tune_lookup(const std::string& key, scl_tuning* out);
void tune_store(const std::string& key, const scl_tuning& t);
bool autotune_enabled();
bool untuned(const scl_tuning* t);  // null or only spin_limit set
int tuned_launch(scl_program* p, const char* skel, uint64_t size, const scl_tuning* tu, bool safe,
                 const std::vector<scl_tuning>& cands,
                 const std::function<int(const scl_tuning*)>& run);
}  // namespace scl

#endif  // SKELCL_GB300_INTERNAL_H_
