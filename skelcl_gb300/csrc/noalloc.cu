// scl_launch_scan_noalloc: the single-pass scan of scl_launch_scan with its
// scratch in a fixed device array instead of a per-program allocation, for
// callers that must not allocate device memory (their GPU memory belongs to
// another allocator, or they cannot afford cudaFree's device-wide wait).
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"

// The scan's tile counter (first 256 bytes) and per-tile status.  One array
// per GPU that loads this library, held until the process exits and shared
// by every call.  In host code this name is the host-side stand-in for the
// array, not a device address: kernels get the address looked up below.
static __device__ __align__(256) unsigned char scl_noalloc_scratch[SCL_NOALLOC_SCRATCH_BYTES];

namespace scl {
namespace {

constexpr int kMaxDevices = 64;
constexpr size_t kCounterBytes = 256;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kMaxDevices] = {};

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

// Scratch bytes for `tiles` tiles in the layout of scl_launch_scan (one
// status half: every call starts from a cleared array, so the kernel only
// ever uses half 0): [control words | status], the status being one 128-byte
// line per tile (carries of at most 4 bytes, or double) or [flags |
// aggregates | inclusive prefixes].  `clear` receives the bytes that must
// start at zero.
size_t scratch_bytes(int status_mode, size_t carry, uint64_t tiles, size_t* clear) {
  if (status_mode != 0) {
    *clear = kCounterBytes + round256(tiles * 128);
    return *clear;
  }
  *clear = kCounterBytes + round256(tiles * 4);
  return *clear + 2 * round256(tiles * carry);
}

// Device address of the array on `device`, looked up once per device with
// that device current.
int scratch_address(int device, void** out) {
  if (device < 0 || device >= kMaxDevices)
    return fail(SCL_ERR_ARG, "device index beyond the no-allocation scratch table");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    int current = -1;
    SCL_CUDA(cudaGetDevice(&current));
    if (current != device) SCL_CUDA(cudaSetDevice(device));
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, scl_noalloc_scratch);
    if (current != device) cudaSetDevice(current);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scl_noalloc_scratch)");
    if (!ptr || (reinterpret_cast<uintptr_t>(ptr) & 255u) != 0)
      return fail(SCL_ERR_CUDA, "no-allocation scratch: unexpected device address");
    g_noalloc_addr[device] = ptr;
  }
  *out = g_noalloc_addr[device];
  return SCL_OK;
}

}  // namespace
}  // namespace scl

using namespace scl;

extern "C" int scl_launch_scan_noalloc(scl_program* p, const scl_shape* sh, void* const* bufs,
                                       const void* extra, size_t extra_bytes,
                                       const scl_tuning* tu) {
  if (int st = require_init()) return st;
  if (!p) return fail(SCL_ERR_ARG, "null program");
  if (p->kind != SCL_KIND_SCAN)
    return fail(SCL_ERR_ARG, "scl_launch_scan_noalloc needs a Scan program");
  if (!sh || !bufs || !bufs[0] || !bufs[1]) return fail(SCL_ERR_ARG, "scan needs {in, out}");
  if (sh->n_segments)
    return fail(SCL_ERR_UNSUPPORTED,
                "scl_launch_scan_noalloc scans one vector; segmented scans need scl_launch_scan");
  void* in = bufs[0];
  void* out = bufs[1];
  uint64_t n = sh->n;
  const unsigned int flags = sh->flags & (SCL_SHAPE_INCLUSIVE | SCL_SHAPE_REVERSE);
  const bool reverse = (flags & SCL_SHAPE_REVERSE) != 0;
  const size_t tsz = p->type_sizes[0], csz = p->carry_size ? p->carry_size : tsz;
  const uint64_t V = (tsz <= 16 && 16 % tsz == 0) ? 16 / tsz : 1;  // as the kernel's scl_vec_width
  const uint64_t tile = 8 * 256 * V;                                 // 8 rows x 256 threads
  // scl_launch_scan's default kernel (the tile staged in shared memory), or
  // the register kernel when the tile does not fit in shared memory
  const size_t smem = (size_t)tile * tsz;
  const bool staged = smem + 2048 <= rt().smem_optin;
  const uint64_t tiles = scan_tiles(in, tsz, n, tile, staged, reverse);

  // size check before anything touches the GPU
  const uint64_t cap = SCL_NOALLOC_SCRATCH_BYTES;
  size_t clear = 0;
  bool fits = tiles <= cap / 4 && scratch_bytes(p->status_mode, csz, tiles, &clear) <= cap;
  if (!fits) {
    uint64_t lo = 0, hi = cap / 4;  // largest tile count that fits
    while (lo < hi) {
      uint64_t mid = (lo + hi + 1) / 2;
      size_t c;
      if (scratch_bytes(p->status_mode, csz, mid, &c) <= cap) lo = mid; else hi = mid - 1;
    }
    // an input that does not start on a 16-byte boundary may need one tile
    // more (the staged kernel lays tiles on the 16-byte grid)
    return fail(SCL_ERR_ARG, "scl_launch_scan_noalloc: " + std::to_string(n) + " elements of " +
                                 std::to_string(tsz) + " bytes need more than the fixed " +
                                 std::to_string(cap) + "-byte scratch; it holds at most " +
                                 std::to_string(lo * tile) +
                                 " elements of this type starting on a 16-byte boundary (" +
                                 std::to_string(lo > 0 ? (lo - 1) * tile : 0) +
                                 " otherwise; scl_launch_scan has no such limit)");
  }
  if (n == 0) return SCL_OK;
  if (tiles > 0x7fffffffull) return fail(SCL_ERR_ARG, "scan input too large");

  // only kernels loaded when the program was built: no module load here
  const char* kname = staged ? "scl_scan_s<8, 6>" : "scl_scan_k<8, 4>";
  auto it = p->kernels.find(kname);
  if (it == p->kernels.end() || !it->second.fn)
    return fail(SCL_ERR_LAUNCH, std::string("kernel ") + kname + " missing from the program");
  CUfunction fn = it->second.fn;

  void* base = nullptr;
  if (int st = scratch_address(rt().device, &base)) return st;
  // one status region of `tiles` tiles after the ticket line, cleared by
  // every call (nothing for the kernel to clear for a next launch)
  ScanStatusArgs sargs = {nullptr, nullptr, nullptr, nullptr};
  ScanClearArgs clr = {nullptr, nullptr, nullptr, 0};
  char* b = static_cast<char*>(base);
  if (p->status_mode != 0) {
    sargs.slots = b + kCounterBytes;
  } else {
    const size_t fl = round256(tiles * 4), vals = round256(tiles * csz);
    sargs.flags = b + kCounterBytes;
    sargs.agg = b + kCounterBytes + fl;
    sargs.incl = b + kCounterBytes + fl + vals;
  }
  void* ticket = base;
  // the previous call left its ticket and status behind
  SCL_CUDA(cudaMemsetAsync(base, 0, clear, rt().stream));

  unsigned int fl = flags;
  int aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0;
  unsigned int spin = (tu && tu->spin_limit) ? tu->spin_limit : (1u << 22);
  unsigned int* err = rt().dev_err;
  const void* seg_off = nullptr;
  const void* tile_start = nullptr;
  uint64_t n_seg = 0, short_max = 0;
  unsigned int no_tiles = ~0u;  // (not segmented: unused)
  ArgPack pack;
  pack.ptrs = {&in, &out, &n, &fl, &aligned, &ticket, &sargs, &clr, &spin, &err};
  if (staged) {
    pack.ptrs.push_back(&seg_off);
    pack.ptrs.push_back(&tile_start);
    pack.ptrs.push_back(&n_seg);
    pack.ptrs.push_back(&short_max);
    pack.ptrs.push_back(&tile_start);  // (no window table)
    pack.ptrs.push_back(&tile_start);  // (no tile owners)
    pack.ptrs.push_back(&no_tiles);
  }
  if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
    return st;
  p->last_variant = staged ? SCL_VARIANT_TMA : SCL_VARIANT_VECTOR;
  return launch(fn, dim3((unsigned)tiles), dim3(256), staged ? smem : 0, pack);
}
