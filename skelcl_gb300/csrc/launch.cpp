// Skeleton launches: the GB300 counterparts of the reference's execute()
// bodies (MapDef.h:118-166, ZipDef.h:119-173, ReduceDef.h:164-245,
// ScanDef.h:178-259, MapOverlapDef.h:116-178, AllPairsDef.h:146-210) and of
// the argument marshalling in detail::kernelUtil::setKernelArgs
// (include/SkelCL/detail/KernelUtil.h:132-245).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.h"

// tcgen05 contraction (allpairs_tc.cu)
namespace scl {
int allpairs_tc_launch(const float* A, const float* B, float* P, uint32_t M, uint32_t N,
                       uint32_t K, int parts, int trans, int drain, int wide, uint32_t group_rows,
                       void* scratch, size_t scratch_bytes, cudaStream_t stream, uint32_t spin_limit,
                       unsigned int* err);
// row-major rows x cols -> cols x rows, elements of 4 or 8 bytes (adjoint.cu)
int transpose_launch(const void* src, void* dst, uint64_t rows, uint64_t cols, size_t elem,
                     cudaStream_t stream);
size_t allpairs_tc_scratch_bytes(uint32_t M, uint32_t N, uint32_t K, int parts);
bool allpairs_tc_supported(uint32_t M, uint32_t N, uint32_t K, const void* A, const void* B,
                           const void* P);
}  // namespace scl

namespace scl {
namespace {

constexpr uint32_t kDefaultSpin = 1u << 22;  // polls; ~0.1-1 s with back-off

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

const char* kind_name(uint32_t k) {
  switch (k) {
    case SCL_ARG_VALUE: return "scalar";
    case SCL_ARG_BUFFER: return "Vector";
    case SCL_ARG_MATRIX: return "Matrix";
    case SCL_ARG_LOCAL: return "Local";
    default: return "unknown";
  }
}

}  // namespace

// Walks the blob against program parameters [first, first+count) and appends
// kernel-parameter pointers.  `fixed` = number of skeleton kernel params
// before the extras (for the parameter-size check).
int pack_extra(scl_program* p, CUfunction fn, size_t fixed, const unsigned char* blob,
               size_t bytes, ArgPack* pack) {
  size_t off = 0;
  size_t kparam = fixed;  // kernel parameter index
  const size_t count = p->extra.size();
  for (size_t i = 0; i < count; ++i) {
    if (off + 8 > bytes)
      return fail(SCL_ERR_ARG, "too few extra arguments: the user function declares " +
                                   std::to_string(count) + ", the call passes " + std::to_string(i));
    uint32_t kind, size;
    std::memcpy(&kind, blob + off, 4);
    std::memcpy(&size, blob + off + 4, 4);
    const unsigned char* payload = blob + off + 8;
    size_t rec = 8 + ((size + 7u) & ~7u);
    if (off + rec > bytes) return fail(SCL_ERR_ARG, "truncated extra-argument record");
    const Param& prm = p->extra[i];
    auto mismatch = [&](const char* want) {
      return fail(SCL_ERR_ARG, "extra argument " + std::to_string(i) + " ('" + prm.name +
                                   "'): the user function expects " + want + ", the call passes " +
                                   kind_name(kind));
    };
    switch (prm.kind) {
      case ParamKind::Value: {
        if (kind != SCL_ARG_VALUE) return mismatch("a scalar");
        if (rt().drv.cuFuncGetParamInfo && fn) {
          size_t po = 0, ps = 0;
          if (rt().drv.cuFuncGetParamInfo(fn, kparam, &po, &ps) == CUDA_SUCCESS && ps != size)
            return fail(SCL_ERR_ARG, "extra argument " + std::to_string(i) + " ('" + prm.name +
                                         "'): " + std::to_string(size) + " bytes passed, " +
                                         std::to_string(ps) + " expected");
        }
        pack->ptrs.push_back(const_cast<unsigned char*>(payload));
        ++kparam;
        break;
      }
      case ParamKind::Buffer: {
        if (kind == SCL_ARG_BUFFER) {
          pack->ptrs.push_back(const_cast<unsigned char*>(payload));
          ++kparam;
        } else if (kind == SCL_ARG_MATRIX) {
          // reference form: `__global T* m, uint m_col_count` (KernelUtil.h:189)
          if (i + 1 >= count || p->extra[i + 1].kind != ParamKind::Value)
            return mismatch("a pointer followed by a column count");
          pack->ptrs.push_back(const_cast<unsigned char*>(payload));
          pack->ptrs.push_back(const_cast<unsigned char*>(payload + 8));
          kparam += 2;
          ++i;  // the column-count parameter is consumed
        } else {
          return mismatch("a Vector");
        }
        break;
      }
      case ParamKind::Matrix: {
        if (kind != SCL_ARG_MATRIX) return mismatch("a Matrix");
        pack->ptrs.push_back(const_cast<unsigned char*>(payload));
        pack->ptrs.push_back(const_cast<unsigned char*>(payload + 8));
        kparam += 2;
        break;
      }
      case ParamKind::Local: {
        if (kind != SCL_ARG_LOCAL) return mismatch("Local memory");
        uint64_t lb = 0;
        std::memcpy(&lb, payload, 8);
        size_t o = (pack->local_bytes + 15) & ~(size_t)15;
        if (pack->nvals >= 64) return fail(SCL_ERR_ARG, "too many Local arguments");
        pack->vals[pack->nvals] = (uint32_t)o;
        pack->ptrs.push_back(&pack->vals[pack->nvals]);
        ++pack->nvals;
        pack->local_bytes = o + lb;
        ++kparam;
        break;
      }
    }
    off += rec;
  }
  if (off != bytes)
    return fail(SCL_ERR_ARG, "too many extra arguments: the user function declares " +
                                 std::to_string(count));
  return SCL_OK;
}

int launch(CUfunction fn, dim3 grid, dim3 block, size_t smem, ArgPack& pack) {
  // `smem` is the kernel's own dynamic shared memory; Local arguments
  // (offsets packed from 0) follow it, 16-byte aligned
  if (pack.nvals > 0) {
    const size_t base = (smem + 15) & ~(size_t)15;
    if (base + pack.local_bytes > 0xffffffffull) return fail(SCL_ERR_ARG, "Local arguments too large");
    for (int i = 0; i < pack.nvals; ++i) pack.vals[i] += (uint32_t)base;
    smem = base + pack.local_bytes;
    pack.nvals = 0;  // offsets are final: a second launch of this pack keeps them
  }
  if (smem > 32 * 1024) {  // beyond the default dynamic limit once static smem is counted
    CUresult r = rt().drv.cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                             (int)smem);
    if (r != CUDA_SUCCESS) return cu_fail(r, "cuFuncSetAttribute(max dynamic smem)");
  }
  void** params = pack.ptrs.empty() ? nullptr : pack.ptrs.data();
  if (rt().pdl) {
    // Programmatic stream serialization: this grid may be scheduled while the
    // previous kernel of the stream drains; every template kernel's first
    // statement (SCL_EXTRA_SETUP) waits for that kernel's completion.
    CUlaunchAttribute attr;
    std::memset(&attr, 0, sizeof(attr));
    attr.id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
    attr.value.programmaticStreamSerializationAllowed = 1;
    CUlaunchConfig cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.gridDimX = grid.x;
    cfg.gridDimY = grid.y;
    cfg.gridDimZ = grid.z;
    cfg.blockDimX = block.x;
    cfg.blockDimY = block.y;
    cfg.blockDimZ = block.z;
    cfg.sharedMemBytes = (unsigned)smem;
    cfg.hStream = (CUstream)rt().stream;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    CUresult r = rt().drv.cuLaunchKernelEx(&cfg, fn, params, nullptr);
    if (r != CUDA_SUCCESS) return cu_fail(r, "cuLaunchKernelEx");
    ++rt().launches;
    ++rt().pdl_launches;
    return SCL_OK;
  }
  CUresult r = rt().drv.cuLaunchKernel(fn, grid.x, grid.y, grid.z, block.x, block.y, block.z,
                                       (unsigned)smem, (CUstream)rt().stream, params, nullptr);
  if (r != CUDA_SUCCESS) return cu_fail(r, "cuLaunchKernel");
  ++rt().launches;
  return SCL_OK;
}

namespace {

int max_resident_blocks(CUfunction fn, int block, size_t smem) {
  int per_sm = 0;
  // the query counts only what the function may use: raise its dynamic limit
  // first, as launch() does
  if (smem > 32 * 1024)
    rt().drv.cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem);
  if (rt().drv.cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem) != CUDA_SUCCESS ||
      per_sm < 1)
    per_sm = 1;
  return per_sm * rt().sm_count;
}

int vec_width(size_t s0, size_t s1 = 1, size_t s2 = 1) {
  size_t s = std::max(s0, std::max(s1, s2));
  if (s <= 16 && 16 % s == 0 && 16 % s0 == 0 && 16 % s1 == 0 && 16 % s2 == 0) return (int)(16 / s);
  return 1;
}

uint32_t pick_block(const scl_tuning* t, uint32_t dflt) {
  uint32_t b = (t && t->workgroup) ? t->workgroup : dflt;
  if (b > 1024) b = 1024;
  if (b == 0) b = dflt;
  return b;
}

uint32_t spin_of(const scl_tuning* t) { return (t && t->spin_limit) ? t->spin_limit : kDefaultSpin; }

int check_prog(scl_program* p, std::initializer_list<int> kinds) {
  if (int st = require_init()) return st;
  if (!p) return fail(SCL_ERR_ARG, "null program");
  for (int k : kinds)
    if (p->kind == k) return SCL_OK;
  return fail(SCL_ERR_ARG, "program kind " + std::to_string(p->kind) + " does not match this launch");
}

}  // namespace
}  // namespace scl

using namespace scl;

// ---- Map / Zip ----------------------------------------------------------------
// (the exported scl_launch_* are the autotuning wrappers at the end of this file)
static int launch_map_impl(scl_program* p, const scl_shape* sh, void* const* bufs,
                              const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  if (int st = check_prog(p, {SCL_KIND_MAP, SCL_KIND_MAP_VOID, SCL_KIND_MAP_INDEX,
                              SCL_KIND_MAP_INDEX_VOID, SCL_KIND_MAP_POINT,
                              SCL_KIND_MAP_POINT_VOID, SCL_KIND_ZIP, SCL_KIND_ZIP_VOID,
                              SCL_KIND_MAP_ADJOINT, SCL_KIND_ZIP_ADJOINT}))
    return st;
  if (!sh) return fail(SCL_ERR_ARG, "null shape");
  const int kind = p->kind;
  const bool point = kind == SCL_KIND_MAP_POINT || kind == SCL_KIND_MAP_POINT_VOID;
  int nbuf = 0;
  switch (kind) {
    case SCL_KIND_MAP: nbuf = 2; break;
    case SCL_KIND_MAP_VOID: nbuf = 1; break;
    case SCL_KIND_MAP_INDEX: nbuf = 1; break;
    case SCL_KIND_MAP_POINT: nbuf = 1; break;
    case SCL_KIND_ZIP: nbuf = 3; break;
    case SCL_KIND_ZIP_VOID: nbuf = 2; break;
    case SCL_KIND_MAP_ADJOINT: nbuf = 3; break;  // x, g, gx
    case SCL_KIND_ZIP_ADJOINT: nbuf = 5; break;  // x, y, g, gx, gy
    default: nbuf = 0;
  }
  if (nbuf && !bufs) return fail(SCL_ERR_ARG, "null buffer list");
  void* b[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int i = 0; i < nbuf; ++i) {
    b[i] = bufs[i];
    // the Zip adjoint may skip one of its two gradients
    const bool optional = kind == SCL_KIND_ZIP_ADJOINT && i >= 3;
    if (!b[i] && !optional) return fail(SCL_ERR_ARG, "null device buffer " + std::to_string(i));
  }
  int acc = 0;
  if (kind == SCL_KIND_ZIP_ADJOINT) {
    if (!b[3] && !b[4]) return fail(SCL_ERR_ARG, "Zip adjoint: both gradient buffers are null");
    if (b[4] && p->source.find("#define SCL_HAS_FUNC2") == std::string::npos)
      return fail(SCL_ERR_ARG, "Zip adjoint: a right gradient needs the right derivative (func2)");
    acc = ((sh->flags & SCL_SHAPE_ACCUMULATE) ? 1 : 0) | ((sh->flags & SCL_SHAPE_ACCUMULATE_RIGHT) ? 2 : 0);
  } else if (kind == SCL_KIND_MAP_ADJOINT) {
    acc = (sh->flags & SCL_SHAPE_ACCUMULATE) ? 1 : 0;
  }
  const bool adjoint = kind == SCL_KIND_MAP_ADJOINT || kind == SCL_KIND_ZIP_ADJOINT;
  uint64_t n = sh->n, rows = sh->rows, cols = sh->cols, offset = sh->offset;
  if (point) n = rows * cols;
  if (n == 0) return SCL_OK;
  bool simple = p->uses_workitem || (tu && tu->variant == SCL_VARIANT_SIMPLE);
  int aligned = 1;
  for (int i = 0; i < nbuf; ++i) aligned &= (!b[i] || aligned16(b[i])) ? 1 : 0;
  uint32_t items = (tu && tu->items) ? tu->items : 4;
  if (items != 1 && items != 2 && items != 4) items = 4;
  std::string kname = simple ? "scl_map_simple" : "scl_map_k<" + std::to_string(items) + ">";
  CUfunction fn = find_kernel(p, kname);
  if (!fn) return fail(SCL_ERR_LAUNCH, "kernel " + kname + " missing from the program");

  ArgPack pack;
  pack.ptrs.reserve(32);
  for (int i = 0; i < nbuf; ++i) pack.ptrs.push_back(&b[i]);
  if (point) {
    pack.ptrs.push_back(&rows);
    pack.ptrs.push_back(&cols);
    pack.ptrs.push_back(&offset);
  } else {
    pack.ptrs.push_back(&n);
    if (kind == SCL_KIND_MAP_INDEX || kind == SCL_KIND_MAP_INDEX_VOID) pack.ptrs.push_back(&offset);
    if (adjoint) pack.ptrs.push_back(&acc);
  }
  if (!simple) pack.ptrs.push_back(&aligned);
  const size_t fixed = pack.ptrs.size();
  if (int st = pack_extra(p, fn, fixed, (const unsigned char*)extra, extra_bytes, &pack)) return st;

  uint32_t wg = pick_block(tu, 256);
  dim3 grid, block;
  if (simple) {
    if (point) {
      // reference: local = floorPow2(sqrt(wg))^2 (MapDef.h:590-597)
      uint32_t s = 1;
      while ((s * 2) * (s * 2) <= wg) s *= 2;
      block = dim3(s, s, 1);
      uint64_t gx = (cols + s - 1) / s, gy = (rows + s - 1) / s;
      if (gx > 0x7fffffffull || gy > 65535) return fail(SCL_ERR_ARG, "matrix too large for the one-thread-per-element shape");
      grid = dim3((unsigned)gx, (unsigned)gy, 1);
    } else {
      block = dim3(wg, 1, 1);
      uint64_t g = (n + wg - 1) / wg;
      if (g > 0x7fffffffull) return fail(SCL_ERR_ARG, "vector too large for the one-thread-per-element shape");
      grid = dim3((unsigned)g, 1, 1);
    }
    p->last_variant = SCL_VARIANT_SIMPLE;
  } else {
    const int maxb = max_resident_blocks(fn, (int)wg, pack.local_bytes);
    if (point) {
      uint32_t bx = 256;
      block = dim3(bx, 1, 1);
      uint64_t gx = (cols + bx - 1) / bx;
      if (gx > (uint64_t)maxb) gx = (uint64_t)maxb;
      uint64_t gy = rows;
      uint64_t cap = std::max<uint64_t>(1, (uint64_t)maxb * 4 / gx);
      if (gy > cap) gy = cap;
      if (gy > 65535) gy = 65535;
      grid = dim3((unsigned)gx, (unsigned)std::max<uint64_t>(gy, 1), 1);
    } else {
      size_t s0 = p->type_sizes.size() > 0 ? p->type_sizes[0] : 4;
      size_t s1 = p->type_sizes.size() > 1 ? p->type_sizes[1] : s0;
      size_t s2 = p->type_sizes.size() > 2 ? p->type_sizes[2] : s0;
      int V = (kind == SCL_KIND_MAP_INDEX_VOID) ? 1 : vec_width(s0, s1, s2);
      uint64_t units = aligned ? (n + V - 1) / V : n;
      uint64_t g = (units + wg - 1) / wg;
      if (g > (uint64_t)maxb) g = (uint64_t)maxb;
      block = dim3(wg, 1, 1);
      grid = dim3((unsigned)std::max<uint64_t>(g, 1), 1, 1);
    }
    p->last_variant = SCL_VARIANT_VECTOR;
  }
  return launch(fn, grid, block, 0, pack);
}

extern "C" int scl_launch_zip(scl_program* p, const scl_shape* sh, void* const* bufs,
                              const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  if (int st = check_prog(p, {SCL_KIND_ZIP, SCL_KIND_ZIP_VOID})) return st;
  return scl_launch_map(p, sh, bufs, extra, extra_bytes, tu);
}

// ---- Reduce -------------------------------------------------------------------
static int launch_zipreduce(scl_program* p, const scl_shape* sh, void* const* bufs,
                            const void* extra, size_t extra_bytes, const scl_tuning* tu);

static int launch_reduce_impl(scl_program* p, const scl_shape* sh, void* const* bufs,
                                 const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  if (int st = check_prog(p, {SCL_KIND_REDUCE, SCL_KIND_ZIP_REDUCE})) return st;
  if (p->kind == SCL_KIND_ZIP_REDUCE) return launch_zipreduce(p, sh, bufs, extra, extra_bytes, tu);
  if (!sh || !bufs || !bufs[0] || !bufs[1]) return fail(SCL_ERR_ARG, "reduce needs {in, out}");
  void* in = bufs[0];
  void* out = bufs[1];
  uint64_t n = sh->n;
  const size_t tsz = p->type_sizes[0], csz = p->carry_size ? p->carry_size : tsz;
  const int V = vec_width(tsz);
  int aligned = aligned16(in) ? 1 : 0;
  if (sh->n_segments && sh->seg_plan) {
    // a segment plan: one launch, the tiles of the long segments first, then
    // one block per window of short segments (staged in shared memory)
    SegPlan* pl = segplan_find(sh->seg_plan);
    if (!pl) return fail(SCL_ERR_ARG, "segmented reduce: no segment plan " + std::to_string(sh->seg_plan));
    if (pl->n_seg != sh->n_segments || pl->n_total > n)
      return fail(SCL_ERR_ARG, "segmented reduce: the plan was made for other segments or a longer vector");
    uint64_t n_seg = sh->n_segments;
    const uint32_t R = (tu && tu->items == 8) ? 8 : 32;
    const uint64_t tile = (uint64_t)R * 256 * V;
    // a window block stages wt elements (32 KB for 16-byte vectors): windows
    // of wt / 2 and segments of at most wt / 2 elements, so a window's
    // segments always fit
    const uint64_t wt = (uint64_t)8 * 256 * V;
    uint64_t short_max = wt / 2;
    const SegPlanCfg* cfg = nullptr;
    if (int st = segplan_config(pl, tile, 1, 0, 0, short_max, &cfg)) return st;
    const std::string kname = "scl_reduce_seg<" + std::to_string(R) + ", 1>";
    CUfunction fn = find_kernel(p, kname);
    if (!fn) return fail(SCL_ERR_LAUNCH, "kernel " + kname + " missing");
    // partials after the first 256 bytes: the flat reduce keeps its ticket
    // there, and it must stay zero between launches
    if (int st = ensure_workspace(p, 256 + cfg->tiles * csz)) return st;
    void* partials = (char*)p->ws.ptr + 256;
    void* offs = pl->off;
    void* tstart = cfg->tile_start;
    void* tickets = pl->tickets;
    void* wseg = cfg->win_rec;
    unsigned int* err = rt().dev_err;
    unsigned int spin = spin_of(tu);
    ArgPack pack;
    void* towner = cfg->tile_seg;
    unsigned int ntiles = (unsigned int)cfg->tiles;
    pack.ptrs = {&in, &out, &offs, &tstart, &n_seg, &aligned, &partials, &tickets, &err, &short_max, &wseg,
                 &spin, &towner, &ntiles};
    if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
      return st;
    const uint64_t grid = cfg->tiles + cfg->n_rec;
    if (grid == 0) return SCL_OK;  // (every vector is either a tile's or in a record)
    if (grid > 0x7fffffffull) return fail(SCL_ERR_ARG, "segmented reduce: too many tiles");
    p->last_variant = SCL_VARIANT_VECTOR;
    // (a record's elements keep their 16-byte phase: one vector more)
    return launch(fn, dim3((unsigned)grid), dim3(256), wt * tsz + 16, pack);
  }
  if (sh->n_segments) {
    // one result per segment, one launch (plus the offsets pre-pass)
    if (!sh->seg_offsets) return fail(SCL_ERR_ARG, "segmented reduce: null seg_offsets");
    uint64_t n_seg = sh->n_segments;
    // 128 KB tiles for 16-byte vectors by default: few blocks, each with long
    // streams of loads (tuning.items = 8: 32 KB tiles)
    const uint32_t R = (tu && tu->items == 8) ? 8 : 32;
    const uint64_t tile = (uint64_t)R * 256 * V;
    // tiles exist only for segments longer than kSegShort (ceil(len / tile)
    // each): at most n / tile + 1 per such segment
    const uint64_t n_long = std::min<uint64_t>(n_seg, n / (kSegShort + 1) + 1);
    const uint64_t tiles = (n + tile - 1) / tile + n_long;
    if (tiles > 0x7fffffffull) return fail(SCL_ERR_ARG, "segmented reduce: too many tiles");
    const std::string kname = "scl_reduce_seg<" + std::to_string(R) + ">";
    CUfunction fn = find_kernel(p, kname);
    if (!fn) return fail(SCL_ERR_LAUNCH, "kernel " + kname + " missing");
    CUfunction fn_short = find_kernel(p, "scl_reduce_short<8>");
    if (!fn_short) return fail(SCL_ERR_LAUNCH, "kernel scl_reduce_short<8> missing");
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t tk = up(n_seg * 4), pa = up(tiles * csz), of = up((n_seg + 1) * 8),
                 ts = up((n_seg + 1) * 4);
    if (int st = ensure_workspace(p, tk + pa + of + ts + up(segments_prepare_scratch(n_seg)))) return st;
    char* ws = static_cast<char*>(p->ws.ptr);
    void* tickets = ws;
    void* partials = ws + tk;
    void* offs = ws + tk + pa;
    void* tstart = ws + tk + pa + of;
    uint64_t* scratch = reinterpret_cast<uint64_t*>(ws + tk + pa + of + ts);
    SCL_CUDA(cudaMemsetAsync(tickets, 0, tk, rt().stream));
    uint64_t short_max = kSegShort;
    if (int st = segments_prepare(sh->seg_offsets, n_seg, n, tile, 1, 0, 0, short_max, (uint64_t*)offs,
                                  (unsigned int*)tstart, scratch, rt().stream))
      return st;
    unsigned int* err = rt().dev_err;
    // segments of at most kSegShort elements (empty ones included): one warp each
    ArgPack spack;
    spack.ptrs = {&in, &out, &offs, &n_seg, &short_max};
    if (int st = pack_extra(p, fn_short, spack.ptrs.size(), (const unsigned char*)extra, extra_bytes,
                            &spack))
      return st;
    uint64_t sblocks = (n_seg + 7) / 8;  // 8 warps per block
    const uint64_t smax = (uint64_t)max_resident_blocks(fn_short, 256, spack.local_bytes);
    if (sblocks > smax) sblocks = smax;
    if (int st = launch(fn_short, dim3((unsigned)sblocks), dim3(256), 0, spack)) return st;
    // longer segments: tiles (blocks past the last tile return at once)
    ArgPack pack;
    void* no_windows = nullptr;
    unsigned int spin = spin_of(tu);
    void* no_owners = nullptr;
    unsigned int ntiles = ~0u;  // (counted on the device by the pre-pass)
    pack.ptrs = {&in, &out, &offs, &tstart, &n_seg, &aligned, &partials, &tickets, &err, &short_max,
                 &no_windows, &spin, &no_owners, &ntiles};
    if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
      return st;
    p->last_variant = SCL_VARIANT_VECTOR;
    return launch(fn, dim3((unsigned)tiles), dim3(256), 0, pack);
  }
  // 8 vectors of 16 bytes in flight per thread by default (measured 2-3 %
  // faster than 4 at 2^24 and 2^26 f32)
  uint32_t items = (tu && tu->items) ? tu->items : 8;
  if (items != 1 && items != 2 && items != 4 && items != 8) items = 8;
  std::string kname = "scl_reduce_k<" + std::to_string(items) + ">";
  CUfunction fn = find_kernel(p, kname);
  if (!fn) return fail(SCL_ERR_LAUNCH, "kernel " + kname + " missing");
  uint32_t wg = pick_block(tu, 256);
  wg = (wg + 31) / 32 * 32;
  const int maxb = max_resident_blocks(fn, (int)wg, 0);
  uint64_t units = aligned ? n / V : n;
  uint64_t g = units == 0 ? 1 : (units + wg - 1) / wg;
  if (g > (uint64_t)maxb) g = (uint64_t)maxb;
  if (g < 1) g = 1;
  const size_t part_off = 256;
  if (int st = ensure_workspace(p, part_off + g * csz)) return st;
  void* partials = (char*)p->ws.ptr + part_off;
  void* ticket = p->ws.ptr;
  unsigned int* err = rt().dev_err;
  ArgPack pack;
  pack.ptrs = {&in, &out, &n, &aligned, &partials, &ticket, &err};
  if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
    return st;
  p->last_variant = SCL_VARIANT_VECTOR;
  return launch(fn, dim3((unsigned)g), dim3(wg), 0, pack);
}

// Reduce(Zip(left, right)) in one pass: buffers {left, right, out}.
static int launch_zipreduce(scl_program* p, const scl_shape* sh, void* const* bufs,
                            const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  if (!sh || !bufs || !bufs[0] || !bufs[1] || !bufs[2])
    return fail(SCL_ERR_ARG, "fused zip-reduce needs {left, right, out}");
  if (sh->n_segments) return fail(SCL_ERR_UNSUPPORTED, "fused zip-reduce: no segmented form");
  void* l = bufs[0];
  void* r = bufs[1];
  void* out = bufs[2];
  uint64_t n = sh->n;
  const size_t s0 = p->type_sizes[0], s1 = p->type_sizes[1], tsz = p->type_sizes[2];
  const size_t csz = p->carry_size ? p->carry_size : tsz;
  const int V = vec_width(s0, s1);
  int aligned = (aligned16(l) && aligned16(r)) ? 1 : 0;
  uint32_t items = (tu && tu->items) ? tu->items : 4;
  if (items != 1 && items != 2 && items != 4) items = 4;
  const std::string kname = "scl_zipreduce_k<" + std::to_string(items) + ">";
  CUfunction fn = find_kernel(p, kname);
  if (!fn) return fail(SCL_ERR_LAUNCH, "kernel " + kname + " missing");
  uint32_t wg = pick_block(tu, 256);
  wg = (wg + 31) / 32 * 32;
  const int maxb = max_resident_blocks(fn, (int)wg, 0);
  uint64_t units = aligned ? n / V : n;
  uint64_t g = units == 0 ? 1 : (units + wg - 1) / wg;
  if (g > (uint64_t)maxb) g = (uint64_t)maxb;
  if (g < 1) g = 1;
  const size_t part_off = 256;
  if (int st = ensure_workspace(p, part_off + g * csz)) return st;
  void* partials = (char*)p->ws.ptr + part_off;
  void* ticket = p->ws.ptr;
  unsigned int* err = rt().dev_err;
  ArgPack pack;
  pack.ptrs = {&l, &r, &out, &n, &aligned, &partials, &ticket, &err};
  if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
    return st;
  p->last_variant = SCL_VARIANT_VECTOR;
  return launch(fn, dim3((unsigned)g), dim3(wg), 0, pack);
}

// ---- Scan ---------------------------------------------------------------------
namespace scl {
size_t scan_region_bytes(int status_mode, size_t carry, uint64_t cap) {
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  if (status_mode != 0) return 256 + up(cap * 128);
  return 256 + up(cap * 4) + 2 * up(cap * carry);
}
size_t scan_status_bytes(int status_mode, size_t carry, uint64_t cap) {
  return 3 * scan_region_bytes(status_mode, carry, cap);
}
size_t scan_region_clear_bytes(int status_mode, uint64_t tiles) {
  return 256 + (status_mode != 0 ? tiles * 128 : tiles * 4);
}
ScanStatusArgs scan_region(void* base, int status_mode, size_t carry, uint64_t cap, int r,
                           void** ticket) {
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  char* b = static_cast<char*>(base) + (size_t)r * scan_region_bytes(status_mode, carry, cap);
  if (ticket) *ticket = b;
  ScanStatusArgs a = {nullptr, nullptr, nullptr, nullptr};
  if (status_mode != 0) {
    a.slots = b + 256;
  } else {
    a.flags = b + 256;
    a.agg = b + 256 + up(cap * 4);
    a.incl = b + 256 + up(cap * 4) + up(cap * carry);
  }
  return a;
}
// The staged kernel lays tiles on the 16-byte grid of `in`: first element
// index `a` on a 16-byte boundary, one grid point every `vg` elements (vg = 1
// and a = 0 without a grid: odd element sizes, misaligned pointers, or the
// register kernel).
void scan_grid(const void* in, size_t tsz, bool staged, uint64_t* vg, uint64_t* a) {
  const bool grid = staged && (tsz == 4 || tsz == 8 || tsz == 16) &&
                    reinterpret_cast<uintptr_t>(in) % tsz == 0;
  *vg = grid ? 16 / tsz : 1;
  *a = grid ? ((16u - (reinterpret_cast<uintptr_t>(in) & 15u)) & 15u) / tsz : 0;
}
uint64_t scan_tiles(const void* in, size_t tsz, uint64_t n, uint64_t tile, bool staged, bool reverse) {
  uint64_t vg, ga;
  scan_grid(in, tsz, staged, &vg, &ga);
  if (!staged) return (n + tile - 1) / tile;
  const uint64_t m = reverse ? (ga + vg - n % vg) % vg : (vg - ga) % vg;
  return (n + m + tile - 1) / tile;
}
}  // namespace scl

static int launch_scan_impl(scl_program* p, const scl_shape* sh, void* const* bufs,
                               const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  if (int st = check_prog(p, {SCL_KIND_SCAN, SCL_KIND_SCAN_MAP})) return st;
  if (!sh || !bufs || !bufs[0] || !bufs[1]) return fail(SCL_ERR_ARG, "scan needs {in, out}");
  void* in = bufs[0];
  void* out = bufs[1];
  uint64_t n = sh->n;
  if (n == 0) return SCL_OK;
  const size_t tsz = p->type_sizes[0], csz = p->carry_size ? p->carry_size : tsz;
  const int V = vec_width(tsz);
  unsigned int flags = sh->flags & (SCL_SHAPE_INCLUSIVE | SCL_SHAPE_REVERSE);
  const bool reverse = (flags & SCL_SHAPE_REVERSE) != 0;
  int aligned = (aligned16(in) && aligned16(out)) ? 1 : 0;
  // 32 KB tiles by default: fewer tiles to look back over (measured on GB300)
  uint32_t R = (tu && tu->items) ? tu->items : 8;
  if (R != 2 && R != 4 && R != 6 && R != 8 && R != 16) R = 8;
  // default: the shared-memory staged kernel (measured 5.7 TB/s on int32 2^28
  // against 5.1 for the tile held in registers); SCL_VARIANT_VECTOR selects
  // the register kernel
  bool staged = !(tu && tu->variant == SCL_VARIANT_VECTOR) || p->kind == SCL_KIND_SCAN_MAP;
  if (staged && R == 2) R = 4;
  if (!staged && R == 6) R = 8;
  size_t smem = staged ? (size_t)R * 256 * V * tsz : 0;
  if (staged && smem + 2048 > rt().smem_optin) {
    if (p->kind == SCL_KIND_SCAN_MAP)
      return fail(SCL_ERR_UNSUPPORTED, "fused scan-map: the tile does not fit in shared memory");
    staged = false;
    smem = 0;
  }
  uint64_t n_seg = sh->n_segments;
  SegPlan* plan = nullptr;
  if (n_seg && sh->seg_plan) {
    plan = segplan_find(sh->seg_plan);
    if (!plan) return fail(SCL_ERR_ARG, "segmented scan: no segment plan " + std::to_string(sh->seg_plan));
    if (plan->n_seg != n_seg || plan->n_total > n)
      return fail(SCL_ERR_ARG, "segmented scan: the plan was made for other segments or a longer vector");
  }
  if (n_seg) {  // segmented: the staged kernel with the default tile shape
    if (!sh->seg_offsets && !plan) return fail(SCL_ERR_ARG, "segmented scan: null seg_offsets");
    staged = true;
    R = (tu && tu->items == 16) ? 16 : 8;
    smem = (size_t)R * 256 * V * tsz;
    if (smem + 2048 > rt().smem_optin)
      return fail(SCL_ERR_UNSUPPORTED, "segmented scan: the tile does not fit in shared memory");
  }
  const uint64_t tile = (uint64_t)R * 256 * V;
  uint64_t vg = 1, ga = 0;
  scan_grid(in, tsz, staged, &vg, &ga);
  uint64_t tiles;
  const SegPlanCfg* pcfg = nullptr;
  if (plan) {
    // the plan's exact tile count; windows of tile / 2 elements and short
    // segments of at most tile / 2, so a window's segments fit in one staged
    // tile
    if (int st = segplan_config(plan, tile, vg, ga, reverse ? 1 : 0, tile / 2, &pcfg)) return st;
    tiles = pcfg->tiles;
  } else if (n_seg) {
    // an upper bound (the pre-pass has the count): tiles exist only for
    // segments longer than kSegShort, at most n / tile + 2 per such segment
    const uint64_t n_long = std::min<uint64_t>(n_seg, n / (kSegShort + 1) + 1);
    tiles = (n + tile - 1) / tile + 2 * n_long;
  } else {
    tiles = scan_tiles(in, tsz, n, tile, staged, reverse);
  }
  if (tiles > 0x7fffffffull) return fail(SCL_ERR_ARG, "scan input too large");
  // resident tiles per SM the register (or shared-memory) budget is sized for
  uint32_t minb = (tu && tu->tile_w) ? tu->tile_w : 0;
  if (staged) {
    if (!((R == 16 && (minb == 2 || minb == 3)) || (R == 8 && minb >= 4 && minb <= 6) ||
          (R == 6 && minb == 8) || (R == 4 && minb == 8)))
      minb = R == 16 ? 3 : (R == 8 ? 6 : 8);
  } else if (!((R == 16 && (minb == 1 || minb == 2)) || (R == 8 && (minb == 2 || minb == 3 || minb == 4)) ||
               (R == 4 && (minb == 4 || minb == 6)) || (R == 2 && minb == 8))) {
    minb = R == 16 ? 2 : (R == 8 ? 4 : (R == 4 ? 6 : 8));
  }
  if (n_seg) minb = R == 16 ? 3 : 6;
  const std::string kname = std::string(staged ? "scl_scan_s<" : "scl_scan_k<") + std::to_string(R) +
                            ", " + std::to_string(minb) + (plan ? ", 2>" : (n_seg ? ", 1>" : ">"));
  CUfunction fn = find_kernel(p, kname);
  if (!fn) return fail(SCL_ERR_LAUNCH, "kernel " + kname + " missing");
  // workspace: three status regions (scan_region_bytes); segmented launches
  // add [clamped offsets | tile numbering | pre-pass scratch] after them
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const bool prepass = n_seg && !plan;
  const size_t seg_of = prepass ? up((n_seg + 1) * 8) : 0, seg_ts = prepass ? up((n_seg + 1) * 4) : 0,
               seg_sc = prepass ? up(segments_prepare_scratch(n_seg)) : 0;
  Workspace& ws = p->ws;
  const uint64_t cap = std::max<uint64_t>({tiles, ws.scan_cap, 256});
  const size_t total = scan_status_bytes(p->status_mode, csz, cap);
  // a new status layout in an allocation a graph has recorded would move
  // the graph's region under it: take a fresh allocation instead
  const bool relayout = cap != ws.scan_cap || ws.scan_layout != ws.ptr;
  if (int st = ensure_workspace(p, total + seg_of + seg_ts + seg_sc, relayout && ws.recorded)) return st;
  if (cap != ws.scan_cap || ws.scan_layout != ws.ptr) {
    SCL_CUDA(cudaMemsetAsync(ws.ptr, 0, total, rt().stream));
    ws.scan_cap = cap;
    ws.scan_layout = ws.ptr;
    ws.scan_epoch = 0;
    ws.scan_used[0] = ws.scan_used[1] = 0;
  }
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  SCL_CUDA(cudaStreamIsCapturing(rt().stream, &capture));
  const bool recorded = capture != cudaStreamCaptureStatusNone;
  // eager launches alternate between regions 0 and 1 and clear the other
  // one for the next launch; a recorded launch uses region 2 and the graph
  // clears it first, so every replay finds it clean
  const int region = recorded ? 2 : (int)(ws.scan_epoch & 1);
  void* counter = nullptr;
  ScanStatusArgs sargs = scan_region(ws.ptr, p->status_mode, csz, cap, region, &counter);
  ScanClearArgs clr = {nullptr, nullptr, nullptr, 0};
  if (recorded) {
    SCL_CUDA(cudaMemsetAsync(counter, 0, scan_region_clear_bytes(p->status_mode, tiles), rt().stream));
  } else {
    ScanStatusArgs o = scan_region(ws.ptr, p->status_mode, csz, cap, region ^ 1, &clr.ticket);
    clr.slots = o.slots;
    clr.flags = o.flags;
    clr.n = ws.scan_used[region ^ 1];
  }
  void* seg_off = prepass ? (char*)ws.ptr + total : (plan ? (void*)plan->off : nullptr);
  void* tile_start = prepass ? (char*)ws.ptr + total + seg_of : (plan ? (void*)pcfg->tile_start : nullptr);
  uint64_t short_max = plan ? pcfg->short_max : (n_seg ? kSegShort : 0);
  void* win_seg = plan ? (void*)pcfg->win_rec : nullptr;
  void* tile_owner = plan ? (void*)pcfg->tile_seg : nullptr;
  unsigned int n_tiles = plan ? (unsigned int)pcfg->tiles : ~0u;
  uint64_t grid = tiles;
  if (plan) {
    // the blocks past the tiles take one window record of short segments
    // each; a record keeps its 16-byte phase in shared memory, so it needs
    // one vector more than a tile
    grid = tiles + pcfg->n_rec;
    if (grid == 0) return SCL_OK;  // (every vector is either a tile's or in a record)
    if (grid > 0x7fffffffull) return fail(SCL_ERR_ARG, "segmented scan: too many tiles");
    smem += 16;
  }
  if (prepass) {
    uint64_t* scratch = reinterpret_cast<uint64_t*>((char*)p->ws.ptr + total + seg_of + seg_ts);
    if (int st = segments_prepare(sh->seg_offsets, n_seg, n, tile, vg, ga, reverse ? 1 : 0, short_max,
                                  (uint64_t*)seg_off, (unsigned int*)tile_start, scratch, rt().stream))
      return st;
    // segments of at most kSegShort elements: one warp each
    CUfunction fn_short = find_kernel(p, "scl_scan_short<8>");
    if (!fn_short) return fail(SCL_ERR_LAUNCH, "kernel scl_scan_short<8> missing");
    ArgPack spack;
    spack.ptrs = {&in, &out, &seg_off, &n_seg, &flags, &short_max};
    if (int st = pack_extra(p, fn_short, spack.ptrs.size(), (const unsigned char*)extra, extra_bytes,
                            &spack))
      return st;
    uint64_t sblocks = (n_seg + 7) / 8;  // 8 warps per block
    const uint64_t smax = (uint64_t)max_resident_blocks(fn_short, 256, spack.local_bytes);
    if (sblocks > smax) sblocks = smax;
    if (int st = launch(fn_short, dim3((unsigned)sblocks), dim3(256), 0, spack)) return st;
  }
  unsigned int spin = spin_of(tu);
  unsigned int* err = rt().dev_err;
  ArgPack pack;
  pack.ptrs = {&in, &out, &n, &flags, &aligned, &counter, &sargs, &clr, &spin, &err};
  if (staged) {
    pack.ptrs.push_back(&seg_off);
    pack.ptrs.push_back(&tile_start);
    pack.ptrs.push_back(&n_seg);
    pack.ptrs.push_back(&short_max);
    pack.ptrs.push_back(&win_seg);
    pack.ptrs.push_back(&tile_owner);
    pack.ptrs.push_back(&n_tiles);
  }
  if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
    return st;
  p->last_variant = staged ? SCL_VARIANT_TMA : SCL_VARIANT_VECTOR;
  if (int st = launch(fn, dim3((unsigned)grid), dim3(256), smem, pack)) return st;
  if (!recorded) {  // this launch's region now holds up to `tiles` slots; the other is clean
    ws.scan_used[region] = tiles;
    ws.scan_used[region ^ 1] = 0;
    ws.scan_epoch++;
  }
  return SCL_OK;
}

// ---- MapOverlap -----------------------------------------------------------------
static int launch_mapoverlap_impl(scl_program* p, const scl_shape* sh, void* const* bufs,
                                     const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  if (int st = check_prog(p, {SCL_KIND_MAPOVERLAP})) return st;
  if (!sh || !bufs || !bufs[0] || !bufs[1]) return fail(SCL_ERR_ARG, "mapoverlap needs {in, out}");
  void* in = bufs[0];
  void* out = bufs[1];
  uint64_t rows = sh->rows, cols = sh->cols;
  if (rows == 0 || cols == 0) return SCL_OK;
  if (rows > 0x7fffffffull || cols > 0x7fffffffull) return fail(SCL_ERR_ARG, "matrix too large");
  const size_t tsz = p->type_sizes[0];
  const bool want_tma = !(tu && tu->variant == SCL_VARIANT_LDST);
  // output rows per thread; default 16 outputs per thread (4 x 4, or 8 x 2
  // with two columns, 8 x 1 with one)
  const int py_default = p->stencil_px == 4 ? 4 : 8;
  int PY = (tu && tu->tile_h) ? (int)tu->tile_h : py_default;
  if (PY != 4 && PY != 8 && PY != 16) PY = py_default;
  const int R = p->overlap_range, TW = 32 * p->stencil_px;
  const int xal = tsz <= 16 ? (int)std::max<size_t>(1, 16 / tsz) : 1;
  const int xlead = (R + xal - 1) / xal * xal;
  const int win_w = (xlead + TW + R + xal - 1) / xal * xal;
  const bool tma_shape_ok = (tsz == 1 || tsz == 2 || tsz == 4 || tsz == 8) &&
                            (cols * tsz) % 16 == 0 && aligned16(in) && win_w <= 256;
  if (PY == 16 && !(want_tma && tma_shape_ok)) PY = 8;  // 16 rows only in the TMA form
  if (8 * PY + 2 * R > 256 && PY > 4) PY = 4;
  const int TH = 8 * PY;
  const int win_h = TH + 2 * R;
  const size_t win_bytes = (size_t)win_w * win_h * tsz;
  if (win_bytes > rt().smem_optin) return fail(SCL_ERR_ARG, "overlap range too large for shared memory");
  dim3 grid((unsigned)((cols + TW - 1) / TW), (unsigned)((rows + TH - 1) / TH)), block(32, 8);
  if (grid.y > 65535) return fail(SCL_ERR_ARG, "matrix has too many rows for one launch");
  const bool tma_ok = tma_shape_ok && win_h <= 256;
  const std::string py = "<" + std::to_string(PY) + ">";
  unsigned int spin = spin_of(tu);
  unsigned int* err = rt().dev_err;
  if (want_tma && tma_ok) {
    CUfunction fn = find_kernel(p, "scl_mapoverlap_tma" + py);
    if (!fn) return fail(SCL_ERR_LAUNCH, "kernel scl_mapoverlap_tma" + py + " missing");
    alignas(64) CUtensorMap tmap;
    CUtensorMapDataType dt = tsz == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                           : tsz == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                           : tsz == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                                      : CU_TENSOR_MAP_DATA_TYPE_UINT64;
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {cols * tsz};
    cuuint32_t box[2] = {(cuuint32_t)win_w, (cuuint32_t)win_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = rt().drv.cuTensorMapEncodeTiled(
        &tmap, dt, 2, in, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cu_fail(r, "cuTensorMapEncodeTiled");
    ArgPack pack;
    pack.ptrs = {&tmap, &out, &rows, &cols, &spin, &err};
    if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
      return st;
    p->last_variant = SCL_VARIANT_TMA;
    return launch(fn, grid, block, win_bytes, pack);
  }
  CUfunction fn = find_kernel(p, "scl_mapoverlap_ldst" + py);
  if (!fn) return fail(SCL_ERR_LAUNCH, "kernel scl_mapoverlap_ldst" + py + " missing");
  ArgPack pack;
  pack.ptrs = {&in, &out, &rows, &cols};
  if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
    return st;
  p->last_variant = SCL_VARIANT_LDST;
  return launch(fn, grid, block, win_bytes, pack);
}

// ---- AllPairs -------------------------------------------------------------------
extern "C" int scl_launch_allpairs(scl_program* p, const scl_shape* sh, void* const* bufs,
                                   const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  if (int st = check_prog(p, {SCL_KIND_ALLPAIRS, SCL_KIND_ALLPAIRS_GENERIC})) return st;
  if (!sh || !bufs || !bufs[0] || !bufs[1] || !bufs[2])
    return fail(SCL_ERR_ARG, "allpairs needs {left, right, out}");
  void* A = bufs[0];
  void* B = bufs[1];
  void* P = bufs[2];
  if (sh->rows > 0xffffffffull || sh->cols > 0xffffffffull || sh->dim > 0xffffffffull)
    return fail(SCL_ERR_ARG, "AllPairs dimensions must fit 32 bits");
  unsigned int M = (unsigned int)sh->rows, N = (unsigned int)sh->cols, K = (unsigned int)sh->dim;
  if (M == 0 || N == 0) return SCL_OK;
  if (K == 0) return fail(SCL_ERR_ARG, "AllPairs inner dimension is 0");
  const int trans = ((sh->flags & SCL_SHAPE_TRANS_LEFT) ? 1 : 0) |
                    ((sh->flags & SCL_SHAPE_TRANS_RIGHT) ? 2 : 0);
  if (p->kind == SCL_KIND_ALLPAIRS) {
    const uint32_t want = tu ? tu->variant : SCL_VARIANT_AUTO;
    if (p->tc_eligible && want != SCL_VARIANT_SIMT && extra_bytes == 0 &&
        allpairs_tc_supported(M, N, K, A, B, P)) {
      // tuning.items == 2: two bf16 parts, 3 products; otherwise three parts, 6 products
      const int parts = (tu && tu->items == 2) ? 2 : 3;
      const size_t need = allpairs_tc_scratch_bytes(M, N, K, parts);
      if (int st = ensure_workspace(p, need)) return st;
      p->last_variant = SCL_VARIANT_TC3XBF16;
      // tuning.tile_w: k-blocks accumulated in tensor memory per drain of a
      // 128-column tile (1, 2 or 4)
      const int drain = (tu && tu->tile_w) ? (int)tu->tile_w : 1;
      // tuning.tile_h: output-tile columns, 128 or 256 (k-blocks of 32, drained
      // every 2); 0 takes 256 when the 128 x 256 tiles still give every SM one
      const uint32_t cols = tu ? tu->tile_h : 0u;
      const uint64_t wide_tiles = (uint64_t)((M + 127u) / 128u) * ((N + 255u) / 256u);
      const uint64_t sms = rt().sm_count > 0 ? (uint64_t)rt().sm_count : 148u;
      const int wide = cols == 256u || (cols == 0u && wide_tiles >= sms) ? 1 : 0;
      // tuning.workgroup: output-tile rows per group of the tile order (0: 16)
      const uint32_t group_rows = tu ? tu->workgroup : 0u;
      return allpairs_tc_launch((const float*)A, (const float*)B, (float*)P, M, N, K, parts, trans,
                                drain, wide, group_rows, p->ws.ptr, p->ws.bytes, rt().stream,
                                spin_of(tu), rt().dev_err);
    }
    if (want == SCL_VARIANT_TC3XBF16)
      return fail(SCL_ERR_UNSUPPORTED, "the tensor-core AllPairs needs zip x*y, reduce x+y, identity 0, "
                                       "float operands, no extra arguments and supported shapes");
    CUfunction fn = find_kernel(p, "scl_allpairs_simt");
    if (!fn) return fail(SCL_ERR_LAUNCH, "kernel scl_allpairs_simt missing");
    if (trans) {
      // CUDA-core kernel: transposed operands are first stored row-major in
      // the program's workspace
      const size_t s0 = p->type_sizes[0], s1 = p->type_sizes[1];
      const size_t a_bytes = (trans & 1) ? ((size_t)M * K * s0 + 255) / 256 * 256 : 0;
      const size_t b_bytes = (trans & 2) ? (size_t)K * N * s1 : 0;
      if (int st = ensure_workspace(p, a_bytes + b_bytes)) return st;
      char* ws = static_cast<char*>(p->ws.ptr);
      if (trans & 1) {
        if (int st = transpose_launch(A, ws, K, M, s0, rt().stream)) return st;
        A = ws;
      }
      if (trans & 2) {
        if (int st = transpose_launch(B, ws + a_bytes, N, K, s1, rt().stream)) return st;
        B = ws + a_bytes;
      }
    }
    int vec_a = (p->type_sizes[0] == 4 && K % 4 == 0 && aligned16(A)) ? 1 : 0;
    int vec_b = (p->type_sizes[1] == 4 && N % 4 == 0 && aligned16(B)) ? 1 : 0;
    ArgPack pack;
    pack.ptrs = {&A, &B, &P, &M, &N, &K, &vec_a, &vec_b};
    if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
      return st;
    dim3 grid((N + 127) / 128, (M + 127) / 128);
    if (grid.y > 65535) return fail(SCL_ERR_ARG, "too many rows");
    p->last_variant = SCL_VARIANT_SIMT;
    return launch(fn, grid, dim3(256), 0, pack);
  }
  if (trans) return fail(SCL_ERR_UNSUPPORTED, "transposed operands: only the Reduce/Zip AllPairs");
  CUfunction fn = find_kernel(p, "scl_allpairs_generic");
  if (!fn) return fail(SCL_ERR_LAUNCH, "kernel scl_allpairs_generic missing");
  const size_t s0 = p->type_sizes[0], s1 = p->type_sizes[1];
  size_t stage = ((16ull * K * s0 + 15) & ~15ull) + 16ull * K * s1;
  int staged = (stage + 1024 <= rt().smem_optin) ? 1 : 0;
  ArgPack pack;
  pack.ptrs = {&A, &B, &P, &K, &M, &N, &staged};
  if (int st = pack_extra(p, fn, pack.ptrs.size(), (const unsigned char*)extra, extra_bytes, &pack))
    return st;
  dim3 grid((N + 15) / 16, (M + 15) / 16);
  if (grid.y > 65535) return fail(SCL_ERR_ARG, "too many rows");
  p->last_variant = SCL_VARIANT_SIMT;
  return launch(fn, grid, dim3(16, 16), staged ? stage : 0, pack);
}


// ---- exported launches: the autotuner in front of each skeleton -------------------
namespace {

bool overlaps(const void* a, size_t abytes, const void* b, size_t bbytes) {
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  return a && b && x < y + bbytes && y < x + abytes;
}
// extra arguments the user function cannot write through
bool extras_are_values(const scl_program* p) {
  for (const Param& e : p->extra)
    if (e.kind != ParamKind::Value) return false;
  return true;
}
scl_tuning shape(uint32_t workgroup, uint32_t items, uint32_t tile_w, uint32_t tile_h, uint32_t variant) {
  scl_tuning t{};
  t.workgroup = workgroup;
  t.items = items;
  t.tile_w = tile_w;
  t.tile_h = tile_h;
  t.variant = variant;
  return t;
}

}  // namespace

extern "C" int scl_launch_map(scl_program* p, const scl_shape* sh, void* const* bufs,
                              const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  auto run = [&](const scl_tuning* t) { return launch_map_impl(p, sh, bufs, extra, extra_bytes, t); };
  if (!p || !sh || !bufs || untuned(tu) == false || p->uses_workitem) return run(tu);
  const uint64_t n = (p->kind == SCL_KIND_MAP_POINT || p->kind == SCL_KIND_MAP_POINT_VOID) ? sh->rows * sh->cols
                                                                                          : sh->n;
  const auto& ts = p->type_sizes;
  auto sz = [&](size_t i) { return ts.size() > i ? ts[i] : 0; };
  bool safe = extras_are_values(p);
  switch (p->kind) {
    case SCL_KIND_MAP: safe = safe && !overlaps(bufs[0], n * sz(0), bufs[1], n * sz(1)); break;
    case SCL_KIND_ZIP:
      safe = safe && !overlaps(bufs[0], n * sz(0), bufs[2], n * sz(2)) &&
             !overlaps(bufs[1], n * sz(1), bufs[2], n * sz(2));
      break;
    case SCL_KIND_MAP_INDEX:
    case SCL_KIND_MAP_POINT: break;
    case SCL_KIND_MAP_ADJOINT:
      safe = safe && !(sh->flags & SCL_SHAPE_ACCUMULATE) && !overlaps(bufs[0], n * sz(0), bufs[2], n * sz(0)) &&
             !overlaps(bufs[1], n * sz(1), bufs[2], n * sz(0));
      break;
    default: safe = false;  // side effects or accumulation: not repeatable
  }
  std::vector<scl_tuning> cands;
  for (uint32_t wg : {128u, 256u, 512u})
    for (uint32_t items : {1u, 2u, 4u}) cands.push_back(shape(wg, items, 0, 0, 0));
  return tuned_launch(p, "map", n, tu, safe, cands, run);
}

extern "C" int scl_launch_reduce(scl_program* p, const scl_shape* sh, void* const* bufs,
                                 const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  auto run = [&](const scl_tuning* t) { return launch_reduce_impl(p, sh, bufs, extra, extra_bytes, t); };
  if (!p || !sh || !bufs || !bufs[0] || !bufs[1] || p->type_sizes.empty()) return run(tu);
  if (p->kind == SCL_KIND_ZIP_REDUCE) {
    if (!bufs[2] || p->type_sizes.size() < 3) return run(tu);
    const bool safe = extras_are_values(p) &&
                      !overlaps(bufs[0], sh->n * p->type_sizes[0], bufs[2], p->type_sizes[2]) &&
                      !overlaps(bufs[1], sh->n * p->type_sizes[1], bufs[2], p->type_sizes[2]);
    std::vector<scl_tuning> cands;
    for (uint32_t wg : {256u, 512u})
      for (uint32_t items : {1u, 2u, 4u}) cands.push_back(shape(wg, items, 0, 0, 0));
    return tuned_launch(p, "zipreduce", sh->n, tu, safe, cands, run);
  }
  const size_t tsz = p->type_sizes[0];
  const uint64_t nout = sh->n_segments ? sh->n_segments : 1;
  const bool safe = extras_are_values(p) && !overlaps(bufs[0], sh->n * tsz, bufs[1], nout * tsz);
  std::vector<scl_tuning> cands;
  if (sh->n_segments) {
    for (uint32_t r : {8u, 32u}) cands.push_back(shape(0, r, 0, 0, 0));
    return tuned_launch(p, "reduce_seg", sh->n, tu, safe, cands, run);
  }
  for (uint32_t wg : {256u, 512u})
    for (uint32_t items : {2u, 4u, 8u}) cands.push_back(shape(wg, items, 0, 0, 0));
  return tuned_launch(p, "reduce", sh->n, tu, safe, cands, run);
}

extern "C" int scl_launch_scan(scl_program* p, const scl_shape* sh, void* const* bufs,
                               const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  auto run = [&](const scl_tuning* t) { return launch_scan_impl(p, sh, bufs, extra, extra_bytes, t); };
  if (!p || !sh || !bufs || !bufs[0] || !bufs[1] || p->type_sizes.empty()) return run(tu);
  const size_t bytes = sh->n * p->type_sizes[0];
  const bool safe = extras_are_values(p) && !overlaps(bufs[0], bytes, bufs[1], bytes);
  std::vector<scl_tuning> cands;
  if (sh->n_segments) {
    cands = {shape(0, 8, 6, 0, 0), shape(0, 16, 3, 0, 0)};
    return tuned_launch(p, "scan_seg", sh->n, tu, safe, cands, run);
  }
  cands = {shape(0, 8, 6, 0, 0), shape(0, 8, 5, 0, 0), shape(0, 16, 3, 0, 0),
           shape(0, 8, 4, 0, SCL_VARIANT_VECTOR)};
  return tuned_launch(p, "scan", sh->n, tu, safe, cands, run);
}

extern "C" int scl_launch_mapoverlap(scl_program* p, const scl_shape* sh, void* const* bufs,
                                     const void* extra, size_t extra_bytes, const scl_tuning* tu) {
  auto run = [&](const scl_tuning* t) { return launch_mapoverlap_impl(p, sh, bufs, extra, extra_bytes, t); };
  if (!p || !sh || !bufs) return run(tu);
  const bool safe = extras_are_values(p) || [&] {
    // weights passed as Vector / Matrix arguments are read by the stencil, not written
    for (const Param& e : p->extra)
      if (e.kind == ParamKind::Local) return false;
    return true;
  }();
  std::vector<scl_tuning> cands;
  // four columns per thread: 16 rows would unroll 64 user calls (slow to
  // compile, measured slower)
  const std::vector<uint32_t> pys =
      p->stencil_px == 4 ? std::vector<uint32_t>{4u, 8u} : std::vector<uint32_t>{4u, 8u, 16u};
  for (uint32_t v : {SCL_VARIANT_TMA, SCL_VARIANT_LDST})
    for (uint32_t py : pys) cands.push_back(shape(0, 0, 0, py, v));
  return tuned_launch(p, "mapoverlap", sh->rows * sh->cols, tu, safe, cands, run);
}
