/*
 * skelcl_cuda.h -- the C ABI between the SkelCL C++ headers and the GB300
 * (sm_103a) runtime in libskelcl_cuda.so.
 *
 * The SkelCL header templates (the headers under include/SkelCL) call only these entry
 * points.  Every function returns an int status (SCL_OK == 0); the message of
 * the last failure on the calling thread is returned by scl_last_error_string().
 * Arguments are plain pointers and sizes: no C++ or torch types cross this
 * boundary, so ctypes / cffi / JNI / cgo bind it directly.
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the SkelCL source tree).
 */
#ifndef SKELCL_CUDA_H_
#define SKELCL_CUDA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCL_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum scl_status {
  SCL_OK = 0,
  SCL_ERR_ARG = 1,         /* bad argument: null pointer, size, arg list   */
  SCL_ERR_OOM = 2,         /* device allocation failed                     */
  SCL_ERR_COMPILE = 3,     /* user source did not splice or compile        */
  SCL_ERR_LAUNCH = 4,      /* kernel launch failed                         */
  SCL_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up           */
  SCL_ERR_CUDA = 6,        /* any other CUDA runtime / driver error        */
  SCL_ERR_NOT_INIT = 7,    /* scl_init() was not called                    */
  SCL_ERR_UNSUPPORTED = 8  /* valid request this build does not implement  */
};

/* ---- skeleton kinds (one program per skeleton object) ------------------- */
enum scl_kind {
  SCL_KIND_MAP = 1,             /* Tout f(Tin, extra...)        MapDef.h:75-195    */
  SCL_KIND_MAP_VOID = 2,        /* void f(Tin, extra...)        MapDef.h:219-332   */
  SCL_KIND_MAP_INDEX = 3,       /* Tout f(Index, extra...)      MapDef.h:335-469   */
  SCL_KIND_MAP_INDEX_VOID = 4,  /* void f(Index, extra...)      src/Map.cpp:50-95  */
  SCL_KIND_MAP_POINT = 5,       /* Tout f(IndexPoint, extra...) MapDef.h:533-684   */
  SCL_KIND_MAP_POINT_VOID = 6,  /* void f(IndexPoint, extra...) src/Map.cpp:97-150 */
  SCL_KIND_ZIP = 7,             /* Tout f(Tl, Tr, extra...)     ZipDef.h:70-206    */
  SCL_KIND_ZIP_VOID = 8,        /* void f(Tl, Tr, extra...)     ZipDef.h:287-397   */
  SCL_KIND_REDUCE = 9,          /* T f(T, T, extra...)          ReduceDef.h:79-275 */
  SCL_KIND_SCAN = 10,           /* T f(T, T, extra...)          ScanDef.h:70-297   */
  SCL_KIND_MAPOVERLAP = 11,     /* Tout f(input_matrix_t, ...)  MapOverlapDef.h:71-279 */
  SCL_KIND_ALLPAIRS = 12,       /* reduce + zip pair            AllPairsDef.h:77-91,213-280 */
  SCL_KIND_ALLPAIRS_GENERIC = 13, /* Tout f(lmatrix_t*, rmatrix_t*, dim, ...) AllPairsDef.h:93-107,283-344 */
  /* Adjoints (no counterpart in the reference).  `source`/`func` give the
   * vector-Jacobian product of the forward function; type_names are the
   * forward's (Tin, Tout / Tl, Tr, Tout).  Launched with scl_launch_map. */
  SCL_KIND_MAP_ADJOINT = 14,    /* Tin  d(Tin x, Tout g, extra...)            */
  SCL_KIND_ZIP_ADJOINT = 15,    /* Tl dl(Tl x, Tr y, Tout g, extra...) = func,
                                   Tr dr(Tl x, Tr y, Tout g, extra...) = func2
                                   (in `source`, or in `source2` if given;
                                   same extra parameters as dl; optional) */
  /* Fused pairs (no counterpart in the reference, which materialises the
   * intermediate vector).  `source`/`func` are the first skeleton's, i.e.
   * the Reduce's / the Scan's, `source2`/`func2` the Zip's / the Map's; extra
   * arguments: the first function's, then the second's. */
  SCL_KIND_ZIP_REDUCE = 16,     /* Reduce(Zip(l, r)): types Tl, Tr, T; buffers
                                   {left, right, out}; launched with
                                   scl_launch_reduce                        */
  SCL_KIND_SCAN_MAP = 17        /* Map(Scan(x)): types T, Tout; buffers
                                   {in, out}; launched with scl_launch_scan  */
};

/* MapOverlap padding modes (include/SkelCL/detail/Padding.h:47-50). */
enum scl_padding { SCL_PAD_NEUTRAL = 0, SCL_PAD_NEAREST = 1 };

/* Program description.  Field meaning follows the reference constructors:
 * `source`/`func` are the user source and function name (Map.h:141-142,
 * Zip.h:96-120, Reduce.h:95-120, Scan.h:80-99, MapOverlap.h:119-140,
 * AllPairs.h:127-140).  For SCL_KIND_ALLPAIRS `source`/`func` are the
 * Reduce's and `source2`/`func2` the Zip's.  `type_names` are the OpenCL C
 * spellings of the element types in skeleton order (Tin, Tout / Tl, Tr, Tout /
 * T), as detail::util::typeToString produces them (detail/Util.h:81-98). */
typedef struct scl_program_desc {
  int kind;                       /* enum scl_kind */
  const char* source;             /* user source (OpenCL C)                  */
  const char* func;               /* user function name, "func" if NULL      */
  const char* source2;            /* AllPairs: the Zip's source              */
  const char* func2;              /* AllPairs: the Zip's function name       */
  const char* identity;           /* Reduce/Scan/AllPairs identity, "0"      */
  const char* type_names[3];      /* element types                           */
  int n_types;
  int overlap_range;              /* MapOverlap radius R                     */
  int padding;                    /* enum scl_padding                        */
  const char* neutral;            /* MapOverlap neutral element (C literal)  */
  const char* common_source;      /* CommonDefinitions (src/Source.cpp:118-126) */
  uint32_t flags;                 /* SCL_PROG_* below                        */
} scl_program_desc;

/* Program flags. */
#define SCL_PROG_NO_F64_CARRY 0x1u  /* keep float carries in float            */
#define SCL_PROG_STENCIL_COLS1 0x2u /* MapOverlap: one output column per thread
                                       (default: four, sharing their taps)    */
#define SCL_PROG_STENCIL_COLS2 0x4u /* MapOverlap: two output columns per thread */
#define SCL_PROG_COMPILE_ALL 0x8u   /* every kernel variant at once (build or
                                       compile check), none on first use      */

typedef struct scl_program scl_program;

/* Launch shape.  Only the fields a skeleton uses are read. */
typedef struct scl_shape {
  uint64_t n;            /* element count (Map/Zip/Reduce/Scan, flat length)  */
  uint64_t rows;         /* matrix rows (MapOverlap, Map<IndexPoint>, AllPairs output) */
  uint64_t cols;         /* matrix columns                                     */
  uint64_t dim;          /* AllPairs inner dimension                          */
  uint64_t offset;       /* Map<Index>: first index; Map<IndexPoint>: row offset */
  const uint64_t* seg_offsets; /* segmented launches: DEVICE array, n_segments+1 */
  uint64_t n_segments;   /* 0 = not segmented.  Segment s = elements
                            [seg_offsets[s], seg_offsets[s+1]) of the flat
                            vector of n elements.  Scan: one scan per segment;
                            Reduce: out gets n_segments results (SCL_IDENTITY
                            for an empty segment); a small pre-pass, then one
                            launch for the segments of up to 4096 elements
                            (a warp each) and one for the longer ones (tiles).
                            Offsets must be non-decreasing and at most n
                            (otherwise they are clamped to n, a segment whose
                            end lies before its start is empty, and the next
                            scl_sync reports SCL_ERR_ARG).  Map/Zip are
                            element-wise: segments do not change them.  No
                            counterpart in the reference.                     */
  uint32_t flags;        /* SCL_SHAPE_* below                                 */
  uint32_t seg_plan;     /* 0, or a segment plan (scl_segplan_create) made for
                            these offsets and n_segments (and a length up to
                            n): the segmented Scan or Reduce is then one
                            launch, without the offsets pre-pass             */
} scl_shape;

#define SCL_SHAPE_INCLUSIVE 0x1u  /* Scan: inclusive instead of exclusive     */
#define SCL_SHAPE_REVERSE   0x2u  /* Scan: scan from the end (adjoint of Scan) */
#define SCL_SHAPE_ACCUMULATE 0x4u /* adjoint kinds: add into the first gradient
                                     instead of overwriting it                 */
#define SCL_SHAPE_ACCUMULATE_RIGHT 0x8u /* Zip adjoint: add into the second */
#define SCL_SHAPE_TRANS_LEFT  0x10u /* AllPairs x*y/x+y: the left operand is
                                       stored transposed (dim x rows)          */
#define SCL_SHAPE_TRANS_RIGHT 0x20u /* ... the right operand (cols x dim)      */

/* Launch tuning; NULL means "defaults or autotuned".  Zero fields keep their
 * default.  workgroup mirrors Skeleton::setWorkGroupSize (src/Skeleton.cpp:75-78). */
/* Launch shape; a zero field takes the default. */
typedef struct scl_tuning {
  uint32_t workgroup;    /* threads per block (Map/Zip/Reduce); AllPairs
                            tensor cores: output-tile rows per group of the
                            tile order (0: 16)                                */
  uint32_t items;        /* 16-byte vectors per thread (Map/Zip/Reduce/Scan);
                            AllPairs tensor cores: bf16 parts, 2 or 3          */
  uint32_t tile_w;       /* Scan: tiles per SM; AllPairs tensor cores:
                            k-blocks per drain of 128-column tiles (1, 2, 4)  */
  uint32_t tile_h;       /* MapOverlap rows per thread / AllPairs tile columns */
  uint32_t variant;      /* SCL_VARIANT_*                                     */
  uint32_t spin_limit;   /* bounded-wait polls before SCL_ERR_TIMEOUT, 0 = default */
} scl_tuning;

#define SCL_VARIANT_AUTO 0u
#define SCL_VARIANT_SIMPLE 1u     /* one element per thread (reference shape) */
#define SCL_VARIANT_VECTOR 2u     /* grid-stride 128-bit vectorised           */
#define SCL_VARIANT_SIMT 3u       /* AllPairs: FP32 SIMT register tiles       */
#define SCL_VARIANT_TC3XBF16 4u   /* AllPairs: tcgen05 3xBF16 contraction     */
#define SCL_VARIANT_TMA 5u        /* MapOverlap: TMA-staged tile              */
#define SCL_VARIANT_LDST 6u       /* MapOverlap: cooperative-load tile        */

/* ---- extra-argument blob ----------------------------------------------- *
 * The extra arguments of a skeleton call are packed in call order into one
 * blob of records { uint32 kind; uint32 size; payload padded to 8 bytes }.
 * Kinds follow detail::kernelUtil::setKernelArgs (detail/KernelUtil.h:132-245):
 *   SCL_ARG_VALUE   payload = `size` raw bytes of a scalar / struct
 *   SCL_ARG_BUFFER  payload = device pointer (Vector argument)
 *   SCL_ARG_MATRIX  payload = device pointer, uint32 column count (Matrix)
 *   SCL_ARG_LOCAL   payload = uint64 byte count of __local memory (Local)   */
enum scl_arg_kind {
  SCL_ARG_VALUE = 1,
  SCL_ARG_BUFFER = 2,
  SCL_ARG_MATRIX = 3,
  SCL_ARG_LOCAL = 4
};

/* ---- runtime: replaces skelcl::init / terminate (include/SkelCL/SkelCL.h:144-207,
 *      src/SkelCL.cpp:51-85, src/DeviceList.cpp:82-123, src/Device.cpp:95-122) */
int scl_init(int device);
int scl_terminate(void);
int scl_is_initialized(void);
int scl_device_info(int* sm_count, size_t* global_mem, char* name, size_t name_cap);
const char* scl_last_error_string(void);
int scl_abi_version(void);

/* ---- memory: replaces detail::DeviceBuffer and Device::enqueueWrite/Read/Copy
 *      (src/DeviceBuffer.cpp:60-135, src/Device.cpp:169-330).  All copies are
 *      ordered on the library stream; scl_h2d/scl_d2h return after the copy is
 *      complete (host buffers may be reused), the _async forms do not. */
int scl_alloc(size_t bytes, void** dptr);
int scl_free(void* dptr);
int scl_h2d(void* dst, const void* src, size_t bytes);
int scl_d2h(void* dst, const void* src, size_t bytes);
int scl_d2d(void* dst, const void* src, size_t bytes);
int scl_h2d_async(void* dst, const void* src, size_t bytes);
int scl_d2h_async(void* dst, const void* src, size_t bytes);
int scl_memset(void* dst, int value, size_t bytes);
int scl_host_alloc(size_t bytes, void** hptr); /* pinned host memory */
int scl_host_free(void* hptr);
int scl_sync(void);                 /* wait for the stream; reports device-side errors */
/* Transfers on copy streams, to overlap them with launches (the reference
 * enqueues transfers asynchronously on its command queues,
 * src/Device.cpp:124-167, src/DeviceBuffer.cpp:60-135).  stream 0 is the
 * library stream every launch runs on; 1 and 2 are copy streams.  Order
 * streams with scl_event_record_on / scl_stream_wait; scl_sync waits for all. */
int scl_h2d_on(int stream, void* dst, const void* src, size_t bytes);
int scl_d2h_on(int stream, void* dst, const void* src, size_t bytes);

/* ---- events: replaces detail::Event (src/Event.cpp) and the profiling queue */
typedef struct scl_event scl_event;
int scl_event_create(scl_event** ev);
int scl_event_record(scl_event* ev);
int scl_event_record_on(scl_event* ev, int stream);  /* see scl_h2d_on            */
int scl_stream_wait(int stream, scl_event* ev);       /* `stream` waits for `ev`   */
int scl_event_elapsed_ms(scl_event* start, scl_event* stop, float* ms);
int scl_event_destroy(scl_event* ev);

/* ---- programs: replaces detail::Program + stooling rewriting
 *      (src/Program.cpp:83-250, include/SkelCL/detail/Program.h:61-132,
 *      libraries/stooling/src/SourceCode.cpp:98-263).  Splices the user
 *      function into the sm_103a skeleton template and compiles it with NVRTC.
 *      On failure `log` (if given) receives the splice / NVRTC log. */
int scl_program_build(const scl_program_desc* desc, scl_program** out,
                      char* log, size_t log_cap);
int scl_program_release(scl_program* prog);
/* Splice and compile only (no device needed, nothing loaded): the check that
 * a user source is accepted, usable before scl_init(). */
int scl_program_compile(const scl_program_desc* desc, char* log, size_t log_cap);
/* Number of extra (non-skeleton) parameters the user function declares. */
int scl_program_extra_count(const scl_program* prog, int* count);
/* Hex SHA-1 of the assembled source (the program-cache key, src/Util.cpp:159-180). */
int scl_program_hash(const scl_program* prog, char* out41);
/* Splice-only dry run: writes the generated CUDA source, compiles nothing. */
int scl_program_source(const scl_program_desc* desc, char* out, size_t cap,
                       size_t* needed);
/* Program binary cache: replaces Program::loadBinary / saveBinary
 * (src/Program.cpp:136-175, 252-281) and keeps its switches:
 * SKELCL_LOAD_BINARY=YES reuses cubins from SKELCL_CACHE_DIR (default
 * $HOME/.cache/skelcl_gb300), SKELCL_SAVE_BINARY=YES writes them there,
 * SKELCL_PRINT_BUILD_LOG=YES prints NVRTC's log.  A cubin is keyed by the
 * generated source, the kernel names, the NVRTC options and version, this
 * library's ABI version and (once scl_init has run) the device's compute
 * capability and driver version; a file that is truncated, garbled or for
 * another key is rejected and the program is compiled instead.  Counters
 * since the library was loaded: NVRTC compilations, cubins loaded from
 * disk, files rejected, files written (any pointer may be NULL). */
int scl_cache_stats(uint64_t* nvrtc_compiles, uint64_t* disk_loads,
                    uint64_t* disk_rejects, uint64_t* disk_saves);

/* SHA-1 of arbitrary bytes as 40 hex characters + NUL (util::hash). */
int scl_sha1_hex(const void* data, size_t bytes, char* out41);

/* ---- launches: replace the per-skeleton execute() bodies.  `buffers` holds
 *      device pointers in skeleton order:
 *        map:        {in, out}      (void map: {in}; Index maps: {out} / {})
 *        zip:        {left, right, out}   (void zip: {left, right})
 *        reduce:     {in, out}      out receives 1 element (n_segments elements
 *                                   for a segmented reduce)
 *        scan:       {in, out}
 *        mapoverlap: {in, out}      rows x cols, row-major
 *        allpairs:   {left, right, out}  left rows x dim, right dim x cols
 *      All launches are asynchronous on the library stream. */
int scl_launch_map(scl_program* prog, const scl_shape* shape,
                   void* const* buffers, const void* extra, size_t extra_bytes,
                   const scl_tuning* tuning);
int scl_launch_zip(scl_program* prog, const scl_shape* shape,
                   void* const* buffers, const void* extra, size_t extra_bytes,
                   const scl_tuning* tuning);
int scl_launch_reduce(scl_program* prog, const scl_shape* shape,
                      void* const* buffers, const void* extra,
                      size_t extra_bytes, const scl_tuning* tuning);
int scl_launch_scan(scl_program* prog, const scl_shape* shape,
                    void* const* buffers, const void* extra, size_t extra_bytes,
                    const scl_tuning* tuning);
int scl_launch_mapoverlap(scl_program* prog, const scl_shape* shape,
                          void* const* buffers, const void* extra,
                          size_t extra_bytes, const scl_tuning* tuning);
int scl_launch_allpairs(scl_program* prog, const scl_shape* shape,
                        void* const* buffers, const void* extra,
                        size_t extra_bytes, const scl_tuning* tuning);

/* ---- Scan that allocates nothing.  No counterpart in the reference.
 *      Same arguments and results as scl_launch_scan, but the scan's scratch
 *      (tile counter and per-tile status) is one fixed array compiled into
 *      this library, so the call never allocates or frees device memory.
 *      It is for callers that must not: a process whose GPU memory belongs
 *      to another allocator (a framework's caching allocator, a server that
 *      reserves nearly all HBM at start-up), where an allocation behind the
 *      owner's back can fail or take memory it had counted on; and a
 *      latency-bound loop, where cudaFree waits for the whole device.
 *      Limit: the scratch must fit in SCL_NOALLOC_SCRATCH_BYTES (4 MiB), which
 *      holds the status of 32766 tiles: 268,419,072 elements of int,
 *      unsigned int or float, or 134,209,536 of double.  Longer inputs return
 *      SCL_ERR_ARG with the limit for their element type in the message;
 *      scl_launch_scan has no such limit.
 *      Only the default tile shape is used (of `tuning`, only spin_limit).
 *      Every GPU that loads this library holds the array until the process
 *      exits.  The first call on a device looks up the array's device
 *      address (once per device), so make that first call before any stream
 *      capture.  All calls share the array and it keeps the last call's
 *      contents; each call clears the part it needs before its kernel runs.
 *      Calls that overlap on the GPU race on it (the library stream runs
 *      its calls one after another). */
#define SCL_NOALLOC_SCRATCH_BYTES (4u << 20)
int scl_launch_scan_noalloc(scl_program* prog, const scl_shape* shape,
                            void* const* buffers, const void* extra,
                            size_t extra_bytes, const scl_tuning* tuning);

/* ---- segment plans (no counterpart in the reference): the offsets pre-pass
 *      of segmented Scan and Reduce, done once per offsets array instead of
 *      on every call.  scl_segplan_create copies `seg_offsets` (DEVICE,
 *      n_segments + 1 entries, for a flat vector of n elements), clamps them
 *      as a segmented launch would (bad offsets are reported by the next
 *      scl_sync) and returns a plan id.  A shape with seg_plan = that id (the
 *      same n_segments, and n at least the plan's) runs its segmented Scan or
 *      Reduce as ONE
 *      launch: the tiles of the long segments first, then one block per
 *      window of segments of up to 4096 elements (a thread per segment of up
 *      to 256 elements, a warp per longer one).  The plan keeps, per tile
 *      shape, which tiles belong to which segment (and each tile's segment)
 *      and the windows; the first launch with a tile shape builds them (four
 *      small launches and a read-back of the offsets), so make it before
 *      capturing a graph.  Later changes to the caller's offsets are not
 *      seen: release the plan and create another. */
int scl_segplan_create(const uint64_t* seg_offsets, uint64_t n_segments, uint64_t n,
                       uint32_t* plan);
int scl_segplan_release(uint32_t plan);
/* The window records a segment plan makes of its short segments (host only,
 * no device): for HOST offsets (n_segments + 1, clamped, non-decreasing)
 * and short_max > 0 (a plan uses half a scan tile), *count receives the
 * number of records and, when `records` is not NULL, up to `capacity`
 * records of four words {first segment, end segment, first element,
 * elements}.  For tests of the plan's host logic. */
int scl_debug_window_records(const uint64_t* offsets, uint64_t n_segments, uint64_t short_max,
                             uint64_t* records, uint64_t capacity, uint64_t* count);

/* ---- adjoint building blocks (no counterpart in the reference; used by the
 *      reverse-mode tape in include/SkelCL/Adjoint.h).  Element types:   */
enum scl_dtype { SCL_DTYPE_F32 = 1, SCL_DTYPE_F64 = 2 };
/* Adjoint of Reduce(+): gx[i] = g (or gx[i] += g with `accumulate`), g read
 * from DEVICE memory (the gradient of the reduced scalar). */
int scl_adjoint_broadcast(const void* g, void* gx, uint64_t n, int dtype, int accumulate);
/* Adjoint of a segmented Reduce(+): gx[i] = g[s] (or += with `accumulate`)
 * for every element i of segment s (shape.seg_offsets semantics, DEVICE
 * offsets, n = length of gx). */
int scl_adjoint_broadcast_segments(const void* g, void* gx, const uint64_t* seg_offsets,
                                   uint64_t n_segments, uint64_t n, int dtype, int accumulate);
/* dst[i] += src[i]: gradient accumulation where an adjoint cannot add itself. */
int scl_adjoint_accumulate(void* dst, const void* src, uint64_t n, int dtype);
/* Adjoint of a linear MapOverlap with NEAREST padding, edge part.  With
 * w = the (2R+1)^2 transposed-stencil weights (w[(dy+R)(2R+1)+dx+R] multiplies
 * g[y+dy][x+dx]) and gin already holding the zero-padded transposed stencil
 * of g, adds to every edge pixel of gin what the clamped reads of the forward
 * sent there from outside the matrix.  Float only. */
int scl_mapoverlap_adjoint_edges(const float* g, const float* w, float* gin, uint64_t rows,
                                 uint64_t cols, int R);

/* ---- autotuner (no counterpart in the reference).  With mode 1 (or
 *      SKELCL_AUTOTUNE=1), a launch given no tuning (NULL or only spin_limit)
 *      whose outputs overlap none of its inputs is timed once per (device,
 *      program, skeleton, log2 size) over a few block sizes / items per thread
 *      (Map, Zip, Reduce), tile shapes (Scan, segmented Scan and Reduce) or
 *      rows per thread and staging (MapOverlap); the fastest is cached in
 *      memory and in SKELCL_CACHE_DIR/autotune.tsv.  Not during a graph
 *      capture: run the sequence once before capturing it. */
int scl_autotune_set(int mode);
int scl_autotune_get(int* mode);

/* Variant the last launch of `prog` used (SCL_VARIANT_*). */
int scl_program_last_variant(const scl_program* prog, uint32_t* variant);
/* Kernels this library launched since scl_init (all programs). */
int scl_launch_count(uint64_t* count);
/* Overlapped launches (no counterpart in the reference).  Skeleton kernels
 * are launched with programmatic stream serialization: a kernel's blocks may
 * be scheduled while the previous kernel on the library stream drains, and
 * each block first waits (griddepcontrol.wait) until that kernel has
 * completed, so results are the same; what is saved is the launch gap
 * between dependent kernels (about 2 us a launch).  On by default;
 * SKELCL_PDL=0 at scl_init, or scl_pdl_set(0), launches them plainly.
 * *previous (may be NULL) receives the earlier setting. */
int scl_pdl_set(int enable, int* previous);
/* Skeleton launches made with programmatic stream serialization since
 * scl_init. */
int scl_pdl_launch_count(uint64_t* count);
/* Device allocations the library has made since scl_init (scl_alloc and its
 * own scratch) and cubins it has loaded; for tests that check a call
 * allocates or loads nothing.  No counterpart in the reference. */
int scl_debug_counters(uint64_t* device_allocs, uint64_t* module_loads);
/* FP32 peak probe (no counterpart in the reference): one launch of 16
 * independent FMA chains per thread, `iters` rounds, 2048 threads per SM,
 * scalar fma.rn.f32 or (packed != 0) fma.rn.f32x2; `sink` receives one float
 * per thread (at least SMs x 2048 floats).  *flops = the launch's FP32 flop
 * count; time it with events on the library stream. */
int scl_debug_fp32_peak(int packed, uint32_t iters, float* sink, uint64_t sink_floats,
                        uint64_t* flops);
/* The split pass of the tensor-core AllPairs alone (no counterpart in the
 * reference): A (M x K) and B (K x N), or their transposes per the
 * SCL_SHAPE_TRANS_* bits in `trans` (bit 0 left, bit 1 right), into `parts`
 * bf16 planes in `scratch`; with scratch NULL only *needed is set.  For
 * timing the split apart from the contraction. */
int scl_debug_allpairs_split(const float* A, const float* B, uint32_t M, uint32_t N,
                             uint32_t K, int parts, int trans, void* scratch,
                             size_t scratch_bytes, size_t* needed);

/* ---- CUDA graphs (no reference counterpart: skeleton sequences captured
 *      from the library stream and replayed with one launch). */
typedef struct scl_graph scl_graph;
int scl_graph_begin(void);
int scl_graph_end(scl_graph** graph);
int scl_graph_launch(scl_graph* graph);
int scl_graph_destroy(scl_graph* graph);

/* ---- test hook for the bounded-wait machinery: launches one block that
 *      waits on a flag nothing sets, with at most `polls` polls, and stores
 *      the kernel's status in *status (SCL_OK or SCL_ERR_TIMEOUT).  Faults
 *      nothing and returns when the wait gives up. */
int scl_debug_bounded_wait(uint32_t polls, int* status);

#ifdef __cplusplus
}
#endif

#endif /* SKELCL_CUDA_H_ */
