"""Python access to libskelcl_cuda.so through its C ABI (include/skelcl_cuda.h).

This module is the plumbing the tests and bench.py use to drive the GB300
skeleton runtime directly; programs written against the SkelCL C++ API use
the headers in include/SkelCL instead.  There is no CPU fallback: if the
CUDA library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import struct
from pathlib import Path
from typing import Iterable, Optional, Sequence

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libskelcl_cuda.so"

# ---- constants (mirror include/skelcl_cuda.h) ------------------------------
OK, ERR_ARG, ERR_OOM, ERR_COMPILE, ERR_LAUNCH, ERR_TIMEOUT, ERR_CUDA, ERR_NOT_INIT, ERR_UNSUPPORTED = range(9)
KIND_MAP, KIND_MAP_VOID, KIND_MAP_INDEX, KIND_MAP_INDEX_VOID = 1, 2, 3, 4
KIND_MAP_POINT, KIND_MAP_POINT_VOID, KIND_ZIP, KIND_ZIP_VOID = 5, 6, 7, 8
KIND_REDUCE, KIND_SCAN, KIND_MAPOVERLAP, KIND_ALLPAIRS, KIND_ALLPAIRS_GENERIC = 9, 10, 11, 12, 13
KIND_MAP_ADJOINT, KIND_ZIP_ADJOINT, KIND_ZIP_REDUCE, KIND_SCAN_MAP = 14, 15, 16, 17
PAD_NEUTRAL, PAD_NEAREST = 0, 1
SHAPE_INCLUSIVE, SHAPE_REVERSE = 1, 2
SHAPE_ACCUMULATE, SHAPE_ACCUMULATE_RIGHT, SHAPE_TRANS_LEFT, SHAPE_TRANS_RIGHT = 4, 8, 16, 32
DTYPE_F32, DTYPE_F64 = 1, 2
VARIANT_AUTO, VARIANT_SIMPLE, VARIANT_VECTOR, VARIANT_SIMT, VARIANT_TC3XBF16, VARIANT_TMA, VARIANT_LDST = range(7)
ARG_VALUE, ARG_BUFFER, ARG_MATRIX, ARG_LOCAL = 1, 2, 3, 4
PROG_NO_F64_CARRY, PROG_STENCIL_COLS1, PROG_STENCIL_COLS2, PROG_COMPILE_ALL = 1, 2, 4, 8

CL_TYPE = {
    np.dtype(np.float32): "float", np.dtype(np.float64): "double",
    np.dtype(np.int32): "int", np.dtype(np.uint32): "unsigned int",
    np.dtype(np.int64): "long", np.dtype(np.uint64): "unsigned long",
    np.dtype(np.int16): "short", np.dtype(np.uint16): "unsigned short",
    np.dtype(np.int8): "char", np.dtype(np.uint8): "unsigned char",
}


class SclError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status
        self.message = message


class ProgramDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("source", ctypes.c_char_p), ("func", ctypes.c_char_p),
                ("source2", ctypes.c_char_p), ("func2", ctypes.c_char_p),
                ("identity", ctypes.c_char_p), ("type_names", ctypes.c_char_p * 3),
                ("n_types", ctypes.c_int), ("overlap_range", ctypes.c_int),
                ("padding", ctypes.c_int), ("neutral", ctypes.c_char_p),
                ("common_source", ctypes.c_char_p), ("flags", ctypes.c_uint32)]


class Shape(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("rows", ctypes.c_uint64), ("cols", ctypes.c_uint64),
                ("dim", ctypes.c_uint64), ("offset", ctypes.c_uint64),
                ("seg_offsets", ctypes.c_void_p), ("n_segments", ctypes.c_uint64),
                ("flags", ctypes.c_uint32), ("seg_plan", ctypes.c_uint32)]


class Tuning(ctypes.Structure):
    _fields_ = [("workgroup", ctypes.c_uint32), ("items", ctypes.c_uint32),
                ("tile_w", ctypes.c_uint32), ("tile_h", ctypes.c_uint32),
                ("variant", ctypes.c_uint32), ("spin_limit", ctypes.c_uint32)]


# Every function the header declares, with its ctypes signature.
_VP, _SZ, _I, _U32, _U64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64
SIGNATURES = {
    "scl_init": ([_I], _I), "scl_terminate": ([], _I), "scl_is_initialized": ([], _I),
    "scl_device_info": ([ctypes.POINTER(_I), ctypes.POINTER(_SZ), ctypes.c_char_p, _SZ], _I),
    "scl_last_error_string": ([], ctypes.c_char_p), "scl_abi_version": ([], _I),
    "scl_alloc": ([_SZ, ctypes.POINTER(_VP)], _I), "scl_free": ([_VP], _I),
    "scl_h2d": ([_VP, _VP, _SZ], _I), "scl_d2h": ([_VP, _VP, _SZ], _I),
    "scl_d2d": ([_VP, _VP, _SZ], _I), "scl_h2d_async": ([_VP, _VP, _SZ], _I),
    "scl_d2h_async": ([_VP, _VP, _SZ], _I), "scl_memset": ([_VP, _I, _SZ], _I),
    "scl_host_alloc": ([_SZ, ctypes.POINTER(_VP)], _I), "scl_host_free": ([_VP], _I),
    "scl_sync": ([], _I),
    "scl_event_create": ([ctypes.POINTER(_VP)], _I), "scl_event_record": ([_VP], _I),
    "scl_event_elapsed_ms": ([_VP, _VP, ctypes.POINTER(ctypes.c_float)], _I),
    "scl_event_destroy": ([_VP], _I),
    "scl_program_build": ([ctypes.POINTER(ProgramDesc), ctypes.POINTER(_VP), ctypes.c_char_p, _SZ], _I),
    "scl_program_compile": ([ctypes.POINTER(ProgramDesc), ctypes.c_char_p, _SZ], _I),
    "scl_program_release": ([_VP], _I),
    "scl_program_extra_count": ([_VP, ctypes.POINTER(_I)], _I),
    "scl_program_hash": ([_VP, ctypes.c_char_p], _I),
    "scl_program_source": ([ctypes.POINTER(ProgramDesc), ctypes.c_char_p, _SZ, ctypes.POINTER(_SZ)], _I),
    "scl_program_last_variant": ([_VP, ctypes.POINTER(_U32)], _I),
    "scl_sha1_hex": ([_VP, _SZ, ctypes.c_char_p], _I),
    "scl_cache_stats": ([ctypes.POINTER(ctypes.c_uint64)] * 4, _I),
    "scl_segplan_create": ([_VP, _U64, _U64, ctypes.POINTER(_U32)], _I),
    "scl_segplan_release": ([_U32], _I),
    "scl_launch_map": ([_VP, ctypes.POINTER(Shape), ctypes.POINTER(_VP), _VP, _SZ, ctypes.POINTER(Tuning)], _I),
    "scl_launch_zip": ([_VP, ctypes.POINTER(Shape), ctypes.POINTER(_VP), _VP, _SZ, ctypes.POINTER(Tuning)], _I),
    "scl_launch_reduce": ([_VP, ctypes.POINTER(Shape), ctypes.POINTER(_VP), _VP, _SZ, ctypes.POINTER(Tuning)], _I),
    "scl_launch_scan": ([_VP, ctypes.POINTER(Shape), ctypes.POINTER(_VP), _VP, _SZ, ctypes.POINTER(Tuning)], _I),
    "scl_launch_scan_noalloc": ([_VP, ctypes.POINTER(Shape), ctypes.POINTER(_VP), _VP, _SZ, ctypes.POINTER(Tuning)], _I),
    "scl_launch_mapoverlap": ([_VP, ctypes.POINTER(Shape), ctypes.POINTER(_VP), _VP, _SZ, ctypes.POINTER(Tuning)], _I),
    "scl_launch_allpairs": ([_VP, ctypes.POINTER(Shape), ctypes.POINTER(_VP), _VP, _SZ, ctypes.POINTER(Tuning)], _I),
    "scl_launch_count": ([ctypes.POINTER(_U64)], _I),
    "scl_pdl_set": ([ctypes.c_int, ctypes.POINTER(ctypes.c_int)], _I),
    "scl_debug_window_records": ([_VP, _U64, _U64, _VP, _U64, ctypes.POINTER(_U64)], _I),
    "scl_pdl_launch_count": ([ctypes.POINTER(_U64)], _I),
    "scl_debug_counters": ([ctypes.POINTER(_U64), ctypes.POINTER(_U64)], _I),
    "scl_debug_fp32_peak": ([_I, _U32, _VP, _U64, ctypes.POINTER(_U64)], _I),
    "scl_debug_allpairs_split": ([_VP, _VP, _U32, _U32, _U32, _I, _I, _VP, _SZ, ctypes.POINTER(_SZ)], _I),
    "scl_graph_begin": ([], _I), "scl_graph_end": ([ctypes.POINTER(_VP)], _I),
    "scl_graph_launch": ([_VP], _I), "scl_graph_destroy": ([_VP], _I),
    "scl_debug_bounded_wait": ([_U32, ctypes.POINTER(_I)], _I),
    "scl_adjoint_broadcast": ([_VP, _VP, _U64, _I, _I], _I),
    "scl_adjoint_accumulate": ([_VP, _VP, _U64, _I], _I),
    "scl_adjoint_broadcast_segments": ([_VP, _VP, _VP, _U64, _U64, _I, _I], _I),
    "scl_autotune_set": ([_I], _I), "scl_autotune_get": ([ctypes.POINTER(_I)], _I),
    "scl_h2d_on": ([_I, _VP, _VP, _SZ], _I), "scl_d2h_on": ([_I, _VP, _VP, _SZ], _I),
    "scl_event_record_on": ([_VP, _I], _I), "scl_stream_wait": ([_I, _VP], _I),
    "scl_mapoverlap_adjoint_edges": ([_VP, _VP, _VP, _U64, _U64, _I], _I),
}

_LIB: Optional[ctypes.CDLL] = None


def lib() -> ctypes.CDLL:
    """Load libskelcl_cuda.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built: run `python -m skelcl_gb300.build`")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def check(status: int) -> None:
    if status != OK:
        raise SclError(status, lib().scl_last_error_string().decode(errors="replace"))


def init(device: int = 0) -> None:
    check(lib().scl_init(device))


def terminate() -> None:
    check(lib().scl_terminate())


def sync() -> None:
    check(lib().scl_sync())


def launch_count() -> int:
    v = ctypes.c_uint64(0)
    check(lib().scl_launch_count(ctypes.byref(v)))
    return v.value


def set_overlapped_launches(enable: bool) -> bool:
    """Launch skeleton kernels with programmatic stream serialization (the
    default) or plainly; returns the previous setting."""
    prev = ctypes.c_int(0)
    check(lib().scl_pdl_set(1 if enable else 0, ctypes.byref(prev)))
    return bool(prev.value)


def overlapped_launch_count() -> int:
    """Skeleton launches made with programmatic stream serialization."""
    v = ctypes.c_uint64(0)
    check(lib().scl_pdl_launch_count(ctypes.byref(v)))
    return v.value


def window_records(offsets, short_max: int):
    """The window records a segment plan makes of its short segments, as an
    (n, 4) uint64 array {first segment, end segment, first element,
    elements}; host only."""
    import numpy as np
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    n_seg = len(off) - 1
    cnt = ctypes.c_uint64(0)
    check(lib().scl_debug_window_records(off.ctypes.data, n_seg, short_max, None, 0, ctypes.byref(cnt)))
    rec = np.zeros((cnt.value, 4), np.uint64)
    check(lib().scl_debug_window_records(off.ctypes.data, n_seg, short_max, rec.ctypes.data, cnt.value,
                                         ctypes.byref(cnt)))
    return rec


def sha1_hex(data: bytes) -> str:
    out = ctypes.create_string_buffer(41)
    check(lib().scl_sha1_hex(data, len(data), out))
    return out.value.decode()


# ---- device memory -----------------------------------------------------------
class DeviceArray:
    """A device allocation with a dtype and a flat element count."""

    def __init__(self, n: int, dtype, ptr: Optional[int] = None):
        self.dtype = np.dtype(dtype)
        self.n = int(n)
        self.nbytes = self.n * self.dtype.itemsize
        if ptr is None:
            p = ctypes.c_void_p()
            check(lib().scl_alloc(max(self.nbytes, 16), ctypes.byref(p)))
            self.ptr = p.value
            self._owned = True
        else:
            self.ptr = ptr
            self._owned = False

    @classmethod
    def from_numpy(cls, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a)
        d = cls(a.size, a.dtype)
        if a.nbytes:
            check(lib().scl_h2d(d.ptr, a.ctypes.data, a.nbytes))
        return d

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.size == self.n
        check(lib().scl_h2d(self.ptr, a.ctypes.data, a.nbytes))

    def to_numpy(self) -> np.ndarray:
        out = np.empty(self.n, dtype=self.dtype)
        if self.nbytes:
            check(lib().scl_d2h(out.ctypes.data, self.ptr, self.nbytes))
        return out

    def view(self, offset_elems: int, n: int) -> "DeviceArray":
        v = DeviceArray(n, self.dtype, ptr=self.ptr + offset_elems * self.dtype.itemsize)
        v._base = self  # the allocation lives as long as its views
        return v

    def free(self) -> None:
        if self._owned and self.ptr:
            check(lib().scl_free(self.ptr))
        self.ptr = 0

    def __del__(self):
        try:
            if self._owned and self.ptr and _LIB is not None and _LIB.scl_is_initialized():
                _LIB.scl_free(self.ptr)
                self.ptr = 0
        except Exception:
            pass


# ---- extra-argument blob -------------------------------------------------------
def _record(kind: int, payload: bytes) -> bytes:
    pad = (-len(payload)) % 8
    return struct.pack("<II", kind, len(payload)) + payload + b"\0" * pad


def value(v, dtype=None) -> bytes:
    if isinstance(v, (bytes, bytearray)):
        return _record(ARG_VALUE, bytes(v))
    arr = np.asarray(v, dtype=dtype) if dtype is not None else np.asarray(v)
    return _record(ARG_VALUE, arr.tobytes())


def buffer(d: DeviceArray) -> bytes:
    return _record(ARG_BUFFER, struct.pack("<Q", d.ptr))


def matrix(d: DeviceArray, cols: int) -> bytes:
    return _record(ARG_MATRIX, struct.pack("<QI", d.ptr, cols))


def local(nbytes: int) -> bytes:
    return _record(ARG_LOCAL, struct.pack("<Q", nbytes))


def pack(*records: bytes) -> bytes:
    return b"".join(records)


# ---- programs ---------------------------------------------------------------------
def make_desc(kind: int, source: str, types: Sequence[str], func: str = "func",
              identity: Optional[str] = None, source2: Optional[str] = None,
              func2: Optional[str] = None, overlap_range: int = 0, padding: int = PAD_NEAREST,
              neutral: Optional[str] = None, common: Optional[str] = None,
              flags: int = 0):
    d = ProgramDesc()
    keep = []

    def enc(s):
        if s is None:
            return None
        b = s.encode()
        keep.append(b)
        return b

    d.kind = kind
    d.source = enc(source)
    d.func = enc(func)
    d.source2 = enc(source2)
    d.func2 = enc(func2 if func2 is not None else ("func" if source2 is not None else None))
    d.identity = enc(identity)
    d.n_types = len(types)
    for i, t in enumerate(types):
        d.type_names[i] = enc(t)
    d.overlap_range = overlap_range
    d.padding = padding
    d.neutral = enc(neutral)
    d.common_source = enc(common)
    d.flags = flags
    return d, keep


def compile_only(kind: int, source: str, types: Sequence[str], **kw) -> str:
    """Splice + NVRTC-compile without a device; returns the build log."""
    d, keep = make_desc(kind, source, types, **kw)
    log = ctypes.create_string_buffer(1 << 16)
    check(lib().scl_program_compile(ctypes.byref(d), log, len(log)))
    return log.value.decode(errors="replace")


def debug_counters() -> dict:
    """Device allocations and module loads the library has made."""
    a, m = ctypes.c_uint64(0), ctypes.c_uint64(0)
    check(lib().scl_debug_counters(ctypes.byref(a), ctypes.byref(m)))
    return {"device_allocs": a.value, "module_loads": m.value}


def cache_stats() -> dict:
    """Counters of the program binary cache since the library was loaded."""
    v = [ctypes.c_uint64(0) for _ in range(4)]
    check(lib().scl_cache_stats(*[ctypes.byref(x) for x in v]))
    return dict(zip(("nvrtc_compiles", "disk_loads", "disk_rejects", "disk_saves"), (x.value for x in v)))


def generated_source(kind: int, source: str, types: Sequence[str], **kw) -> str:
    d, keep = make_desc(kind, source, types, **kw)
    need = ctypes.c_size_t(0)
    check(lib().scl_program_source(ctypes.byref(d), None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(need.value)
    check(lib().scl_program_source(ctypes.byref(d), buf, need.value, None))
    return buf.value.decode()


_LAUNCH = {KIND_MAP: "scl_launch_map", KIND_MAP_VOID: "scl_launch_map",
           KIND_MAP_INDEX: "scl_launch_map", KIND_MAP_INDEX_VOID: "scl_launch_map",
           KIND_MAP_POINT: "scl_launch_map", KIND_MAP_POINT_VOID: "scl_launch_map",
           KIND_ZIP: "scl_launch_zip", KIND_ZIP_VOID: "scl_launch_zip",
           KIND_REDUCE: "scl_launch_reduce", KIND_SCAN: "scl_launch_scan",
           KIND_MAPOVERLAP: "scl_launch_mapoverlap", KIND_ALLPAIRS: "scl_launch_allpairs",
           KIND_ALLPAIRS_GENERIC: "scl_launch_allpairs",
           KIND_MAP_ADJOINT: "scl_launch_map", KIND_ZIP_ADJOINT: "scl_launch_map",
           KIND_ZIP_REDUCE: "scl_launch_reduce", KIND_SCAN_MAP: "scl_launch_scan"}


class SegPlan:
    """A segment plan (scl_segplan_create) for a DeviceArray of n_segments+1
    uint64 offsets over a flat vector of n elements: segmented Scan and
    Reduce launches given it run as one kernel each."""

    def __init__(self, offsets: "DeviceArray", n: int):
        self.offsets, self.n = offsets, n
        pid = ctypes.c_uint32(0)
        check(lib().scl_segplan_create(offsets.ptr, offsets.n - 1, n, ctypes.byref(pid)))
        self.id = pid.value

    def release(self) -> None:
        if getattr(self, "id", 0):
            lib().scl_segplan_release(self.id)
            self.id = 0

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class Program:
    """A built skeleton program (one NVRTC module)."""

    def __init__(self, kind: int, source: str, types: Sequence[str], **kw):
        d, keep = make_desc(kind, source, types, **kw)
        h = ctypes.c_void_p()
        log = ctypes.create_string_buffer(1 << 16)
        st = lib().scl_program_build(ctypes.byref(d), ctypes.byref(h), log, len(log))
        if st != OK:
            raise SclError(st, lib().scl_last_error_string().decode(errors="replace"))
        self.handle = h.value
        self.kind = kind

    def launch(self, bufs: Iterable, n: int = 0, rows: int = 0, cols: int = 0, dim: int = 0,
               offset: int = 0, flags: int = 0, extra: bytes = b"",
               tuning: Optional[Tuning] = None, segments=None) -> None:
        """`segments`: a DeviceArray of n_segments+1 uint64 offsets, or a
        SegPlan made for them (segmented Scan/Reduce)."""
        ptrs = [b.ptr if isinstance(b, DeviceArray) else (b or 0) for b in bufs]
        arr = (ctypes.c_void_p * max(1, len(ptrs)))(*ptrs)
        plan = 0
        if isinstance(segments, SegPlan):
            plan, segments = segments.id, segments.offsets
        sh = Shape(n=n, rows=rows, cols=cols, dim=dim, offset=offset,
                   seg_offsets=segments.ptr if segments is not None else None,
                   n_segments=(segments.n - 1) if segments is not None else 0, flags=flags,
                   seg_plan=plan)
        eb = ctypes.create_string_buffer(extra, len(extra)) if extra else None
        fn = getattr(lib(), _LAUNCH[self.kind])
        check(fn(self.handle, ctypes.byref(sh), arr, eb, len(extra),
                 ctypes.byref(tuning) if tuning is not None else None))

    @property
    def last_variant(self) -> int:
        v = ctypes.c_uint32(0)
        check(lib().scl_program_last_variant(self.handle, ctypes.byref(v)))
        return v.value

    @property
    def extra_count(self) -> int:
        v = ctypes.c_int(0)
        check(lib().scl_program_extra_count(self.handle, ctypes.byref(v)))
        return v.value

    def release(self) -> None:
        if self.handle:
            lib().scl_program_release(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            if self.handle and _LIB is not None:
                _LIB.scl_program_release(self.handle)
                self.handle = 0
        except Exception:
            pass


class Event:
    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().scl_event_create(ctypes.byref(h)))
        self.handle = h.value

    def record(self) -> None:
        check(lib().scl_event_record(self.handle))

    def record_on(self, stream: int) -> None:
        """Record on stream 0 (launches) or copy stream 1 / 2."""
        check(lib().scl_event_record_on(self.handle, stream))

    def wait_on(self, stream: int) -> None:
        """Make `stream` wait for this event."""
        check(lib().scl_stream_wait(stream, self.handle))

    def elapsed_ms(self, later: "Event") -> float:
        ms = ctypes.c_float(0)
        check(lib().scl_event_elapsed_ms(self.handle, later.handle, ctypes.byref(ms)))
        return ms.value

    def __del__(self):
        try:
            if self.handle and _LIB is not None:
                _LIB.scl_event_destroy(self.handle)
        except Exception:
            pass
