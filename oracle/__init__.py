"""ctypes access to the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as
the checker; the product path (libskelcl_cuda.so and include/SkelCL) never
calls it.  The C sources (oracle.c) say which reference code each function
restates.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_SZ, _U64, _I, _D = ctypes.c_size_t, ctypes.c_uint64, ctypes.c_int, ctypes.c_double

_SIG = {
    "orc_fill_uniform_f32": ([_f32p, _SZ, _U64, _D, _D], None),
    "orc_fill_mod_i32": ([_i32p, _SZ, _U64, ctypes.c_uint32], None),
    "orc_fill_normal_f32": ([_f32p, _SZ, _U64], None),
    "orc_zip_mul_f32": ([_f32p, _f32p, _f32p, _SZ], None),
    "orc_map_mod_i32": ([_i32p, _i32p, _SZ, ctypes.c_int32, _I], None),
    "orc_map_sq1_f32": ([_f32p, _f32p, _SZ], None),
    "orc_sum_f64": ([_f32p, _SZ], _D),
    "orc_dot_f64": ([_f32p, _f32p, _SZ], _D),
    "orc_sum_i32": ([_i32p, _SZ], ctypes.c_int32),
    "orc_sum_f32_reference_order": ([_f32p, _SZ, _SZ, _SZ], ctypes.c_float),
    "orc_scan_excl_i32": ([_i32p, _i32p, _SZ, ctypes.c_int32], None),
    "orc_scan_incl_i32": ([_i32p, _i32p, _SZ], None),
    "orc_scan_incl_mod_i32_mt": ([_i32p, _i32p, _SZ, ctypes.c_int32, _I], None),
    "orc_scan_incl_i32_mt": ([_i32p, _i32p, _SZ, _I], None),
    "orc_scan_f64": ([_f32p, _f64p, _SZ, _I, _I], None),
    "orc_scan_affine_u32": ([_u32p, _u32p, _SZ, _I, _I], None),
    "orc_stencil_f64": ([_f32p, _SZ, _SZ, _I, _f32p, _I, _D, _f64p, _I], None),
    "orc_stencil_adjoint_f64": ([_f32p, _SZ, _SZ, _I, _f32p, _I, _f64p, _I], None),
    "orc_gemm_f64": ([_f32p, _f32p, _SZ, _SZ, _SZ, _f64p, _I], None),
    "orc_gemm_f32_seq": ([_f32p, _f32p, _SZ, _SZ, _SZ, _f32p, _I], None),
    "orc_manhattan_f64": ([_f32p, _f32p, _SZ, _SZ, _SZ, _f64p, _I], None),
}

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            from skelcl_gb300 import build as _b
            _b.build_oracle()
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIG.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _LIB = L
    return _LIB


def threads() -> int:
    import os
    return max(1, min(64, os.cpu_count() or 1))


# ---- generators --------------------------------------------------------------
def uniform_f32(n: int, seed: int, a: float, b: float) -> np.ndarray:
    out = np.empty(n, np.float32)
    lib().orc_fill_uniform_f32(out, n, seed, a, b)
    return out


def mod_i32(n: int, seed: int, modulus: int) -> np.ndarray:
    out = np.empty(n, np.int32)
    lib().orc_fill_mod_i32(out, n, seed, modulus)
    return out


def normal_f32(n: int, seed: int) -> np.ndarray:
    out = np.empty(n, np.float32)
    lib().orc_fill_normal_f32(out, n, seed)
    return out


# ---- skeleton restatements ------------------------------------------------------
def dot_f64(x, y) -> float:
    return lib().orc_dot_f64(np.ascontiguousarray(x, np.float32), np.ascontiguousarray(y, np.float32), len(x))


def sum_f64(x) -> float:
    return lib().orc_sum_f64(np.ascontiguousarray(x, np.float32), len(x))


def sum_i32(x) -> int:
    return lib().orc_sum_i32(np.ascontiguousarray(x, np.int32), len(x))


def sum_f32_reference_order(x, global_size=8192, local_size=256) -> float:
    return lib().orc_sum_f32_reference_order(np.ascontiguousarray(x, np.float32), len(x),
                                             global_size, local_size)


def scan_excl_i32(x, identity=0) -> np.ndarray:
    x = np.ascontiguousarray(x, np.int32)
    out = np.empty_like(x)
    lib().orc_scan_excl_i32(x, out, len(x), identity)
    return out


def scan_incl_i32(x) -> np.ndarray:
    x = np.ascontiguousarray(x, np.int32)
    out = np.empty_like(x)
    lib().orc_scan_incl_i32(x, out, len(x))
    return out


def scan_incl_mod_i32_mt(x, m: int, nthreads: int = 0, out=None) -> np.ndarray:
    x = np.ascontiguousarray(x, np.int32)
    out = np.empty_like(x) if out is None else out
    lib().orc_scan_incl_mod_i32_mt(x, out, len(x), m, nthreads or threads())
    return out


def map_mod_i32(x, m: int, nthreads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x, np.int32)
    out = np.empty_like(x)
    lib().orc_map_mod_i32(x, out, len(x), m, nthreads or threads())
    return out


def scan_f64(x, inclusive=False, reverse=False) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty(len(x), np.float64)
    lib().orc_scan_f64(x, out, len(x), int(inclusive), int(reverse))
    return out


def scan_affine_u32(pairs, inclusive=False, reverse=False) -> np.ndarray:
    """Ordered scan of affine maps {a, b} (x -> a*x + b, uint32 wrapping),
    f(earlier, later) = later after earlier; `pairs` has shape (n, 2)."""
    p = np.ascontiguousarray(pairs, np.uint32).reshape(-1)
    out = np.empty_like(p)
    lib().orc_scan_affine_u32(p, out, len(p) // 2, int(inclusive), int(reverse))
    return out.reshape(-1, 2)


def stencil_f64(img, R: int, w, padding: int, neutral: float = 0.0, nthreads: int = 0) -> np.ndarray:
    img = np.ascontiguousarray(img, np.float32)
    rows, cols = img.shape
    out = np.empty((rows, cols), np.float64)
    lib().orc_stencil_f64(img.ravel(), rows, cols, R, np.ascontiguousarray(w, np.float32).ravel(),
                          padding, neutral, out.ravel(), nthreads or threads())
    return out


def stencil_adjoint_f64(g, R: int, w, padding: int, nthreads: int = 0) -> np.ndarray:
    g = np.ascontiguousarray(g, np.float32)
    rows, cols = g.shape
    out = np.empty((rows, cols), np.float64)
    lib().orc_stencil_adjoint_f64(g.ravel(), rows, cols, R, np.ascontiguousarray(w, np.float32).ravel(),
                                  padding, out.ravel(), nthreads or threads())
    return out


def gemm_f64(A, B, nthreads: int = 0) -> np.ndarray:
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    M, K = A.shape
    K2, N = B.shape
    assert K == K2
    out = np.empty((M, N), np.float64)
    lib().orc_gemm_f64(A.ravel(), B.ravel(), M, N, K, out.ravel(), nthreads or threads())
    return out


def gemm_f32_seq(A, B, nthreads: int = 0) -> np.ndarray:
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    M, K = A.shape
    _, N = B.shape
    out = np.empty((M, N), np.float32)
    lib().orc_gemm_f32_seq(A.ravel(), B.ravel(), M, N, K, out.ravel(), nthreads or threads())
    return out


def manhattan_f64(A, B, nthreads: int = 0) -> np.ndarray:
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    M, K = A.shape
    _, N = B.shape
    out = np.empty((M, N), np.float64)
    lib().orc_manhattan_f64(A.ravel(), B.ravel(), M, N, K, out.ravel(), nthreads or threads())
    return out


def gaussian_weights(R: int = 5, sigma: float = 2.0) -> np.ndarray:
    """(2R+1)^2 Gaussian weights, normalised to sum 1, row-major by (dy, dx)."""
    ax = np.arange(-R, R + 1, dtype=np.float64)
    g = np.exp(-(ax[:, None] ** 2 + ax[None, :] ** 2) / (2 * sigma * sigma))
    return (g / g.sum()).astype(np.float32)
