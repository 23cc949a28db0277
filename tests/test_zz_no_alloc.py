"""scl_launch_scan_noalloc: the scan entry point for callers that may not
allocate device memory (their GPU memory is owned by another allocator, or
they cannot afford cudaFree's wait for the whole device).  Its scratch is a
fixed array inside the library, shared by every call, so these tests call it
twice in a row and compare each result with the oracle's and with
scl_launch_scan's, check that a call allocates nothing and loads no module,
and run this file once more alone in a fresh process.  Collected last."""
import ctypes
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
ADD_I = "int func(int x, int y){ return x + y; }"
ADD_D = "double func(double x, double y){ return x + y; }"
ADD_F = "float func(float x, float y){ return x + y; }"


def scratch_limit_bytes() -> int:
    text = (ROOT / "include" / "skelcl_cuda.h").read_text()
    m = re.search(r"#define SCL_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", text)
    return int(m.group(1)) << int(m.group(2))


def call_noalloc(prog, bufs, n, flags=0, segments=None, n_segments=0):
    ptrs = (ctypes.c_void_p * 2)(*[b.ptr for b in bufs])
    sh = S.Shape(n=n, rows=0, cols=0, dim=0, offset=0,
                 seg_offsets=segments.ptr if segments is not None else None,
                 n_segments=n_segments, flags=flags, seg_plan=0)
    return S.lib().scl_launch_scan_noalloc(prog.handle, ctypes.byref(sh), ptrs, None, 0, None)


def scan_both(p_noalloc, p_ref, x, flags):
    d_in = S.DeviceArray.from_numpy(x)
    d_a = S.DeviceArray(len(x), x.dtype)
    d_b = S.DeviceArray(len(x), x.dtype)
    st = call_noalloc(p_noalloc, [d_in, d_a], len(x), flags)
    assert st == S.OK, S.lib().scl_last_error_string()
    p_ref.launch([d_in, d_b], n=len(x), flags=flags)
    return d_a.to_numpy(), d_b.to_numpy()


def oracle_scan_i32(orc, x, flags):
    v = x[::-1] if flags & S.SHAPE_REVERSE else x
    r = orc.scan_incl_i32(v) if flags & S.SHAPE_INCLUSIVE else orc.scan_excl_i32(v)
    return r[::-1] if flags & S.SHAPE_REVERSE else r


@pytest.mark.parametrize("flags", [0, S.SHAPE_INCLUSIVE, S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE,
                                   S.SHAPE_REVERSE])
def test_two_calls_match_oracle_and_scl_launch_scan_int32(scl, orc, flags):
    """Integer scans are bit-exact: each of two calls in a row equals the
    oracle's wrapping int32 scan and scl_launch_scan's result, and the second
    call does not see the first call's leftovers."""
    p_na = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    p_ref = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    for n, seed in [(3_000_001, 11), (3_000_001, 12), (70_001, 13)]:
        x = orc.mod_i32(n, seed, 1000) - 500
        got, want = scan_both(p_na, p_ref, x, flags)
        assert np.array_equal(got, oracle_scan_i32(orc, x, flags)), (n, seed)
        assert np.array_equal(got, want), (n, seed)


def test_unaligned_views_match_oracle(scl, orc):
    """Inputs and outputs off the 16-byte grid (the tiles shift onto it)."""
    p = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    n = 1_000_007
    x = orc.mod_i32(n + 3, 14, 1000) - 500
    d_in = S.DeviceArray.from_numpy(x)
    d_out = S.DeviceArray(n + 3, np.int32)
    for off in (1, 2, 3):
        vin, vout = d_in.view(off, n), d_out.view(off, n)
        assert call_noalloc(p, [vin, vout], n, S.SHAPE_INCLUSIVE) == S.OK
        assert np.array_equal(d_out.to_numpy()[off:off + n], orc.scan_incl_i32(x[off:off + n])), off


def test_two_calls_match_scl_launch_scan_double(scl, orc):
    """FP64 scans: the look-back may combine tile prefixes in a different
    order on each call, so the results agree to 1e-12 of the running sum of
    magnitudes."""
    p_na = S.Program(S.KIND_SCAN, ADD_D, ["double"], identity="0")
    p_ref = S.Program(S.KIND_SCAN, ADD_D, ["double"], identity="0")
    for seed in (21, 22):
        x = orc.normal_f32(2_000_003, seed).astype(np.float64)
        got, want = scan_both(p_na, p_ref, x, S.SHAPE_INCLUSIVE)
        assert np.all(np.abs(got - want) <= 1e-12 * (np.cumsum(np.abs(x)) + 1.0))


def test_float_scan_matches_fp64_oracle(scl, orc):
    """Float scans (FP64 carries between tiles) against the FP64 oracle, on
    two calls in a row, at the tolerance of the other float scan tests:
    absolute error <= 1e-5 x (1 + sqrt(i)) for U[-1, 1] inputs."""
    p = S.Program(S.KIND_SCAN, ADD_F, ["float"], identity="0.0f")
    n = 4_000_037
    x = orc.uniform_f32(n, 23, -1.0, 1.0)
    ref = orc.scan_f64(x, inclusive=True)
    scale = 1.0 + np.sqrt(np.arange(1, n + 1))
    d_in, d_out = S.DeviceArray.from_numpy(x), S.DeviceArray(n, np.float32)
    for _ in range(2):
        assert call_noalloc(p, [d_in, d_out], n, S.SHAPE_INCLUSIVE) == S.OK
        err = np.abs(d_out.to_numpy().astype(np.float64) - ref)
        assert (err <= 1e-5 * scale).all(), float((err / scale).max())


def test_allocates_nothing_and_loads_no_module(scl, orc):
    """After the program is built, calls make no device allocation and load
    no module (the scan kernels were loaded when the program was built)."""
    p = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    x = orc.mod_i32(5_000_011, 15, 1000)
    d_in, d_out = S.DeviceArray.from_numpy(x), S.DeviceArray(len(x), np.int32)
    S.sync()
    before, launches = S.debug_counters(), S.launch_count()
    for flags in (S.SHAPE_INCLUSIVE, 0, S.SHAPE_REVERSE, S.SHAPE_INCLUSIVE):
        assert call_noalloc(p, [d_in, d_out], len(x), flags) == S.OK
    S.sync()
    assert S.debug_counters() == before
    assert S.launch_count() == launches + 4
    assert np.array_equal(d_out.to_numpy(), orc.scan_incl_i32(x))


def test_rejects_inputs_beyond_the_fixed_scratch(scl):
    """A scan that needs more status lines than the fixed array holds is
    refused before anything runs on the GPU; the message names the limit."""
    p = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    tiles = (scratch_limit_bytes() - 256) // 128  # one 128-byte line per tile
    limit = tiles * 8 * 256 * 4                    # 8 x 256 threads x 4 ints per tile
    n = limit + 1
    d_in = S.DeviceArray(n, np.int32)  # real buffers of that length
    d_out = S.DeviceArray(n, np.int32)
    before = S.launch_count()
    st = call_noalloc(p, [d_in, d_out], n)
    assert st == S.ERR_ARG
    assert str(limit).encode() in S.lib().scl_last_error_string()
    assert S.launch_count() == before
    # the entry point still works after a refusal
    x = np.arange(10_000, dtype=np.int32)
    d_x = S.DeviceArray.from_numpy(x)
    d_y = S.DeviceArray(len(x), np.int32)
    assert call_noalloc(p, [d_x, d_y], len(x), S.SHAPE_INCLUSIVE) == S.OK
    assert np.array_equal(d_y.to_numpy(), np.cumsum(x, dtype=np.int32))


def test_refuses_segmented_shapes(scl):
    """One vector only: a shape with segments is refused (scl_launch_scan
    handles those), and nothing is launched."""
    p = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    off = S.DeviceArray.from_numpy(np.array([0, 5, 10], np.uint64))
    d_x, d_y = S.DeviceArray.from_numpy(np.ones(10, np.int32)), S.DeviceArray(10, np.int32)
    before = S.launch_count()
    assert call_noalloc(p, [d_x, d_y], 10, S.SHAPE_INCLUSIVE, segments=off, n_segments=2) == S.ERR_UNSUPPORTED
    assert b"segment" in S.lib().scl_last_error_string()
    assert S.launch_count() == before


@pytest.mark.skipif(os.environ.get("SKELCL_NOALLOC_CHILD") == "1", reason="already the fresh process")
def test_whole_file_in_a_fresh_process(scl):
    """The same tests, alone in a new process: the first call on the device
    (which looks up the array's address) happens there with nothing run
    before it."""
    env = dict(os.environ, SKELCL_NOALLOC_CHILD="1")
    r = subprocess.run([sys.executable, "-m", "pytest", str(Path(__file__)), "-q", "-x", "-m", "gpu",
                        "-p", "no:cacheprovider"], cwd=str(ROOT), env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
