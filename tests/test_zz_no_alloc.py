"""scl_launch_scan_noalloc: the scan entry point for callers that may not
allocate device memory (their GPU memory is owned by another allocator, or
they cannot afford cudaFree's wait for the whole device).  Its scratch is a
fixed array inside the library, shared by every call, so these tests call it
twice in a row and compare each result with scl_launch_scan's.  Collected
last, and also run alone in a fresh process."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
ADD_I = "int func(int x, int y){ return x + y; }"
ADD_D = "double func(double x, double y){ return x + y; }"


def scratch_limit_bytes() -> int:
    text = (ROOT / "include" / "skelcl_cuda.h").read_text()
    m = re.search(r"#define SCL_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", text)
    return int(m.group(1)) << int(m.group(2))


def call_noalloc(prog, bufs, n, flags=0):
    ptrs = (ctypes.c_void_p * 2)(*[b.ptr for b in bufs])
    sh = S.Shape(n=n, rows=0, cols=0, dim=0, offset=0, seg_offsets=None, n_segments=0,
                 flags=flags, reserved=0)
    return S.lib().scl_launch_scan_noalloc(prog.handle, ctypes.byref(sh), ptrs, None, 0, None)


def scan_both(p_noalloc, p_ref, x, flags):
    d_in = S.DeviceArray.from_numpy(x)
    d_a = S.DeviceArray(len(x), x.dtype)
    d_b = S.DeviceArray(len(x), x.dtype)
    st = call_noalloc(p_noalloc, [d_in, d_a], len(x), flags)
    assert st == S.OK, S.lib().scl_last_error_string()
    p_ref.launch([d_in, d_b], n=len(x), flags=flags)
    return d_a.to_numpy(), d_b.to_numpy()


@pytest.mark.parametrize("flags", [0, S.SHAPE_INCLUSIVE, S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE])
def test_two_calls_match_scl_launch_scan_int32(scl, orc, flags):
    """Integer scans are bit-exact, so the two entry points must agree bit
    for bit, and the second call must not see the first call's leftovers."""
    p_na = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    p_ref = S.Program(S.KIND_SCAN, ADD_I, ["int"], identity="0")
    for n, seed in [(3_000_001, 11), (3_000_001, 12), (70_001, 13)]:
        x = orc.mod_i32(n, seed, 1000) - 500
        got, want = scan_both(p_na, p_ref, x, flags)
        assert np.array_equal(got, want), (n, seed)


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
