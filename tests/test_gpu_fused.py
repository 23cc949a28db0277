"""Fused skeleton pairs: Reduce(Zip(x, y)) and Map(Scan(x)) in one kernel,
against the oracle and against the unfused pair (bit-exact for integers)."""
import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

ADD_F = "float func(float x, float y){ return x + y; }"
MUL_F = "float mult(float x, float y){ return x * y; }"


def dev(a):
    return S.DeviceArray.from_numpy(np.ascontiguousarray(a))


def test_zip_reduce_empty_gives_identity(scl):
    p = S.Program(S.KIND_ZIP_REDUCE, "int func(int x, int y){ return x + y; }", ["int"] * 3,
                  source2="int m(int x, int y){ return x * y; }", func2="m", identity="0")
    out = dev(np.array([12345], np.int32))
    p.launch([out, out, out], n=0)
    assert out.to_numpy()[0] == 0


@pytest.mark.parametrize("n", [1, 5, 4099, 1 << 24])
def test_zip_reduce_dot_product(scl, orc, n):
    x = orc.uniform_f32(n, 0, -1.0, 1.0)
    y = orc.uniform_f32(n, 1, -1.0, 1.0)
    p = S.Program(S.KIND_ZIP_REDUCE, ADD_F, ["float"] * 3, source2=MUL_F, func2="mult", identity="0")
    out = S.DeviceArray(1, np.float32)
    dx, dy = dev(x), dev(y)
    p.launch([dx, dy, out], n=n)
    ref = orc.dot_f64(x, y)
    got = float(out.to_numpy()[0])
    assert abs(got - ref) <= 1e-5 * max(1.0, abs(ref)) + 1e-6 * np.sqrt(n)  # rel 1e-5 (dot tests)


def test_zip_reduce_int_with_extras_exact(scl, orc):
    n = 3_000_001
    x = orc.mod_i32(n, 2, 1001) - 500
    y = orc.mod_i32(n, 3, 1001) - 500
    red = "int func(int a, int b, int bias){ return a + b + 0 * bias; }"
    zip_ = "int f(int a, int b, int k){ return (a - b) * k; }"
    p = S.Program(S.KIND_ZIP_REDUCE, red, ["int"] * 3, source2=zip_, func2="f", identity="0")
    out = S.DeviceArray(1, np.int32)
    p.launch([dev(x), dev(y), out], n=n, extra=S.pack(S.value(np.int32(7)), S.value(np.int32(3))))
    ref = np.int64(((x.astype(np.int64) - y) * 3).sum()).astype(np.int32)
    assert out.to_numpy()[0] == ref


@pytest.mark.parametrize("flags", [0, S.SHAPE_INCLUSIVE, S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE])
def test_scan_map_matches_unfused(scl, orc, flags):
    n = (1 << 22) + 77
    x = orc.mod_i32(n, 4, 1001)
    sp = S.Program(S.KIND_SCAN, "int func(int x, int y){ return x + y; }", ["int"], identity="0")
    mp = S.Program(S.KIND_MAP, "int func(int x){ return x % 7919; }", ["int", "int"])
    fp = S.Program(S.KIND_SCAN_MAP, "int func(int x, int y){ return x + y; }", ["int", "int"],
                   source2="int m(int x){ return x % 7919; }", func2="m", identity="0")
    dx = dev(x)
    a, b = S.DeviceArray(n, np.int32), S.DeviceArray(n, np.int32)
    sp.launch([dx, a], n=n, flags=flags)
    mp.launch([a, a], n=n)
    fp.launch([dx, b], n=n, flags=flags)
    assert np.array_equal(a.to_numpy(), b.to_numpy())
    if flags == S.SHAPE_INCLUSIVE:
        assert np.array_equal(b.to_numpy(), orc.scan_incl_mod_i32_mt(x, 7919))


def test_scan_map_changes_type_and_takes_extras(scl, orc):
    n = 1_000_003
    x = orc.uniform_f32(n, 5, -1.0, 1.0)
    fp = S.Program(S.KIND_SCAN_MAP, "float func(float x, float y){ return x + y; }", ["float", "double"],
                   source2="double m(float s, double k){ return (double)s * k; }", func2="m", identity="0")
    out = S.DeviceArray(n, np.float64)
    fp.launch([dev(x), out], n=n, flags=S.SHAPE_INCLUSIVE, extra=S.value(np.float64(2.0)))
    ref = 2.0 * orc.scan_f64(x, inclusive=True)
    scale = 1.0 + np.sqrt(np.arange(1, n + 1))
    assert np.all(np.abs(out.to_numpy() - ref) <= 2e-5 * scale)


def test_scan_map_segmented(scl, orc):
    off = np.array([0, 1, 10_000, 10_003, 500_000], np.uint64)
    n = int(off[-1])
    x = orc.mod_i32(n, 6, 1001)
    fp = S.Program(S.KIND_SCAN_MAP, "int func(int x, int y){ return x + y; }", ["int", "int"],
                   source2="int m(int x){ return x % 101; }", func2="m", identity="0")
    out = S.DeviceArray(n, np.int32)
    fp.launch([dev(x), out], n=n, flags=S.SHAPE_INCLUSIVE, segments=dev(off))
    x64 = x.astype(np.int64)
    ref = np.concatenate([np.cumsum(x64[int(a):int(b)]) % 101 for a, b in zip(off[:-1], off[1:])])
    assert np.array_equal(out.to_numpy(), ref.astype(np.int32))
