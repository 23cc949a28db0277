"""GPU parity tests: every skeleton through the C ABI against the CPU oracle
and the reference's known answers.  Integer / index results must be
bit-exact; float results are checked against FP64 with the tolerance written
in each test."""
import ctypes
import json
from pathlib import Path

import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def kat(cid):
    return next(k for k in KATS if k["id"] == cid)


def dev(a):
    return S.DeviceArray.from_numpy(np.ascontiguousarray(a))


def run_map(src, x, tout, extra=b"", kind=S.KIND_MAP, tin=None, **kw):
    tin = tin or S.CL_TYPE[x.dtype]
    p = S.Program(kind, src, [tin, S.CL_TYPE[np.dtype(tout)]])
    din = dev(x)
    dout = S.DeviceArray(x.size, tout)
    p.launch([din, dout], n=x.size, extra=extra, **kw)
    return dout.to_numpy(), p


def run_reduce(src, x, extra=b"", identity="0", **kw):
    p = S.Program(S.KIND_REDUCE, src, [S.CL_TYPE[x.dtype]], identity=identity)
    din = dev(x)
    dout = S.DeviceArray(1, x.dtype)
    p.launch([din, dout], n=x.size, extra=extra, **kw)
    return dout.to_numpy()[0]


def run_scan(src, x, identity="0", flags=0, tuning=None):
    p = S.Program(S.KIND_SCAN, src, [S.CL_TYPE[x.dtype]], identity=identity)
    din = dev(x)
    dout = S.DeviceArray(x.size, x.dtype)
    p.launch([din, dout], n=x.size, flags=flags, tuning=tuning)
    return dout.to_numpy()


# ---- Map / Zip (test/MapTests.cpp, test/ZipTests.cpp) ------------------------------
def test_map_simple_and_add_args(scl):
    x = (np.arange(10) * 2.5).astype(np.float32)
    out, _ = run_map("float func(float f){ return -f; }", x, np.float32)
    assert np.array_equal(out, -x)
    out, _ = run_map("float func(float f, float add, float add2) { return f+add+add2; }", x, np.float32,
                     extra=S.pack(S.value(5.25, np.float32), S.value(7.75, np.float32)))
    assert np.array_equal(out, x + np.float32(5.25) + np.float32(7.75))


@pytest.mark.parametrize("n", [1, 3, 4, 5, 1023, 4096, 100_003, 1 << 22])
def test_map_sizes_vector_path(scl, n):
    x = (np.arange(n) % 1000).astype(np.int32)
    out, p = run_map("int func(int x){ return x % 7; }", x, np.int32)
    assert np.array_equal(out, np.fmod(x, 7))
    assert p.last_variant == S.VARIANT_VECTOR


def test_map_unaligned_views(scl):
    x = np.arange(1001, dtype=np.float32)
    p = S.Program(S.KIND_MAP, "float func(float f){ return 2.0f*f; }", ["float", "float"])
    din = dev(x)
    dout = S.DeviceArray(1002, np.float32)
    p.launch([din.view(1, 999), dout.view(3, 999)], n=999)  # views end inside both buffers
    assert np.array_equal(dout.to_numpy()[3:1002], 2 * x[1:1000])


def test_map_void_uses_global_id(scl):
    x = (np.arange(10) * 2.5).astype(np.float32)
    p = S.Program(S.KIND_MAP_VOID, "void func(float f, __global float* out) { out[get_global_id(0)] = f; }",
                  ["float"])
    din, dout = dev(x), S.DeviceArray(10, np.float32)
    p.launch([din], n=10, extra=S.buffer(dout))
    assert np.array_equal(dout.to_numpy(), x)
    assert p.last_variant == S.VARIANT_SIMPLE


def test_map_matrix_extra_args(scl):
    x = (np.arange(12) * 2.5).astype(np.float32)
    mat = np.arange(12, dtype=np.float32)
    mat2 = np.zeros(6, np.int32)
    mat2[1 * 3 + 2] = 5
    dmat, dmat2 = dev(mat), dev(mat2)
    out, _ = run_map("float func( float f, float_matrix_t mat, float add2, int_matrix_t mat2 )"
                     "{ return f + get(mat, 1, 1) + add2 + get(mat2, 1, 2); }", x, np.float32,
                     extra=S.pack(S.matrix(dmat, 3), S.value(7.75, np.float32), S.matrix(dmat2, 3)))
    assert np.array_equal(out, x + mat[1 * 3 + 1] + np.float32(7.75) + np.float32(5))


def test_map_with_local_memory(scl):
    x = np.full(32, 5, np.int32)
    out, p = run_map("int func(int i, __local int* lp) { lp[0] = i; barrier(CLK_LOCAL_MEM_FENCE); return -lp[0]; }",
                     x, np.int32, extra=S.local(4), tuning=S.Tuning(workgroup=16))
    assert np.array_equal(out, -x)


def test_map_float4(scl):
    x = np.tile(np.array([1, 2, 3, 4], np.float32), 10)
    p = S.Program(S.KIND_MAP, "float4 func(float4 f) { return -f; }", ["float4", "float4"])
    din, dout = dev(x), S.DeviceArray(40, np.float32)
    p.launch([din, dout], n=10)
    assert np.array_equal(dout.to_numpy(), -x)


def test_extra_arg_mismatch_is_an_error(scl):
    p = S.Program(S.KIND_MAP, "float func(float f, float a){ return f + a; }", ["float", "float"])
    din, dout = dev(np.ones(4, np.float32)), S.DeviceArray(4, np.float32)
    with pytest.raises(S.SclError) as e:
        p.launch([din, dout], n=4)
    assert e.value.status == S.ERR_ARG
    with pytest.raises(S.SclError) as e:
        p.launch([din, dout], n=4, extra=S.value(1.0, np.float64))
    assert e.value.status == S.ERR_ARG


def test_zip_kats(scl):
    l = (np.arange(10) * 2.5).astype(np.float32)
    r = (np.arange(10) * 7.5).astype(np.float32)
    p = S.Program(S.KIND_ZIP, "float func(float x, float y){ return x+y; }", ["float"] * 3)
    dl, dr, do = dev(l), dev(r), S.DeviceArray(10, np.float32)
    p.launch([dl, dr, do], n=10)
    assert np.array_equal(do.to_numpy(), l + r)
    r2 = (np.arange(10) * 4.5).astype(np.float32)
    p2 = S.Program(S.KIND_ZIP, "float func(float x, float y, float add, float add2) { return (x*y)+add+add2; }",
                   ["float"] * 3)
    dr2 = dev(r2)
    p2.launch([dl, dr2, do], n=10, extra=S.pack(S.value(5.25, np.float32), S.value(7.75, np.float32)))
    assert np.array_equal(do.to_numpy(), (l * r2) + np.float32(5.25) + np.float32(7.75))
    # LeftID: output aliases the left input (test/ZipTests.cpp:134-158)
    p3 = S.Program(S.KIND_ZIP, "float func(float x, float y) { return x; }", ["float"] * 3)
    p3.launch([dl, dr2, dl], n=10)
    assert np.array_equal(dl.to_numpy(), l)
    # void zip writing through get_global_id
    p4 = S.Program(S.KIND_ZIP_VOID, "void func(float x, float y, __global float* out)"
                   "{ out[get_global_id(0)] = x*y; }", ["float", "float"])
    p4.launch([dl, dr2], n=10, extra=S.buffer(do))
    assert np.array_equal(do.to_numpy(), l * r2)


def test_zip_large_in_place(scl):
    n = (1 << 22) + 5
    a = np.arange(n, dtype=np.int32)
    b = np.full(n, 3, np.int32)
    p = S.Program(S.KIND_ZIP, "int func(int x, int y){ return x*y; }", ["int"] * 3)
    da, db = dev(a), dev(b)
    p.launch([da, db, da], n=n)
    assert np.array_equal(da.to_numpy(), a * 3)


def test_index_maps(scl):
    k = kat("index_vector_map")
    p = S.Program(S.KIND_MAP_INDEX, "int func(Index i) { return i; }", ["int"])
    out = S.DeviceArray(k["size"], np.int32)
    p.launch([out], n=k["size"])
    assert np.array_equal(out.to_numpy(), np.arange(k["size"], dtype=np.int32))
    pv = S.Program(S.KIND_MAP_INDEX_VOID, "void func(Index i, __global int* out) { out[i] = i; }", [])
    out2 = S.DeviceArray(1024, np.int32)
    pv.launch([], n=1024, extra=S.buffer(out2))
    assert np.array_equal(out2.to_numpy(), np.arange(1024, dtype=np.int32))
    km = kat("index_matrix_map")
    pm = S.Program(S.KIND_MAP_POINT, "int func(IndexPoint i) { return i.y+i.x; }", ["int"])
    om = S.DeviceArray(km["rows"] * km["cols"], np.int32)
    pm.launch([om], rows=km["rows"], cols=km["cols"])
    yy, xx = np.meshgrid(np.arange(km["rows"]), np.arange(km["cols"]), indexing="ij")
    assert np.array_equal(om.to_numpy().reshape(km["rows"], km["cols"]), (yy + xx).astype(np.int32))
    pmv = S.Program(S.KIND_MAP_POINT_VOID,
                    "void func(IndexPoint ip, int_matrix_t out) { set(out, ip.y, ip.x, ip.y+ip.x); }", [])
    o2 = S.DeviceArray(128 * 32, np.int32)
    pmv.launch([], rows=128, cols=32, extra=S.matrix(o2, 32))
    yy, xx = np.meshgrid(np.arange(128), np.arange(32), indexing="ij")
    assert np.array_equal(o2.to_numpy().reshape(128, 32), (yy + xx).astype(np.int32))


# ---- Reduce (test/ReduceTests.cpp) ---------------------------------------------------
def test_reduce_kats(scl):
    assert run_reduce("float func(float x, float y){ return x+y; }", np.arange(100, dtype=np.float32)) == 4950
    assert run_reduce("float func(float x, float y, float a){ return a*(x+y); }",
                      np.arange(100, dtype=np.float32), extra=S.value(1.0, np.float32)) == 4950
    assert run_reduce("int func(int x, int y){ return x+y; }", np.arange(1587, dtype=np.int32)) == 1258491
    assert run_reduce("int func(int x, int y){ return x+y; }", np.ones(100_000_000, np.int32)) == 100_000_000
    p = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
    dout = S.DeviceArray(1, np.float32)
    big = dev(np.ones(8192 + 256, np.float32))
    for n in list(range(1, 256)) + list(range(8192, 8192 + 256)):
        p.launch([big, dout], n=n)
        assert dout.to_numpy()[0] == n, n


def test_reduce_identity_not_used_and_empty(scl):
    x = -np.arange(1, 1000, dtype=np.float32)
    assert run_reduce("float func(float x, float y){ return max(x, y); }", x, identity="0") == -1.0
    p = S.Program(S.KIND_REDUCE, "int func(int x, int y){ return x+y; }", ["int"], identity="17")
    din, dout = dev(np.ones(4, np.int32)), S.DeviceArray(1, np.int32)
    p.launch([din, dout], n=0)
    assert dout.to_numpy()[0] == 17


@pytest.mark.parametrize("n", [1, 31, 257, 8191, 8193, 1_000_003])
def test_reduce_int_bit_exact(scl, orc, n):
    x = orc.mod_i32(n, 3, 2**31 - 1)
    got = run_reduce("int func(int x, int y){ return x+y; }", x)
    assert got == orc.sum_i32(x)


def test_dot_product_fp64_tolerance(scl, orc):
    n = 1 << 24
    x = orc.uniform_f32(n, 0, -1.0, 1.0)
    y = orc.uniform_f32(n, 1, -1.0, 1.0)
    zp = S.Program(S.KIND_ZIP, "float func(float x, float y){ return x*y; }", ["float"] * 3)
    rp = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
    dx, dy, dz, dr = dev(x), dev(y), S.DeviceArray(n, np.float32), S.DeviceArray(1, np.float32)
    zp.launch([dx, dy, dz], n=n)
    rp.launch([dz, dr], n=n)
    got = float(dr.to_numpy()[0])
    ref = orc.dot_f64(x, y)
    assert abs(got - ref) <= 1e-5 * abs(ref), (got, ref)   # tolerance: rel 1e-5 vs FP64


# ---- Scan (test/ScanTests.cpp) ------------------------------------------------------------
def test_scan_kats(scl):
    for n in (1024, 10):
        out = run_scan("int func(int x, int y){ return x+y; }", np.ones(n, np.int32))
        assert np.array_equal(out, np.arange(n, dtype=np.int32))


@pytest.mark.parametrize("n", [1, 7, 4095, 4096, 4097, 16384, 1_000_003, 1 << 24])
@pytest.mark.parametrize("flags", [0, S.SHAPE_INCLUSIVE, S.SHAPE_REVERSE, S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE])
def test_scan_int_bit_exact(scl, orc, n, flags):
    x = orc.mod_i32(n, 11, 1001)
    out = run_scan("int func(int x, int y){ return x+y; }", x, flags=flags)
    xr = x[::-1] if flags & S.SHAPE_REVERSE else x
    ref = orc.scan_incl_i32(xr) if flags & S.SHAPE_INCLUSIVE else orc.scan_excl_i32(xr, 0)
    if flags & S.SHAPE_REVERSE:
        ref = ref[::-1]
    assert np.array_equal(out, ref)


def test_scan_int_overflow_wraps(scl, orc):
    n = 1 << 22
    x = np.full(n, 1000, np.int32)
    out = run_scan("int func(int x, int y){ return x+y; }", x, flags=S.SHAPE_INCLUSIVE)
    assert np.array_equal(out, orc.scan_incl_i32(x))


def test_scan_float_fp64(scl, orc):
    n = (1 << 22) + 77
    x = orc.uniform_f32(n, 2, -1.0, 1.0)
    out = run_scan("float func(float x, float y){ return x+y; }", x, identity="0.0f", flags=S.SHAPE_INCLUSIVE)
    ref = orc.scan_f64(x, inclusive=True)
    err = np.abs(out.astype(np.float64) - ref)
    # tolerance: abs error <= 1e-5 * (1 + running magnitude scale sqrt(i))
    scale = 1.0 + np.sqrt(np.arange(1, n + 1))
    assert (err <= 1e-5 * scale).all(), float((err / scale).max())


def test_scan_tile_size_variant(scl, orc):
    x = orc.mod_i32(100_000, 5, 1001)
    out = run_scan("int func(int x, int y){ return x+y; }", x, tuning=S.Tuning(items=2))
    assert np.array_equal(out, orc.scan_excl_i32(x, 0))


def test_scan_bounded_wait_returns(scl, orc):
    """With a spin limit of one poll the look-back may give up; the launch
    must still terminate and report either success or SCL_ERR_TIMEOUT."""
    x = orc.mod_i32(1 << 22, 5, 1001)
    p = S.Program(S.KIND_SCAN, "int func(int x, int y){ return x+y; }", ["int"], identity="0")
    din, dout = dev(x), S.DeviceArray(x.size, np.int32)
    p.launch([din, dout], n=x.size, tuning=S.Tuning(spin_limit=1))
    st = S.lib().scl_sync()
    assert st in (S.OK, S.ERR_TIMEOUT)
    S.sync()  # the status word was cleared; the context is still usable
    p.launch([din, dout], n=x.size)
    assert np.array_equal(dout.to_numpy(), orc.scan_excl_i32(x, 0))


def test_debug_bounded_wait(scl):
    st = ctypes.c_int(-1)
    S.check(S.lib().scl_debug_bounded_wait(1000, ctypes.byref(st)))
    assert st.value == S.ERR_TIMEOUT


# ---- MapOverlap (test/MapOverlapTests.cpp) ------------------------------------------------
@pytest.mark.parametrize("variant", [S.VARIANT_AUTO, S.VARIANT_LDST])
@pytest.mark.parametrize("cid", [k["id"] for k in KATS if k.get("skeleton") == "mapoverlap"])
def test_mapoverlap_shift_kats(scl, cid, variant):
    k = kat(cid)
    n, R = k["size"], k["range"]
    i = np.arange(n)[:, None].astype(np.int64)
    j = np.arange(n)[None, :].astype(np.int64)
    fill = {"i*j+i": i * j + i, "j": j + 0 * i, "i": i + 0 * j}[k["fill"]].astype(np.int32)
    src = f"int func(input_matrix_t f){{ return getData(f, {k['dx']}, {k['dy']}); }}"
    p = S.Program(S.KIND_MAPOVERLAP, src, ["int", "int"], overlap_range=R, padding=S.PAD_NEAREST)
    din, dout = dev(fill), S.DeviceArray(n * n, np.int32)
    p.launch([din, dout], rows=n, cols=n, tuning=S.Tuning(variant=variant))
    ys = np.clip(np.arange(n) + k["dy"], 0, n - 1)
    xs = np.clip(np.arange(n) + k["dx"], 0, n - 1)
    assert np.array_equal(dout.to_numpy().reshape(n, n), fill[ys][:, xs])
    if variant == S.VARIANT_LDST:
        assert p.last_variant == S.VARIANT_LDST


GAUSS_SRC = ("float func(input_matrix_t img, __global float* w) { float s = 0.0f;"
             " for (int dy = -5; dy <= 5; ++dy) for (int dx = -5; dx <= 5; ++dx)"
             "  s += getData(img, dx, dy) * w[(dy + 5) * 11 + (dx + 5)]; return s; }")


@pytest.mark.parametrize("shape", [(512, 512), (333, 777), (8, 1000), (1000, 3)])
@pytest.mark.parametrize("padding", [S.PAD_NEUTRAL, S.PAD_NEAREST])
@pytest.mark.parametrize("variant", [S.VARIANT_AUTO, S.VARIANT_LDST])
def test_mapoverlap_gauss_fp64(scl, orc, shape, padding, variant):
    rows, cols = shape
    img = orc.uniform_f32(rows * cols, 5, 0.0, 255.0).reshape(rows, cols)
    w = orc.gaussian_weights(5, 2.0)
    p = S.Program(S.KIND_MAPOVERLAP, GAUSS_SRC, ["float", "float"], overlap_range=5, padding=padding,
                  neutral="0")
    din, dout, dw = dev(img), S.DeviceArray(rows * cols, np.float32), dev(w)
    p.launch([din, dout], rows=rows, cols=cols, extra=S.buffer(dw), tuning=S.Tuning(variant=variant))
    ref = orc.stencil_f64(img, 5, w, padding, 0.0)
    got = dout.to_numpy().reshape(rows, cols).astype(np.float64)
    # tolerance: 121 FP32 FMAs of values <= 255 with weights summing to 1
    assert np.abs(got - ref).max() <= 2e-4, np.abs(got - ref).max()


@pytest.mark.parametrize("cols_flag,py", [(S.PROG_STENCIL_COLS1, 8), (S.PROG_STENCIL_COLS2, 8),
                                          (S.PROG_STENCIL_COLS2, 4), (0, 4), (0, 8)])
@pytest.mark.parametrize("padding", [S.PAD_NEUTRAL, S.PAD_NEAREST])
@pytest.mark.parametrize("variant", [S.VARIANT_TMA, S.VARIANT_LDST])
def test_mapoverlap_thread_shapes_exact(scl, cols_flag, py, padding, variant):
    """One, two or four output columns per thread (default four) and 4 or 8
    rows: an asymmetric integer stencil is exact against numpy, on a ragged
    300 x 520 matrix."""
    rows, cols, R = 300, 520, 4
    img = (np.arange(rows * cols, dtype=np.int64) * 7919 % 1000).astype(np.int32).reshape(rows, cols)
    src = ("int func(input_matrix_t m){ return 3 * getData(m, -3, 2) + getData(m, 4, -1)"
           " - getData(m, 0, -4); }")
    p = S.Program(S.KIND_MAPOVERLAP, src, ["int", "int"], overlap_range=R, padding=padding,
                  neutral="-5", flags=cols_flag)
    din, dout = dev(img), S.DeviceArray(rows * cols, np.int32)
    p.launch([din, dout], rows=rows, cols=cols, tuning=S.Tuning(variant=variant, tile_h=py))
    assert p.last_variant == variant
    if padding == S.PAD_NEAREST:
        def at(dx, dy):
            ys = np.clip(np.arange(rows) + dy, 0, rows - 1)
            xs = np.clip(np.arange(cols) + dx, 0, cols - 1)
            return img[ys][:, xs]
    else:
        pad = np.pad(img, R, constant_values=-5)

        def at(dx, dy):
            return pad[R + dy:R + dy + rows, R + dx:R + dx + cols]
    ref = 3 * at(-3, 2) + at(4, -1) - at(0, -4)
    assert np.array_equal(dout.to_numpy().reshape(rows, cols), ref)


def test_mapoverlap_neutral_nonzero(scl, orc):
    rows, cols = 64, 96
    img = orc.uniform_f32(rows * cols, 9, 0.0, 1.0).reshape(rows, cols)
    src = "float func(input_matrix_t m){ return getData(m, -2, -2) + getData(m, 2, 1); }"
    p = S.Program(S.KIND_MAPOVERLAP, src, ["float", "float"], overlap_range=2, padding=S.PAD_NEUTRAL,
                  neutral="7.5f")
    din, dout = dev(img), S.DeviceArray(rows * cols, np.float32)
    p.launch([din, dout], rows=rows, cols=cols)
    pad = np.pad(img, 2, constant_values=7.5)
    ref = pad[0:rows, 0:cols] + pad[3:rows + 3, 4:cols + 4]
    assert np.array_equal(dout.to_numpy().reshape(rows, cols), ref)


# ---- AllPairs (test/AllPairsTests.cpp) ---------------------------------------------------------
def glibc_matrix(n, mod, libc):
    return np.array([libc.rand() % mod for _ in range(n)], dtype=np.float32)


@pytest.mark.parametrize("variant", [S.VARIANT_AUTO, S.VARIANT_SIMT])
def test_allpairs_kats(scl, orc, variant):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    p = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                  source2="float func(float x, float y){ return x*y; }", identity="0")
    for cid in ("allpairs_matmul_64x64x64", "allpairs_matmul_32x128x32", "allpairs_matmul_100x60x11"):
        k = kat(cid)
        h, d, w = k["height"], k["dim"], k["width"]
        A = glibc_matrix(h * d, 100, libc).reshape(h, d)
        B = glibc_matrix(d * w, 101, libc).reshape(d, w)
        dA, dB, dP = dev(A), dev(B), S.DeviceArray(h * w, np.float32)
        p.launch([dA, dB, dP], rows=h, cols=w, dim=d, tuning=S.Tuning(variant=variant))
        exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float32)
        assert np.array_equal(dP.to_numpy().reshape(h, w), exact), cid


def test_allpairs_extra_args_reduce_first(scl):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    A = glibc_matrix(4096, 100, libc).reshape(64, 64)
    B = glibc_matrix(4096, 101, libc).reshape(64, 64)
    p = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y, float b){ return x+y+b; }", ["float"] * 3,
                  source2="float func(float x, float y, float a){ return x*y+a; }", identity="0")
    dA, dB, dP = dev(A), dev(B), S.DeviceArray(4096, np.float32)
    p.launch([dA, dB, dP], rows=64, cols=64, dim=64,
             extra=S.pack(S.value(6.0, np.float32), S.value(5.0, np.float32)))  # b then a
    ref = np.zeros((64, 64), np.float32)
    for k in range(64):
        ref = ref + (A[:, k:k + 1] * B[k:k + 1, :] + np.float32(5.0)) + np.float32(6.0)
    assert np.array_equal(dP.to_numpy().reshape(64, 64), ref)


def test_allpairs_generic_kats(scl):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    src = ("float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim) {"
           "float res = 0; for (int i = 0; i < dim; ++i) {"
           "  res += getElementFromRow(row, i) * getElementFromColumn(col, i); } return res; }")
    p = S.Program(S.KIND_ALLPAIRS_GENERIC, src, ["float"] * 3)
    A = glibc_matrix(100 * 55, 99, libc).reshape(100, 55)
    B = glibc_matrix(55 * 23, 101, libc).reshape(55, 23)
    dA, dB, dP = dev(A), dev(B), S.DeviceArray(100 * 23, np.float32)
    p.launch([dA, dB, dP], rows=100, cols=23, dim=55)
    assert np.array_equal(dP.to_numpy().reshape(100, 23), (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float32))
    src2 = ("float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim, int start) {"
            "float res = start; for (int i = 0; i < dim; ++i) {"
            "  res += getElementFromRow(row, i) * getElementFromColumn(col, i); } return res; }")
    p2 = S.Program(S.KIND_ALLPAIRS_GENERIC, src2, ["float"] * 3)
    A2 = glibc_matrix(10 * 55, 98, libc).reshape(10, 55)
    B2 = glibc_matrix(55 * 23, 107, libc).reshape(55, 23)
    dA2, dB2, dP2 = dev(A2), dev(B2), S.DeviceArray(10 * 23, np.float32)
    p2.launch([dA2, dB2, dP2], rows=10, cols=23, dim=55, extra=S.value(5, np.int32))
    ref = (A2.astype(np.int64) @ B2.astype(np.int64) + 5).astype(np.float32)
    assert np.array_equal(dP2.to_numpy().reshape(10, 23), ref)


def test_allpairs_fp32_random_vs_fp64(scl, orc):
    M, N, K = 300, 257, 129
    A = orc.normal_f32(M * K, 7).reshape(M, K)
    B = orc.normal_f32(K * N, 8).reshape(K, N)
    p = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                  source2="float func(float x, float y){ return x*y; }", identity="0")
    dA, dB, dP = dev(A), dev(B), S.DeviceArray(M * N, np.float32)
    p.launch([dA, dB, dP], rows=M, cols=N, dim=K, tuning=S.Tuning(variant=S.VARIANT_SIMT))
    ref = orc.gemm_f64(A, B)
    got = dP.to_numpy().reshape(M, N).astype(np.float64)
    rel = np.abs(got - ref).max() / np.abs(ref).max()
    assert rel <= 1e-5, rel   # tolerance: FP32 accumulation over K=129


def test_manhattan_generic_and_special(scl, orc):
    M, N, K = 200, 130, 256
    A = orc.normal_f32(M * K, 10).reshape(M, K)
    B = orc.normal_f32(K * N, 11).reshape(K, N)
    ref = orc.manhattan_f64(A, B)
    gen = S.Program(S.KIND_ALLPAIRS_GENERIC,
                    "float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim) { float s = 0.0f;"
                    " for (unsigned int i = 0; i < dim; ++i) s += fabs(getElementFromRow(row, i) -"
                    " getElementFromColumn(col, i)); return s; }", ["float"] * 3)
    spec = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                     source2="float func(float x, float y){ return fabs(x-y); }", identity="0")
    dA, dB = dev(A), dev(B)
    for p in (gen, spec):
        dP = S.DeviceArray(M * N, np.float32)
        p.launch([dA, dB, dP], rows=M, cols=N, dim=K)
        got = dP.to_numpy().reshape(M, N).astype(np.float64)
        assert (np.abs(got - ref) / ref).max() <= 1e-5   # tolerance: rel 1e-5 vs FP64


# ---- graphs ---------------------------------------------------------------------------------------
def test_graph_capture_dot_product(scl, orc):
    n = 1 << 20
    x = orc.uniform_f32(n, 0, -1.0, 1.0)
    y = orc.uniform_f32(n, 1, -1.0, 1.0)
    zp = S.Program(S.KIND_ZIP, "float func(float x, float y){ return x*y; }", ["float"] * 3)
    rp = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
    dx, dy, dz, dr = dev(x), dev(y), S.DeviceArray(n, np.float32), S.DeviceArray(1, np.float32)
    zp.launch([dx, dy, dz], n=n)
    rp.launch([dz, dr], n=n)  # warm-up sizes the workspaces before capture
    S.sync()
    S.check(S.lib().scl_graph_begin())
    zp.launch([dx, dy, dz], n=n)
    rp.launch([dz, dr], n=n)
    g = ctypes.c_void_p()
    S.check(S.lib().scl_graph_end(ctypes.byref(g)))
    dr.upload(np.zeros(1, np.float32))
    for _ in range(3):
        S.check(S.lib().scl_graph_launch(g))
    got = float(dr.to_numpy()[0])
    ref = orc.dot_f64(x, y)
    assert abs(got - ref) <= 1e-5 * abs(ref)
    S.check(S.lib().scl_graph_destroy(g))


def test_compile_all_builds_every_variant_up_front(scl, orc):
    """SCL_PROG_COMPILE_ALL: the variants otherwise compiled on first use are
    built with the program (no module is loaded by the launches that pick
    them) and give the same results."""
    loads0 = S.debug_counters()["module_loads"]
    n = 100_003
    x = orc.mod_i32(n, 31, 1001)
    rp = S.Program(S.KIND_REDUCE, "int func(int a, int b){ return a + b; }", ["int"], identity="0",
                   flags=S.PROG_COMPILE_ALL)
    dx, dr = dev(x), S.DeviceArray(1, np.int32)
    for items in (1, 2, 4, 8):
        rp.launch([dx, dr], n=n, tuning=S.Tuning(items=items))
        assert int(dr.to_numpy()[0]) == int(x.astype(np.int64).sum()), items
    sp = S.Program(S.KIND_SCAN, "int func(int a, int b){ return a + b; }", ["int"], identity="0",
                   flags=S.PROG_COMPILE_ALL)
    dy = S.DeviceArray(n, np.int32)
    for items, tile_w in ((8, 5), (16, 3), (4, 8)):
        sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, tuning=S.Tuning(items=items, tile_w=tile_w))
        assert np.array_equal(dy.to_numpy(), np.cumsum(x, dtype=np.int64).astype(np.int32)), items
    rows, cols = 200, 256
    img = (np.arange(rows * cols, dtype=np.int64) % 977).astype(np.int32).reshape(rows, cols)
    mo = S.Program(S.KIND_MAPOVERLAP, "int func(input_matrix_t m){ return getData(m, 1, 1) - getData(m, -1, 0); }",
                   ["int", "int"], overlap_range=1, padding=S.PAD_NEAREST, flags=S.PROG_COMPILE_ALL)
    din, dout = dev(img), S.DeviceArray(rows * cols, np.int32)
    ys, xs = np.arange(rows), np.arange(cols)
    ref = img[np.clip(ys + 1, 0, rows - 1)][:, np.clip(xs + 1, 0, cols - 1)] - img[:, np.clip(xs - 1, 0, cols - 1)]
    for variant, py in ((S.VARIANT_TMA, 8), (S.VARIANT_TMA, 16), (S.VARIANT_LDST, 4), (S.VARIANT_LDST, 8)):
        mo.launch([din, dout], rows=rows, cols=cols, tuning=S.Tuning(variant=variant, tile_h=py))
        assert np.array_equal(dout.to_numpy().reshape(rows, cols), ref), (variant, py)
    # one module per program, loaded at construction; none on first use
    assert S.debug_counters()["module_loads"] == loads0 + 3
    # without the flag the same launches load modules as they go
    lazy = S.Program(S.KIND_REDUCE, "int func(int a, int b){ return a + b; }", ["int"], identity="0")
    before = S.debug_counters()["module_loads"]
    lazy.launch([dx, dr], n=n, tuning=S.Tuning(items=1))
    assert S.debug_counters()["module_loads"] == before + 1
