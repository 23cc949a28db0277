"""Pin the CPU oracle against the reference's own known answers
(tests/golden/reference_kats.json, extracted from the reference's gtest files
by tests/golden/make_kats.py).  CPU only."""
import ctypes
import json
from pathlib import Path

import numpy as np
import pytest

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def kat(cid):
    return next(k for k in KATS if k["id"] == cid)


def glibc_rand_matrix(n, mod, libc):
    return np.array([libc.rand() % mod for _ in range(n)], dtype=np.float32)


def test_reduce_kats(orc):
    assert orc.sum_f32_reference_order(np.arange(100, dtype=np.float32)) == kat("reduce_float_sum_0_99")["expected"]
    assert orc.sum_i32(np.arange(1587, dtype=np.int32)) == kat("reduce_int_sum_0_1586")["expected"]
    assert orc.sum_i32(np.ones(100_000_000, np.int32)) == kat("reduce_int_1e8_ones")["expected"]
    for cid in ("reduce_float_sizes_1_255", "reduce_float_sizes_8192_8447"):
        lo, hi = kat(cid)["input"]["ones_sizes"]
        for n in range(lo, hi):
            assert orc.sum_f32_reference_order(np.ones(n, np.float32)) == n


def test_scan_kats(orc):
    for cid in ("scan_int_1024_ones", "scan_int_10_ones"):
        n = kat(cid)["input"]["ones"]
        out = orc.scan_excl_i32(np.ones(n, np.int32), 0)
        assert np.array_equal(out, np.arange(n, dtype=np.int32))


def test_scan_wraps_like_int32(orc):
    x = np.full(10, 2**30, np.int32)
    out = orc.scan_incl_i32(x)
    ref = np.cumsum(x.astype(np.int64)).astype(np.uint64).astype(np.uint32).view(np.int32)
    assert np.array_equal(out, ref)
    mt = orc.scan_incl_mod_i32_mt(x, 7919, nthreads=3)
    assert np.array_equal(mt, np.fmod(ref, 7919))


def shift_expect(inp, dx, dy):
    n = inp.shape[0]
    ys = np.clip(np.arange(n) + dy, 0, n - 1)
    xs = np.clip(np.arange(n) + dx, 0, n - 1)
    return inp[ys][:, xs]


@pytest.mark.parametrize("cid", [k["id"] for k in KATS if k.get("skeleton") == "mapoverlap"])
def test_mapoverlap_shift_kats(orc, cid):
    k = kat(cid)
    n, R = k["size"], k["range"]
    i = np.arange(n)[:, None].astype(np.int64)
    j = np.arange(n)[None, :].astype(np.int64)
    fill = {"i*j+i": i * j + i, "j": j + 0 * i, "i": i + 0 * j}[k["fill"]]
    inp = fill.astype(np.float32)  # values < 2^24: exact in float
    w = np.zeros((2 * R + 1, 2 * R + 1), np.float32)
    w[k["dy"] + R, k["dx"] + R] = 1.0
    out = orc.stencil_f64(inp, R, w, padding=1)
    # the reference test's own expectations, restated (test/MapOverlapTests.cpp:187-447)
    exp = shift_expect(inp.astype(np.float64), k["dx"], k["dy"])
    assert np.array_equal(out, exp)


def test_allpairs_kats(orc):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    for cid in ("allpairs_matmul_64x64x64", "allpairs_matmul_32x128x32", "allpairs_matmul_100x60x11"):
        k = kat(cid)
        h, d, w = k["height"], k["dim"], k["width"]
        A = glibc_rand_matrix(h * d, k["left_mod"], libc).reshape(h, d)
        B = glibc_rand_matrix(d * w, k["right_mod"], libc).reshape(d, w)
        P = orc.gemm_f32_seq(A, B)
        exact = A.astype(np.int64) @ B.astype(np.int64)
        assert np.array_equal(P.astype(np.int64), exact)
        assert np.array_equal(orc.gemm_f64(A, B), exact.astype(np.float64))


def test_stencil_adjoint_is_transpose(orc):
    """<S x, g> == <x, S^T g> for both paddings (linear stencil)."""
    rng = np.random.default_rng(0)
    R = 2
    w = rng.standard_normal((2 * R + 1, 2 * R + 1)).astype(np.float32)
    x = rng.standard_normal((13, 9)).astype(np.float32)
    g = rng.standard_normal((13, 9)).astype(np.float32)
    for pad in (0, 1):
        lhs = float((orc.stencil_f64(x, R, w, pad) * g.astype(np.float64)).sum())
        rhs = float((x.astype(np.float64) * orc.stencil_adjoint_f64(g, R, w, pad)).sum())
        assert abs(lhs - rhs) <= 1e-9 * max(1.0, abs(lhs))


def test_generators_are_seeded(orc):
    a = orc.uniform_f32(1000, 0, -1.0, 1.0)
    b = orc.uniform_f32(1000, 0, -1.0, 1.0)
    c = orc.uniform_f32(1000, 1, -1.0, 1.0)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() >= -1.0 and a.max() < 1.0
    m = orc.mod_i32(1000, 0, 1001)
    assert m.min() >= 0 and m.max() <= 1000
    z = orc.normal_f32(100000, 7)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02
