"""Vectors longer than 2^32 elements: Map, inclusive Scan and Reduce on
2^32 + 17 bytes (about 8.6 GB of device memory), checked at positions either
side of 2^31 and 2^32 against closed forms of a periodic input.  The element
index is 64-bit throughout (the reference's OpenCL kernels use size_t
global ids, include/SkelCL/detail/MapDef.h:187-195)."""
import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

N = (1 << 32) + 17
PERIOD = 251
BASE = ((7 * np.arange(PERIOD) + 3) % PERIOD).astype(np.uint8)  # values 0 .. 250
PICKS = [0, 1, 250, 251, (1 << 31) - 1, 1 << 31, (1 << 31) + 1, (1 << 32) - 1, 1 << 32,
         (1 << 32) + 1, N - 2, N - 1]


@pytest.fixture(scope="module")
def big(scl):
    x = np.tile(BASE, N // PERIOD + 1)[:N]
    x[-1] = 255  # the only 255: the maximum sits in the last element
    d = S.DeviceArray.from_numpy(x)
    yield x, d
    d.free()


def at(d, i):
    return int(d.view(i, 1).to_numpy()[0])


def test_map_beyond_4g(scl, big):
    x, dx = big
    p = S.Program(S.KIND_MAP, "uchar func(uchar v) { return v + 1; }", ["unsigned char", "unsigned char"])
    dy = S.DeviceArray(N, np.uint8)
    p.launch([dx, dy], n=N)
    for i in PICKS:
        assert at(dy, i) == (int(x[i]) + 1) % 256, i
    dy.free()


def test_inclusive_scan_beyond_4g(scl, big):
    x, dx = big
    p = S.Program(S.KIND_SCAN, "uchar func(uchar a, uchar b) { return a + b; }", ["unsigned char"], identity="0")
    dy = S.DeviceArray(N, np.uint8)
    p.launch([dx, dy], n=N, flags=S.SHAPE_INCLUSIVE)
    period_sum = int(BASE.astype(np.int64).sum())
    partial = np.concatenate([[0], np.cumsum(BASE.astype(np.int64))])

    def prefix(i):  # sum of x[0..i] mod 256 (x[N-1] was changed to 255)
        k = i + 1
        s = (k // PERIOD) * period_sum + int(partial[k % PERIOD])
        if i == N - 1:
            s += 255 - int(BASE[(N - 1) % PERIOD])
        return s % 256
    for i in PICKS:
        assert at(dy, i) == prefix(i), i
    dy.free()


def test_reduce_beyond_4g(scl, big):
    _, dx = big
    p = S.Program(S.KIND_REDUCE, "uchar func(uchar a, uchar b) { return a > b ? a : b; }", ["unsigned char"],
                  identity="0")
    dr = S.DeviceArray(1, np.uint8)
    p.launch([dx, dr], n=N)
    assert at(dr, 0) == 255
    p.launch([dx, dr], n=N - 1)  # without the last element the maximum is 250
    assert at(dr, 0) == 250


@pytest.mark.parametrize("variant", [S.VARIANT_TC3XBF16, S.VARIANT_SIMT])
def test_allpairs_output_beyond_4g(scl, orc, variant):
    """P of 65536 x 65536 floats (17 GB): rows past 2^32 / N elements."""
    M = Nn = 1 << 16
    K = 64
    A = orc.normal_f32(M * K, 3).reshape(M, K)
    B = orc.normal_f32(K * Nn, 4).reshape(K, Nn)
    p = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                  source2="float func(float x, float y){ return x*y; }", identity="0")
    dA, dB, dP = S.DeviceArray.from_numpy(A), S.DeviceArray.from_numpy(B), S.DeviceArray(M * Nn, np.float32)
    p.launch([dA, dB, dP], rows=M, cols=Nn, dim=K, tuning=S.Tuning(variant=variant))
    assert p.last_variant == variant
    rows = [0, 1, (1 << 15) - 1, 1 << 15, M - 2, M - 1]
    ref = orc.gemm_f64(np.ascontiguousarray(A[rows]), B)
    got = np.stack([dP.view(r * Nn, Nn).to_numpy() for r in rows]).astype(np.float64)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    dP.free()


@pytest.mark.parametrize("variant", [S.VARIANT_TMA, S.VARIANT_LDST])
def test_mapoverlap_beyond_4g(scl, variant):
    """A 65600 x 65536 byte image: outputs past element 2^32, NEAREST edges."""
    rows, cols = 65600, 1 << 16
    period = 509
    img = np.tile(((13 * np.arange(period) + 5) % 256).astype(np.uint8), rows * cols // period + 1)
    img = img[:rows * cols].reshape(rows, cols)
    src = "uchar func(input_matrix_t m){ return getData(m, -1, 0) + 2 * getData(m, 1, 1); }"
    p = S.Program(S.KIND_MAPOVERLAP, src, ["unsigned char", "unsigned char"], overlap_range=1,
                  padding=S.PAD_NEAREST)
    din, dout = S.DeviceArray.from_numpy(img), S.DeviceArray(rows * cols, np.uint8)
    p.launch([din, dout], rows=rows, cols=cols, tuning=S.Tuning(variant=variant))
    assert p.last_variant == variant
    for y in [0, 1, 32767, 32768, 65535, 65536, rows - 2, rows - 1]:
        got = dout.view(y * cols, cols).to_numpy()
        left = img[y, np.clip(np.arange(cols) - 1, 0, cols - 1)].astype(np.int64)
        below = img[min(y + 1, rows - 1), np.clip(np.arange(cols) + 1, 0, cols - 1)].astype(np.int64)
        assert np.array_equal(got, ((left + 2 * below) % 256).astype(np.uint8)), y
    din.free()
    dout.free()
