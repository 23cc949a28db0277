"""Local (shared-memory) extra arguments in every skeleton: the reference
passes a skelcl::Local as a __local kernel argument of the requested size
(include/SkelCL/detail/KernelUtil.h:201-213, src/Local.cpp:44-57).  Here it is
placed after the skeleton's own dynamic shared memory (the scan tile, the
stencil window), so a user function that writes its slot leaves the
skeleton's data intact."""
import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

SLOTS = S.local(4096)  # 1024 four-byte slots: one per thread of any block


def dev(a):
    return S.DeviceArray.from_numpy(np.ascontiguousarray(a))


@pytest.mark.parametrize("variant", [S.VARIANT_AUTO, S.VARIANT_VECTOR])
def test_scan_with_local(scl, orc, variant):
    n = 3_000_001
    x = orc.mod_i32(n, 3, 1001)
    p = S.Program(S.KIND_SCAN, "int func(int x, int y, __local int* t) {"
                  " t[get_local_id(0)] = x; return x + y; }", ["int"], identity="0")
    dx, dy = dev(x), S.DeviceArray(n, np.int32)
    p.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, extra=SLOTS, tuning=S.Tuning(variant=variant))
    assert np.array_equal(dy.to_numpy(), np.cumsum(x, dtype=np.int64).astype(np.int32))


def test_reduce_with_local(scl, orc):
    n = 1 << 20
    x = orc.mod_i32(n, 4, 100)
    p = S.Program(S.KIND_REDUCE, "int func(int x, int y, __local int* t) {"
                  " t[get_local_id(0)] = y; return x + y; }", ["int"], identity="0")
    dx, dy = dev(x), S.DeviceArray(1, np.int32)
    p.launch([dx, dy], n=n, extra=SLOTS)
    assert int(dy.to_numpy()[0]) == int(x.astype(np.int64).sum())


@pytest.mark.parametrize("variant", [S.VARIANT_TMA, S.VARIANT_LDST])
def test_mapoverlap_with_local(scl, variant):
    rows, cols = 200, 256
    img = (np.arange(rows * cols, dtype=np.int64) % 977).astype(np.int32).reshape(rows, cols)
    src = ("int func(input_matrix_t m, __local int* t) {"
           " t[get_local_id(1) * 32 + get_local_id(0)] = getData(m, 0, 0);"
           " return getData(m, 1, -1) + 2 * getData(m, -2, 2); }")
    p = S.Program(S.KIND_MAPOVERLAP, src, ["int", "int"], overlap_range=2, padding=S.PAD_NEAREST)
    din, dout = dev(img), S.DeviceArray(rows * cols, np.int32)
    p.launch([din, dout], rows=rows, cols=cols, extra=SLOTS, tuning=S.Tuning(variant=variant))
    assert p.last_variant == variant

    def at(dx, dy):
        return img[np.clip(np.arange(rows) + dy, 0, rows - 1)][:, np.clip(np.arange(cols) + dx, 0, cols - 1)]
    assert np.array_equal(dout.to_numpy().reshape(rows, cols), at(1, -1) + 2 * at(-2, 2))


def test_allpairs_with_local(scl):
    M, K, N = 130, 70, 150
    rng = np.random.default_rng(5)
    A = rng.integers(0, 10, (M, K)).astype(np.float32)
    B = rng.integers(0, 10, (K, N)).astype(np.float32)
    p = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y) { return x + y; }", ["float"] * 3,
                  source2="float func(float x, float y, __local float* t) {"
                          " t[get_local_id(0)] = x; return x * y; }", identity="0")
    dA, dB, dP = dev(A), dev(B), S.DeviceArray(M * N, np.float32)
    p.launch([dA, dB, dP], rows=M, cols=N, dim=K, extra=SLOTS)
    assert p.last_variant == S.VARIANT_SIMT
    assert np.array_equal(dP.to_numpy().reshape(M, N), A @ B)
