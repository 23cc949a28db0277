"""AllPairs zip(x*y)/reduce(x+y) on the tcgen05 tensor cores (3xBF16 split,
FP32 accumulation in tensor memory) against the FP64 oracle, the CUDA-core
kernel and the reference's integer-valued known answers."""
import ctypes

import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

ZIP = "float func(float x, float y){ return x*y; }"
RED = "float func(float x, float y){ return x+y; }"


def program():
    return S.Program(S.KIND_ALLPAIRS, RED, ["float"] * 3, source2=ZIP, identity="0")


def run(p, A, B, variant, items=0, cols=0):
    """cols: tensor-core output-tile columns, 128 or 256; 0 = automatic (256
    when the 128 x 256 tiles still give every SM one)."""
    M, K = A.shape
    _, N = B.shape
    dA, dB = S.DeviceArray.from_numpy(A), S.DeviceArray.from_numpy(B)
    dP = S.DeviceArray(M * N, np.float32)
    p.launch([dA, dB, dP], rows=M, cols=N, dim=K,
             tuning=S.Tuning(variant=variant, items=items, tile_h=cols))
    return dP.to_numpy().reshape(M, N)


def rand_ints(M, K, N, seed=1):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(seed)
    A = np.array([libc.rand() % 100 for _ in range(M * K)], np.float32).reshape(M, K)
    B = np.array([libc.rand() % 101 for _ in range(K * N)], np.float32).reshape(K, N)
    return A, B


def normwise(P, ref):
    return float(np.abs(P.astype(np.float64) - ref).max() / np.abs(ref).max())


def test_tc_path_is_selected(scl):
    p = program()
    A = np.ones((128, 64), np.float32)
    B = np.ones((64, 128), np.float32)
    P = run(p, A, B, S.VARIANT_AUTO)
    assert p.last_variant == S.VARIANT_TC3XBF16
    assert np.array_equal(P, np.full((128, 128), 64.0, np.float32))


@pytest.mark.parametrize("shape", [(128, 64, 128), (256, 192, 384), (300, 129, 257), (1000, 520, 130)])
def test_tc_integer_inputs_exact(scl, shape):
    """Integer-valued inputs (the reference's AllPairs tests use rand() % 100):
    every product and partial sum is exact in FP32, so the result is exact."""
    M, K, N = shape
    A, B = rand_ints(M, K, N)
    p = program()
    P = run(p, A, B, S.VARIANT_TC3XBF16, cols=128)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float32)
    assert np.array_equal(P, exact)


@pytest.mark.parametrize("shape", [(128, 64, 256), (256, 96, 384), (300, 129, 257), (1000, 520, 130),
                                   (130, 32, 600)])
def test_tc_wide_tile_integer_inputs_exact(scl, shape):
    """128 x 256 output tiles (k-blocks of 32, SWIZZLE_64B): the same exact
    integer results, also for N below, at and past a multiple of 256."""
    M, K, N = shape
    A, B = rand_ints(M, K, N, seed=2)
    p = program()
    P = run(p, A, B, S.VARIANT_TC3XBF16, cols=256)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float32)
    assert np.array_equal(P, exact)


@pytest.mark.parametrize("items,tol", [(3, 1e-5), (2, 1e-4)])  # tolerance: normwise vs FP64
def test_tc_wide_tile_random_fp64(scl, orc, items, tol):
    M, K, N = 512, 1000, 768
    A = orc.normal_f32(M * K, 17).reshape(M, K)
    B = orc.normal_f32(K * N, 18).reshape(K, N)
    P = run(program(), A, B, S.VARIANT_TC3XBF16, items=items, cols=256)
    assert normwise(P, orc.gemm_f64(A, B)) <= tol


@pytest.mark.parametrize("cols", [128, 256])
def test_tc_transposed_operands(scl, orc, cols):
    """SHAPE_TRANS_LEFT (A stored K x M) and SHAPE_TRANS_RIGHT (B stored N x K)
    give A @ B as the row-major call does."""
    M, K, N = 384, 200, 520
    A = orc.normal_f32(M * K, 21).reshape(M, K)
    B = orc.normal_f32(K * N, 22).reshape(K, N)
    ref = orc.gemm_f64(A, B)
    p = program()
    t = S.Tuning(variant=S.VARIANT_TC3XBF16, tile_h=cols)
    for flags, a, b in [(S.SHAPE_TRANS_LEFT, A.T, B), (S.SHAPE_TRANS_RIGHT, A, B.T),
                        (S.SHAPE_TRANS_LEFT | S.SHAPE_TRANS_RIGHT, A.T, B.T)]:
        dA = S.DeviceArray.from_numpy(np.ascontiguousarray(a))
        dB = S.DeviceArray.from_numpy(np.ascontiguousarray(b))
        dP = S.DeviceArray(M * N, np.float32)
        p.launch([dA, dB, dP], rows=M, cols=N, dim=K, flags=flags, tuning=t)
        assert normwise(dP.to_numpy().reshape(M, N), ref) <= 1e-5, flags


@pytest.mark.parametrize("items,tol", [(3, 1e-5), (2, 1e-4)])  # tolerance: normwise vs FP64
def test_tc_random_fp64(scl, orc, items, tol):
    M, K, N = 512, 1024, 384
    A = orc.normal_f32(M * K, 7).reshape(M, K)
    B = orc.normal_f32(K * N, 8).reshape(K, N)
    ref = orc.gemm_f64(A, B)
    p = program()
    P = run(p, A, B, S.VARIANT_TC3XBF16, items=items, cols=128)
    err = normwise(P, ref)
    assert err <= tol, err


def test_tc_scratch_reused_across_shapes(scl, orc):
    p = program()
    for (M, K, N), cols in [((256, 256, 256), 128), ((130, 70, 1000), 256), ((256, 256, 256), 256),
                            ((130, 70, 1000), 128)]:
        A = orc.normal_f32(M * K, M).reshape(M, K)
        B = orc.normal_f32(K * N, N).reshape(K, N)
        assert normwise(run(p, A, B, S.VARIANT_TC3XBF16, cols=cols), orc.gemm_f64(A, B)) <= 1e-5


def test_tc_automatic_tile_width(scl, orc):
    """Without a tile width the launch takes 128 x 256 tiles once they give
    every SM one (here 20 x 8 = 160 tiles): the result is the explicit
    256-column launch's, bit for bit."""
    M, K, N = 2560, 96, 2048
    A = orc.normal_f32(M * K, 31).reshape(M, K)
    B = orc.normal_f32(K * N, 32).reshape(K, N)
    p = program()
    auto = run(p, A, B, S.VARIANT_AUTO)
    assert p.last_variant == S.VARIANT_TC3XBF16
    assert np.array_equal(auto, run(p, A, B, S.VARIANT_TC3XBF16, cols=256))
    assert normwise(auto, orc.gemm_f64(A, B)) <= 1e-5
