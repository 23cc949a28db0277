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


def run(p, A, B, variant, items=0):
    M, K = A.shape
    _, N = B.shape
    dA, dB = S.DeviceArray.from_numpy(A), S.DeviceArray.from_numpy(B)
    dP = S.DeviceArray(M * N, np.float32)
    p.launch([dA, dB, dP], rows=M, cols=N, dim=K, tuning=S.Tuning(variant=variant, items=items))
    return dP.to_numpy().reshape(M, N)


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
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    A = np.array([libc.rand() % 100 for _ in range(M * K)], np.float32).reshape(M, K)
    B = np.array([libc.rand() % 101 for _ in range(K * N)], np.float32).reshape(K, N)
    p = program()
    P = run(p, A, B, S.VARIANT_TC3XBF16)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float32)
    assert np.array_equal(P, exact)


@pytest.mark.parametrize("items,tol", [(3, 1e-5), (2, 1e-4)])  # tolerance: normwise vs FP64
def test_tc_random_fp64(scl, orc, items, tol):
    M, K, N = 512, 1024, 384
    A = orc.normal_f32(M * K, 7).reshape(M, K)
    B = orc.normal_f32(K * N, 8).reshape(K, N)
    ref = orc.gemm_f64(A, B)
    p = program()
    P = run(p, A, B, S.VARIANT_TC3XBF16, items=items)
    err = normwise(P, ref)
    assert err <= tol, err


def test_tc_scratch_reused_across_shapes(scl, orc):
    p = program()
    for (M, K, N) in [(256, 256, 256), (130, 70, 1000), (256, 256, 256)]:
        A = orc.normal_f32(M * K, M).reshape(M, K)
        B = orc.normal_f32(K * N, N).reshape(K, N)
        assert normwise(run(p, A, B, S.VARIANT_TC3XBF16), orc.gemm_f64(A, B)) <= 1e-5
