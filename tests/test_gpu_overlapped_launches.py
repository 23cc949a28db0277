"""Overlapped launches: skeleton kernels launched with programmatic stream
serialization wait for their predecessor before touching memory, so chains
of dependent skeletons give the same results with and without it."""
import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

INC = "int func(int x){ return x + 1; }"
ADD = "int func(int x, int y){ return x + y; }"
MOD = "int func(int x){ return x % 7919; }"


def dev(a):
    return S.DeviceArray.from_numpy(np.ascontiguousarray(a))


@pytest.fixture
def pdl_on(scl):
    prev = S.set_overlapped_launches(True)
    yield
    S.set_overlapped_launches(prev)


def test_skeleton_launches_are_overlapped_by_default(scl, pdl_on):
    p = S.Program(S.KIND_MAP, INC, ["int", "int"])
    x = dev(np.zeros(1 << 16, np.int32))
    c0, l0 = S.overlapped_launch_count(), S.launch_count()
    for _ in range(5):
        p.launch([x, x], n=1 << 16)
    assert S.launch_count() - l0 == 5
    assert S.overlapped_launch_count() - c0 == 5
    S.set_overlapped_launches(False)
    p.launch([x, x], n=1 << 16)
    assert S.overlapped_launch_count() - c0 == 5
    assert (x.to_numpy() == 6).all()


def test_in_place_chain_with_reductions(scl, orc, pdl_on):
    """200 in-place increments, each followed by a Reduce of the vector it
    just wrote; any kernel starting before its predecessor finished would
    read stale elements."""
    n = 1 << 20
    x0 = orc.mod_i32(n, 11, 1001)
    inc = S.Program(S.KIND_MAP, INC, ["int", "int"])
    red = S.Program(S.KIND_REDUCE, ADD, ["int"], identity="0")
    x = dev(x0)
    sums = S.DeviceArray(200, np.int32)
    for k in range(200):
        inc.launch([x, x], n=n)
        red.launch([x, sums.view(k, 1)], n=n)
    base = int(x0.astype(np.int64).sum())
    want = np.array([base + (k + 1) * n for k in range(200)], np.int64).astype(np.int32)
    assert np.array_equal(sums.to_numpy(), want)
    assert np.array_equal(x.to_numpy(), x0 + 200)


@pytest.mark.parametrize("overlapped", [True, False])
def test_scan_map_ping_pong_matches_oracle(scl, orc, overlapped):
    """Scan A -> B, Map B -> A, twenty times over 2^22 elements: each kernel
    reads what the previous one wrote (the scan also reuses its status
    regions every call)."""
    prev = S.set_overlapped_launches(overlapped)
    try:
        n = 1 << 22
        x0 = orc.mod_i32(n, 12, 1001)
        scan = S.Program(S.KIND_SCAN, ADD, ["int"], identity="0")
        mod = S.Program(S.KIND_MAP, MOD, ["int", "int"])
        a, b = dev(x0), S.DeviceArray(n, np.int32)
        for _ in range(20):
            scan.launch([a, b], n=n, flags=S.SHAPE_INCLUSIVE)
            mod.launch([b, a], n=n)
        ref = x0.copy()
        for _ in range(20):
            ref = orc.map_mod_i32(orc.scan_incl_i32(ref), 7919)
        assert np.array_equal(a.to_numpy(), ref)
    finally:
        S.set_overlapped_launches(prev)
