"""Scan with non-commutative associative operators: the kernels combine
strictly as f(earlier, later) -- inside a thread, across the warp, across the
tile and along the decoupled look-back between tiles -- so any associative
operator scans correctly, commutative or not.

The reference is only well defined for commutative operators: its up-sweep
and uniform add call f(later, earlier) (include/SkelCL/detail/ScanKernel.cl:135,
243) and its down-sweep f(earlier, later) (:177).  These tests pin the order
the GB300 kernels guarantee, against the oracle's ordered fold
(orc_scan_affine_u32), for each encoding of the cross-tile status:

* uint2 affine maps (8-byte carry: flag word + separate values),
* 16-bit affine maps packed in one uint (4-byte carry: one status word),
* "first non-zero" on float (FP64 carries in one status word).

Sizes span one tile up to a few thousand tiles, so the look-back folds
aggregates over several of its 128-tile windows before it meets an
inclusive prefix."""
import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

AFFINE2 = ("uint2 func(uint2 p, uint2 q){ uint2 r; r.x = q.x * p.x; r.y = q.x * p.y + q.y;"
           " return r; }")
AFFINE2_ID = "inline uint2 affine_id(void){ uint2 r; r.x = 1u; r.y = 0u; return r; }"
# {a, b} in the low / high 16 bits, arithmetic mod 2^16
AFFINE16 = ("uint func(uint p, uint q){ uint pa = p & 0xffffu, pb = p >> 16;"
            " uint qa = q & 0xffffu, qb = q >> 16;"
            " return ((qa * pa) & 0xffffu) | (((qa * pb + qb) & 0xffffu) << 16); }")
FIRST_NZ = "float func(float a, float b){ return a != 0.0f ? a : b; }"

FLAGS = [0, S.SHAPE_INCLUSIVE, S.SHAPE_REVERSE, S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE]
KERNELS = {"staged": None, "register": S.Tuning(variant=S.VARIANT_VECTOR)}


def affine_pairs(n, seed):
    rng = np.random.default_rng(seed)
    # odd multipliers keep the composed maps from collapsing to a = 0
    a = (rng.integers(0, 1 << 31, n, dtype=np.uint64) * 2 + 1).astype(np.uint32)
    b = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    return np.stack([a, b], axis=1)


def flags_of(flags):
    return bool(flags & S.SHAPE_INCLUSIVE), bool(flags & S.SHAPE_REVERSE)


@pytest.mark.parametrize("kernel", list(KERNELS))
@pytest.mark.parametrize("flags", FLAGS)
@pytest.mark.parametrize("n", [1, 7, 4095, 4097, 1_000_003])
def test_affine_uint2_in_order(scl, orc, n, flags, kernel):
    p = S.Program(S.KIND_SCAN, AFFINE2, ["uint2"], identity="affine_id()", common=AFFINE2_ID)
    x = affine_pairs(n, seed=n + flags)
    dx = S.DeviceArray.from_numpy(x.reshape(-1))
    dy = S.DeviceArray(2 * n, np.uint32)
    p.launch([dx, dy], n=n, flags=flags, tuning=KERNELS[kernel])
    want = orc.scan_affine_u32(x, *flags_of(flags))
    got = dy.to_numpy().reshape(-1, 2)
    bad = np.flatnonzero(np.any(got != want, axis=1))
    assert bad.size == 0, (int(bad[0]), got[bad[0]], want[bad[0]])


def pack16(pairs):
    return (pairs[:, 0] & 0xFFFF) | ((pairs[:, 1] & 0xFFFF) << 16)


@pytest.mark.parametrize("kernel", list(KERNELS))
@pytest.mark.parametrize("flags", FLAGS)
@pytest.mark.parametrize("n", [5, 8193, 3_000_017, 1 << 24])
def test_affine_packed_u16_in_order(scl, orc, n, flags, kernel):
    """Composition mod 2^16 is the mod-2^32 composition reduced, so the
    uint32 oracle gives the expected maps."""
    p = S.Program(S.KIND_SCAN, AFFINE16, ["uint"], identity="1u")
    x = affine_pairs(n, seed=7 + n + flags)
    x16 = pack16(x).astype(np.uint32)
    dx = S.DeviceArray.from_numpy(x16)
    dy = S.DeviceArray(n, np.uint32)
    p.launch([dx, dy], n=n, flags=flags, tuning=KERNELS[kernel])
    want = pack16(orc.scan_affine_u32(x, *flags_of(flags))).astype(np.uint32)
    got = dy.to_numpy()
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, (int(bad[0]), hex(got[bad[0]]), hex(want[bad[0]]))


def first_nonzero_ref(x, inclusive, reverse):
    """Ordered fold of f(a, b) = a != 0 ? a : b: the first non-zero element
    seen so far (in scan order)."""
    v = x[::-1] if reverse else x
    n = len(v)
    idx = np.where(v != 0, np.arange(n), n)
    first = np.minimum.accumulate(idx)
    if not inclusive:
        first = np.concatenate([[n], first[:-1]])
    ext = np.concatenate([v, np.zeros(1, v.dtype)])
    out = ext[first]
    return out[::-1] if reverse else out


@pytest.mark.parametrize("flags", FLAGS)
def test_first_nonzero_float_in_order(scl, orc, flags):
    """Zeros everywhere except one run of non-zeros per 1,000,000 elements:
    every tile after the first non-zero must carry that value forward, not a
    later tile's."""
    n = 3 << 20
    rng = np.random.default_rng(11 + flags)
    x = np.zeros(n, np.float32)
    for start in range(200_000, n, 1_000_000):
        x[start:start + 50] = rng.uniform(1.0, 2.0, 50).astype(np.float32)
    p = S.Program(S.KIND_SCAN, FIRST_NZ, ["float"], identity="0.0f")
    dy = S.DeviceArray(n, np.float32)
    p.launch([S.DeviceArray.from_numpy(x), dy], n=n, flags=flags)
    want = first_nonzero_ref(x, *flags_of(flags))
    assert np.array_equal(dy.to_numpy(), want)


@pytest.mark.parametrize("planned", [False, True])
@pytest.mark.parametrize("flags", FLAGS)
def test_segmented_affine_in_order(scl, orc, flags, planned):
    """One ordered scan per segment: short segments (a warp each; with a
    segment plan, a warp each within a window staged in shared memory) and
    long ones (tiles with a look-back that stops at the segment's first
    tile)."""
    rng = np.random.default_rng(5 + flags)
    lens = np.concatenate([rng.integers(0, 300, 2000), rng.integers(5000, 200_000, 20)])
    rng.shuffle(lens)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    n = int(off[-1])
    x = affine_pairs(n, seed=13 + flags)
    x16 = pack16(x).astype(np.uint32)
    p = S.Program(S.KIND_SCAN, AFFINE16, ["uint"], identity="1u")
    dy = S.DeviceArray(n, np.uint32)
    doff = S.DeviceArray.from_numpy(off)
    plan = S.SegPlan(doff, n) if planned else None
    p.launch([S.DeviceArray.from_numpy(x16), dy], n=n, flags=flags,
             segments=plan if planned else doff)
    got = dy.to_numpy()
    if plan is not None:
        plan.release()
    inclusive, reverse = flags_of(flags)
    for s in range(len(lens)):
        lo, hi = int(off[s]), int(off[s + 1])
        if lo == hi:
            continue
        want = pack16(orc.scan_affine_u32(x[lo:hi], inclusive, reverse)).astype(np.uint32)
        assert np.array_equal(got[lo:hi], want), (s, lo, hi)
