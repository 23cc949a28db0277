"""Segmented launches: thousands of uneven-length vectors stored back to back,
one Scan / Reduce launch for all of them, against per-segment references
(bit-exact for integers, FP64 oracle tolerances for floats)."""
import ctypes

import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

IADD = "int func(int x, int y){ return x + y; }"
FADD = "float func(float x, float y){ return x + y; }"


def dev(a):
    return S.DeviceArray.from_numpy(np.ascontiguousarray(a))


def log_uniform_offsets(n_seg, lo, hi, seed, zeros=0):
    rng = np.random.default_rng(seed)
    lens = np.floor(2.0 ** rng.uniform(lo, hi, n_seg)).astype(np.uint64)
    if zeros:
        lens[rng.choice(n_seg, zeros, replace=False)] = 0
    return np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)


def seg_ids(off, n):
    return np.searchsorted(off[1:], np.arange(n), side="right")


def seg_scan_ref(x, off, flags):
    """Per-segment scans of int32 x with wrap-around, all four flag forms."""
    n = len(x)
    x64 = x.astype(np.int64)
    ids = seg_ids(off, n)
    cs = np.cumsum(x64)
    before = np.concatenate([[0], cs])[off[:-1].astype(np.int64)]  # sum before each segment
    incl = cs - before[ids]
    total = (np.concatenate([[0], cs])[off[1:].astype(np.int64)] - before)[ids]
    if flags & 2:  # reverse: sum over [i, end of segment]
        incl = total - incl + x64
    res = incl if flags & 1 else incl - x64
    return res.astype(np.int32)  # two's-complement wrap, as the int kernel


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_segmented_scan_int_exact(scl, orc, flags):
    off = log_uniform_offsets(3000, 0, 16, seed=1, zeros=50)  # 1 .. 65536 elements, some empty
    n = int(off[-1])
    x = orc.mod_i32(n, 2, 1001) - 500
    p = S.Program(S.KIND_SCAN, IADD, ["int"], identity="0")
    dy = S.DeviceArray(n, np.int32)
    p.launch([dev(x), dy], n=n, flags=flags, segments=dev(off))
    assert np.array_equal(dy.to_numpy(), seg_scan_ref(x, off, flags))


def mixed_offsets(seed):
    """Mostly short vectors (a warp each), some across and past the 4096-element
    boundary (tiles), some empty, and the boundary lengths themselves."""
    rng = np.random.default_rng(seed)
    short = rng.integers(0, 300, 20_000)
    mid = rng.integers(300, 6000, 1_500)
    long = rng.integers(6000, 40_000, 60)
    edge = np.array([0, 1, 31, 32, 33, 255, 256, 257, 4095, 4096, 4097, 8192, 8193, 0, 0])
    lens = np.concatenate([short, mid, long, edge])
    rng.shuffle(lens)
    return np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_segmented_scan_mixed_lengths_exact(scl, orc, flags):
    off = mixed_offsets(21)
    n = int(off[-1])
    x = orc.mod_i32(n, 22, 1001) - 500
    p = S.Program(S.KIND_SCAN, IADD, ["int"], identity="0")
    dx, dy, doff = dev(x), S.DeviceArray(n, np.int32), dev(off)
    p.launch([dx, dy], n=n, flags=flags, segments=doff)
    assert np.array_equal(dy.to_numpy(), seg_scan_ref(x, off, flags))


def test_segmented_reduce_mixed_lengths_exact(scl, orc):
    off = mixed_offsets(23)
    n = int(off[-1])
    x = orc.mod_i32(n, 24, 1001) - 500
    p = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="0")
    dout, doff = S.DeviceArray(len(off) - 1, np.int32), dev(off)
    p.launch([dev(x), dout], n=n, segments=doff)
    ref = np.bincount(seg_ids(off, n), weights=x.astype(np.float64), minlength=len(off) - 1)
    assert np.array_equal(dout.to_numpy().astype(np.int64), ref.astype(np.int64))


def test_segmented_with_extra_arguments(scl, orc):
    """A scalar and a Local extra argument reach both the warp-per-vector and
    the tiled kernels of a segmented Scan and Reduce."""
    off = mixed_offsets(25)
    n = int(off[-1])
    x = orc.mod_i32(n, 26, 1001) - 500
    src = ("int func(int a, int b, int scale, __local int* t) {"
           " t[get_local_id(0)] = a; return a + b * scale; }")
    sp = S.Program(S.KIND_SCAN, src, ["int"], identity="0")
    rp = S.Program(S.KIND_REDUCE, src, ["int"], identity="0")
    extra = S.value(1, np.int32) + S.local(4096)
    dx, doff = dev(x), dev(off)
    dy, dr = S.DeviceArray(n, np.int32), S.DeviceArray(len(off) - 1, np.int32)
    sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, segments=doff, extra=extra)
    assert np.array_equal(dy.to_numpy(), seg_scan_ref(x, off, 1))
    rp.launch([dx, dr], n=n, segments=doff, extra=extra)
    ref = np.bincount(seg_ids(off, n), weights=x.astype(np.float64), minlength=len(off) - 1)
    assert np.array_equal(dr.to_numpy().astype(np.int64), ref.astype(np.int64))


def test_segmented_reduce_all_empty(scl):
    """Every vector empty, the flat buffer too: one identity per vector."""
    p = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="7")
    dout = S.DeviceArray(5, np.int32)
    dx = S.DeviceArray(1, np.int32)  # a valid pointer; no element is read
    p.launch([dx, dout], n=0, segments=dev(np.zeros(6, np.uint64)))
    assert list(dout.to_numpy()) == [7] * 5
    p.launch([dx, dout], n=1, segments=dev(np.array([0, 0, 0, 0, 0, 1], np.uint64)))
    got = dout.to_numpy()
    assert list(got[:4]) == [7] * 4


def test_segmented_scan_single_segment_equals_plain(scl, orc):
    n = 5_000_003
    x = orc.mod_i32(n, 3, 1001)
    p = S.Program(S.KIND_SCAN, IADD, ["int"], identity="0")
    d1, d2 = S.DeviceArray(n, np.int32), S.DeviceArray(n, np.int32)
    dx = dev(x)
    p.launch([dx, d1], n=n, flags=S.SHAPE_INCLUSIVE, segments=dev(np.array([0, n], np.uint64)))
    p.launch([dx, d2], n=n, flags=S.SHAPE_INCLUSIVE)
    assert np.array_equal(d1.to_numpy(), d2.to_numpy())


def test_segmented_scan_float(scl, orc):
    off = log_uniform_offsets(2000, 6, 17, seed=4)
    n = int(off[-1])
    x = orc.uniform_f32(n, 5, -1.0, 1.0)
    p = S.Program(S.KIND_SCAN, FADD, ["float"], identity="0")
    dy = S.DeviceArray(n, np.float32)
    p.launch([dev(x), dy], n=n, flags=S.SHAPE_INCLUSIVE, segments=dev(off))
    ids = seg_ids(off, n)
    cs = np.cumsum(x.astype(np.float64))
    ref = cs - np.concatenate([[0.0], cs])[off[:-1].astype(np.int64)][ids]
    pos = np.arange(n) - off[:-1].astype(np.int64)[ids] + 1  # terms summed
    assert np.all(np.abs(dy.to_numpy() - ref) <= 1e-5 * (1.0 + np.sqrt(pos)))


@pytest.mark.parametrize("dtype,src,types", [(np.int32, IADD, ["int"]), (np.float32, FADD, ["float"])])
def test_segmented_reduce(scl, orc, dtype, src, types):
    off = log_uniform_offsets(5000, 0, 17, seed=6, zeros=100)
    n = int(off[-1])
    x = (orc.mod_i32(n, 7, 1001) - 500).astype(dtype) if dtype == np.int32 else orc.uniform_f32(n, 7, -1.0, 1.0)
    p = S.Program(S.KIND_REDUCE, src, types, identity="0")
    dout = S.DeviceArray(len(off) - 1, dtype)
    p.launch([dev(x), dout], n=n, segments=dev(off))
    cs = np.concatenate([[0], np.cumsum(x.astype(np.int64 if dtype == np.int32 else np.float64))])
    ref = cs[off[1:].astype(np.int64)] - cs[off[:-1].astype(np.int64)]
    got = dout.to_numpy()
    if dtype == np.int32:
        assert np.array_equal(got, ref.astype(np.int32))
    else:
        lens = (off[1:] - off[:-1]).astype(np.float64)
        assert np.all(np.abs(got - ref) <= 1e-6 * (1.0 + np.sqrt(lens)))
    # a second launch on the same workspace (tickets were reset)
    p.launch([dev(x), dout], n=n, segments=dev(off))
    assert np.array_equal(dout.to_numpy(), got)


def test_segmented_reduce_unaligned_and_empty(scl, orc):
    off = np.array([0, 0, 1, 5, 5, 8200, 8201, 30001, 30001], np.uint64)
    n = 30001
    x = orc.mod_i32(n + 1, 8, 1001)
    p = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="0")
    dout = S.DeviceArray(len(off) - 1, np.int32)
    dx = dev(x).view(1, n)  # unaligned base
    p.launch([dx, dout], n=n, segments=dev(off))
    xs = x[1:].astype(np.int64)
    ref = [int(xs[int(a):int(b)].sum()) for a, b in zip(off[:-1], off[1:])]
    assert list(dout.to_numpy()) == ref


def test_bad_offsets_are_clamped_and_reported(scl, orc):
    n = 1000
    x = orc.mod_i32(n, 9, 1001)
    p = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="0")
    dout = S.DeviceArray(3, np.int32)
    bad = np.array([0, 600, 300, 5000], np.uint64)  # decreasing, and past the end
    p.launch([dev(x), dout], n=n, segments=dev(bad))
    assert S.lib().scl_sync() == S.ERR_ARG
    S.sync()  # status cleared, context usable
    good = np.array([0, 600, 600, 1000], np.uint64)
    p.launch([dev(x), dout], n=n, segments=dev(good))
    xs = x.astype(np.int64)
    assert list(dout.to_numpy()) == [int(xs[:600].sum()), 0, int(xs[600:].sum())]


@pytest.mark.parametrize("dtype,code", [(np.float32, S.DTYPE_F32), (np.float64, S.DTYPE_F64)])
def test_segmented_broadcast(scl, dtype, code):
    off = log_uniform_offsets(777, 0, 14, seed=10, zeros=20)
    n = int(off[-1])
    g = np.arange(1, len(off), dtype=dtype)
    gx = dev(np.full(n, 0.5, dtype))
    dg, doff = dev(g), dev(off)  # keep the allocations alive across the launch
    S.check(S.lib().scl_adjoint_broadcast_segments(dg.ptr, gx.ptr, doff.ptr, len(off) - 1, n, code, 1))
    ids = seg_ids(off, n)
    assert np.array_equal(gx.to_numpy(), (g[ids] + dtype(0.5)).astype(dtype))


@pytest.mark.parametrize("shift", [1, 3])
@pytest.mark.parametrize("accumulate", [0, 1])
def test_segmented_broadcast_unaligned_and_short(scl, shift, accumulate):
    """The broadcast on a gx that does not start on 16 bytes (element-wise
    stores), over many short vectors, empty ones, vectors that start before
    or reach past a warp's 1024-element chunk, and elements before the first
    vector and after the last (left alone)."""
    rng = np.random.default_rng(20 + shift)
    lens = np.concatenate([rng.integers(0, 40, 5000), [0, 1, 1023, 1024, 1025, 5000, 0]])
    rng.shuffle(lens)
    lead, tail = 37, 11
    off = (lead + np.concatenate([[0], np.cumsum(lens)])).astype(np.uint64)
    n = int(off[-1]) + tail
    g = rng.uniform(-1, 1, len(lens)).astype(np.float32)
    base = rng.uniform(-1, 1, n + shift).astype(np.float32)
    dbase, dg, doff = dev(base), dev(g), dev(off)
    gx = dbase.view(shift, n)
    S.check(S.lib().scl_adjoint_broadcast_segments(dg.ptr, gx.ptr, doff.ptr, len(lens), n, S.DTYPE_F32,
                                                   accumulate))
    want = base[shift:].copy()
    ids = np.repeat(np.arange(len(lens)), lens)
    sl = slice(lead, lead + int(lens.sum()))
    want[sl] = (want[sl] + g[ids]).astype(np.float32) if accumulate else g[ids]
    assert np.array_equal(gx.to_numpy(), want)


def test_segmented_pipeline_in_a_graph(scl, orc):
    """Map(x*x+1) -> segmented inclusive Scan -> segmented Reduce, replayed from
    a captured CUDA graph after one eager run (which sizes the workspaces)."""
    off = log_uniform_offsets(1000, 6, 15, seed=11)
    n = int(off[-1])
    x = orc.uniform_f32(n, 12, -1.0, 1.0)
    mp = S.Program(S.KIND_MAP, "float func(float x){ return x*x + 1.0f; }", ["float", "float"])
    sp = S.Program(S.KIND_SCAN, FADD, ["float"], identity="0")
    rp = S.Program(S.KIND_REDUCE, FADD, ["float"], identity="0")
    dx, dm, ds = dev(x), S.DeviceArray(n, np.float32), S.DeviceArray(n, np.float32)
    dr, doff = S.DeviceArray(len(off) - 1, np.float32), dev(off)

    def step():
        mp.launch([dx, dm], n=n)
        sp.launch([dm, ds], n=n, flags=S.SHAPE_INCLUSIVE, segments=doff)
        rp.launch([ds, dr], n=n, segments=doff)

    step()
    eager = dr.to_numpy().copy()
    dr.upload(np.zeros(len(off) - 1, np.float32))
    S.check(S.lib().scl_graph_begin())
    step()
    g = ctypes.c_void_p()
    S.check(S.lib().scl_graph_end(ctypes.byref(g)))
    S.check(S.lib().scl_graph_launch(g))
    S.sync()
    replay = dr.to_numpy()
    S.check(S.lib().scl_graph_destroy(g))
    m = x.astype(np.float64) ** 2 + 1.0
    ids = seg_ids(off, n)
    cs = np.cumsum(m)
    scan = cs - np.concatenate([[0.0], cs])[off[:-1].astype(np.int64)][ids]
    ref = np.bincount(ids, weights=scan, minlength=len(off) - 1)
    assert np.all(np.abs(replay - ref) <= 1e-5 * np.abs(ref) + 1e-3)
    assert np.allclose(replay, eager, rtol=1e-6)


# ---- segment plans: the offsets pre-pass once, one launch per call ----------

@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_plan_scan_mixed_lengths_exact(scl, orc, flags):
    """With a plan the segmented Scan is one merged launch (tiles, then a warp
    per short vector); it gives the pre-pass path's bits and the reference's."""
    off = mixed_offsets(31)
    n = int(off[-1])
    x = orc.mod_i32(n, 32, 1001) - 500
    p = S.Program(S.KIND_SCAN, IADD, ["int"], identity="0")
    dx, dy, dz, doff = dev(x), S.DeviceArray(n, np.int32), S.DeviceArray(n, np.int32), dev(off)
    plan = S.SegPlan(doff, n)
    p.launch([dx, dy], n=n, flags=flags, segments=plan)
    p.launch([dx, dz], n=n, flags=flags, segments=doff)
    want = seg_scan_ref(x, off, flags)
    assert np.array_equal(dy.to_numpy(), want)
    assert np.array_equal(dz.to_numpy(), want)


def test_plan_reduce_mixed_lengths_exact(scl, orc):
    off = mixed_offsets(33)
    n = int(off[-1])
    x = orc.mod_i32(n, 34, 1001) - 500
    p = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="0")
    dout, doff = S.DeviceArray(len(off) - 1, np.int32), dev(off)
    plan = S.SegPlan(doff, n)
    ref = np.bincount(seg_ids(off, n), weights=x.astype(np.float64), minlength=len(off) - 1)
    for _ in range(3):  # the plan's per-vector tickets reset themselves
        dout.upload(np.zeros(len(off) - 1, np.int32))
        p.launch([dev(x), dout], n=n, segments=plan)
        assert np.array_equal(dout.to_numpy().astype(np.int64), ref.astype(np.int64))


def test_plan_one_launch_per_call(scl, orc):
    """After the first call with a tile shape (which numbers the tiles), every
    segmented Scan and Reduce with the plan is exactly one kernel launch --
    for short vectors only, long ones only, and a mix."""
    rng = np.random.default_rng(35)
    for lens in (rng.integers(1, 200, 100_000), rng.integers(5000, 100_000, 300),
                 np.concatenate([rng.integers(1, 200, 20_000), rng.integers(5000, 100_000, 50)])):
        off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
        n = int(off[-1])
        x = orc.uniform_f32(n, 36, -1.0, 1.0)
        sp = S.Program(S.KIND_SCAN, FADD, ["float"], identity="0")
        rp = S.Program(S.KIND_REDUCE, FADD, ["float"], identity="0")
        dx, dy, dr, doff = dev(x), S.DeviceArray(n, np.float32), S.DeviceArray(len(lens), np.float32), dev(off)
        plan = S.SegPlan(doff, n)
        sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, segments=plan)
        rp.launch([dx, dr], n=n, segments=plan)
        for _ in range(3):
            c0 = S.launch_count()
            sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, segments=plan)
            assert S.launch_count() == c0 + 1
            rp.launch([dx, dr], n=n, segments=plan)
            assert S.launch_count() == c0 + 2
        ids = seg_ids(off, n)
        cs = np.concatenate([[0.0], np.cumsum(x.astype(np.float64))])
        ref = cs[off[1:].astype(np.int64)] - cs[off[:-1].astype(np.int64)]
        assert np.all(np.abs(dr.to_numpy() - ref) <= 1e-6 * (1.0 + np.sqrt(lens)))
        scan = cs[1:] - cs[off[:-1].astype(np.int64)][ids]
        pos = np.arange(n) - off[:-1].astype(np.int64)[ids] + 1
        assert np.all(np.abs(dy.to_numpy() - scan) <= 1e-5 * (1.0 + np.sqrt(pos)))


def test_plan_on_a_longer_vector_and_misuse(scl, orc):
    """A plan made for the segments' total serves a longer input (elements
    past the last vector are left alone); a plan for other segments, or a
    shorter vector than the plan's, is refused."""
    off = np.array([0, 3, 3, 10, 5000, 9000], np.uint64)
    n = 12000
    x = orc.mod_i32(n, 37, 1001)
    p = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="0")
    doff = dev(off)
    plan = S.SegPlan(doff, int(off[-1]))
    dout = S.DeviceArray(len(off) - 1, np.int32)
    p.launch([dev(x), dout], n=n, segments=plan)
    xs = x.astype(np.int64)
    assert list(dout.to_numpy()) == [int(xs[int(a):int(b)].sum()) for a, b in zip(off[:-1], off[1:])]
    other = S.SegPlan(dev(np.array([0, 1, 2], np.uint64)), 2)
    ptrs = (ctypes.c_void_p * 2)(dev(x).ptr, dout.ptr)
    sh = S.Shape(n=n, seg_offsets=doff.ptr, n_segments=len(off) - 1, seg_plan=other.id)
    assert S.lib().scl_launch_reduce(p.handle, ctypes.byref(sh), ptrs, None, 0, None) == S.ERR_ARG
    sh = S.Shape(n=8000, seg_offsets=doff.ptr, n_segments=len(off) - 1, seg_plan=plan.id)
    assert S.lib().scl_launch_reduce(p.handle, ctypes.byref(sh), ptrs, None, 0, None) == S.ERR_ARG
    assert S.lib().scl_segplan_release(123456) == S.ERR_ARG


def test_plan_pipeline_in_a_graph(scl, orc):
    """Map -> segmented Scan -> segmented Reduce with a plan, replayed from a
    graph twice: one kernel per skeleton in the recording, and the same
    results on every replay."""
    off = log_uniform_offsets(3000, 0, 15, seed=38, zeros=30)
    n = int(off[-1])
    x = orc.uniform_f32(n, 39, -1.0, 1.0)
    mp = S.Program(S.KIND_MAP, "float func(float x){ return x*x + 1.0f; }", ["float", "float"])
    sp = S.Program(S.KIND_SCAN, FADD, ["float"], identity="0")
    rp = S.Program(S.KIND_REDUCE, FADD, ["float"], identity="0")
    dx, dm, ds = dev(x), S.DeviceArray(n, np.float32), S.DeviceArray(n, np.float32)
    dr, doff = S.DeviceArray(len(off) - 1, np.float32), dev(off)
    plan = S.SegPlan(doff, n)

    def step():
        mp.launch([dx, dm], n=n)
        sp.launch([dm, ds], n=n, flags=S.SHAPE_INCLUSIVE, segments=plan)
        rp.launch([ds, dr], n=n, segments=plan)

    step()
    eager = dr.to_numpy().copy()
    c0 = S.launch_count()
    S.check(S.lib().scl_graph_begin())
    step()
    g = ctypes.c_void_p()
    S.check(S.lib().scl_graph_end(ctypes.byref(g)))
    assert S.launch_count() == c0 + 3
    for _ in range(2):
        dr.upload(np.zeros(len(off) - 1, np.float32))
        S.check(S.lib().scl_graph_launch(g))
        S.sync()
        assert np.allclose(dr.to_numpy(), eager, rtol=1e-6, atol=1e-6)
    S.check(S.lib().scl_graph_destroy(g))


def test_graph_survives_workspace_growth(scl, orc):
    """A graph records the programs' workspace addresses; a later eager call
    that needs a larger workspace (or a new scan status layout) must leave
    the recorded one in place, so the graph replays correctly and the eager
    calls stay correct too."""
    n_small = 1_000_003
    off = mixed_offsets(41)
    n_big = int(off[-1])
    n_all = max(4 * n_small, n_big)
    x = orc.mod_i32(n_all, 40, 1001) - 500
    sp = S.Program(S.KIND_SCAN, IADD, ["int"], identity="0")
    rp = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="0")
    dx, dy, dr = dev(x), S.DeviceArray(n_all, np.int32), S.DeviceArray(1, np.int32)

    def small():
        sp.launch([dx, dy], n=n_small, flags=S.SHAPE_INCLUSIVE)
        rp.launch([dy, dr], n=n_small)

    small()
    S.check(S.lib().scl_graph_begin())
    small()
    g = ctypes.c_void_p()
    S.check(S.lib().scl_graph_end(ctypes.byref(g)))
    # eager calls that grow both workspaces (a longer scan; a segmented reduce)
    sp.launch([dx, dy], n=n_all, flags=S.SHAPE_INCLUSIVE)
    big = dy.to_numpy()
    assert np.array_equal(big, np.cumsum(x, dtype=np.int32))
    dseg = S.DeviceArray(len(off) - 1, np.int32)
    rp.launch([dx, dseg], n=n_big, segments=dev(off))
    want_small = np.cumsum(x[:n_small], dtype=np.int32)
    for _ in range(2):
        dy.upload(np.zeros(n_all, np.int32))
        S.check(S.lib().scl_graph_launch(g))
        S.sync()
        assert np.array_equal(dy.to_numpy()[:n_small], want_small)
        assert int(dr.to_numpy()[0]) == int(want_small.astype(np.int64).sum() & 0xFFFFFFFF) - \
            (1 << 32 if (int(want_small.astype(np.int64).sum()) & 0x80000000) else 0)
    S.check(S.lib().scl_graph_destroy(g))
    sp.launch([dx, dy], n=n_all, flags=S.SHAPE_INCLUSIVE)
    assert np.array_equal(dy.to_numpy(), big)


def test_flat_reduce_after_planned_segmented_reduce(scl, orc):
    """One Reduce program used segmented (with a plan) and flat in turn."""
    off = mixed_offsets(42)
    n = int(off[-1])
    x = orc.mod_i32(n, 43, 1001) - 500
    p = S.Program(S.KIND_REDUCE, IADD, ["int"], identity="0")
    dx, dseg, dflat = dev(x), S.DeviceArray(len(off) - 1, np.int32), S.DeviceArray(1, np.int32)
    plan = S.SegPlan(dev(off), n)
    ref_seg = np.bincount(seg_ids(off, n), weights=x.astype(np.float64), minlength=len(off) - 1)
    total = int(x.astype(np.int64).sum())
    for _ in range(3):
        p.launch([dx, dseg], n=n, segments=plan)
        p.launch([dx, dflat], n=n)
        assert np.array_equal(dseg.to_numpy().astype(np.int64), ref_seg.astype(np.int64))
        assert int(dflat.to_numpy()[0]) == total


def test_plan_double_and_empty_runs(scl, orc):
    """Planned segmented Scan and Reduce on double (8-byte elements: windows
    of 2048 elements, longer vectors on tiles), with runs of empty vectors
    between the others and at both ends: the identity for every empty
    vector's sum, and each scan against an FP64 reference."""
    rng = np.random.default_rng(44)
    lens = np.concatenate([np.zeros(50, np.int64), rng.integers(0, 3000, 3000), np.zeros(200, np.int64),
                           rng.integers(2040, 2060, 200), rng.integers(3000, 20_000, 40), np.zeros(30, np.int64)])
    rng.shuffle(lens[50:-30])
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    n = int(off[-1])
    x = orc.normal_f32(n, 45).astype(np.float64)
    sp = S.Program(S.KIND_SCAN, "double func(double a, double b){ return a + b; }", ["double"], identity="0")
    rp = S.Program(S.KIND_REDUCE, "double func(double a, double b){ return a + b; }", ["double"], identity="0")
    dx, dy, dr = dev(x), S.DeviceArray(n, np.float64), S.DeviceArray(len(lens), np.float64)
    plan = S.SegPlan(dev(off), n)
    ids = seg_ids(off, n)
    cs = np.concatenate([[0.0], np.cumsum(x)])
    starts = off[:-1].astype(np.int64)
    for flags in (S.SHAPE_INCLUSIVE, 0, S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE):
        sp.launch([dx, dy], n=n, flags=flags, segments=plan)
        incl = cs[1:] - cs[starts][ids]
        if flags & S.SHAPE_REVERSE:
            tot = (cs[off[1:].astype(np.int64)] - cs[starts])[ids]
            want = tot - incl + x
        else:
            want = incl if flags & S.SHAPE_INCLUSIVE else incl - x
        assert np.allclose(dy.to_numpy(), want, rtol=0, atol=1e-9 * (1 + np.abs(cs).max())), flags
    dr.upload(np.full(len(lens), 7.0))
    rp.launch([dx, dr], n=n, segments=plan)
    got = dr.to_numpy()
    ref = cs[off[1:].astype(np.int64)] - cs[starts]
    assert np.all(got[lens == 0] == 0.0)
    assert np.allclose(got, ref, rtol=0, atol=1e-9 * (1 + np.abs(cs).max()))
