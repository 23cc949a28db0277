"""Every skeleton over every scalar element type the SkelCL headers map
(char .. unsigned long, float, double): results against numpy with the
types' own wrap-around, so vector widths 16/8/4/2 and the scan's
element-size-dependent staging are all exercised."""
import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

TYPES = [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64,
         np.float32, np.float64]
SIZES = [1, 17, 4096 + 3, 300_001]


def dev(a):
    return S.DeviceArray.from_numpy(np.ascontiguousarray(a))


def data(dtype, n, seed):
    rng = np.random.default_rng(seed)
    if np.issubdtype(dtype, np.floating):
        return rng.uniform(-1.0, 1.0, n).astype(dtype)
    info = np.iinfo(dtype)
    lo, hi = max(info.min, -100), min(info.max, 100)
    return rng.integers(lo, hi + 1, n).astype(dtype)


def close(got, want, dtype, terms=1):
    if np.issubdtype(dtype, np.floating):
        tol = (1e-5 if dtype == np.float32 else 1e-12) * np.sqrt(terms) * (1 + np.abs(want))
        return bool(np.all(np.abs(got.astype(np.float64) - want.astype(np.float64)) <= tol))
    return bool(np.array_equal(got, want))


@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: np.dtype(t).name)
def test_map_zip_types(scl, dtype):
    t = S.CL_TYPE[np.dtype(dtype)]
    mp = S.Program(S.KIND_MAP, f"{t} func({t} x){{ return ({t})(x * ({t})3 + ({t})1); }}", [t, t])
    zp = S.Program(S.KIND_ZIP, f"{t} func({t} x, {t} y){{ return ({t})(x - y); }}", [t, t, t])
    for n in SIZES:
        x, y = data(dtype, n, 1), data(dtype, n, 2)
        dx, dy, do = dev(x), dev(y), S.DeviceArray(n, dtype)
        mp.launch([dx, do], n=n)
        with np.errstate(over="ignore"):
            want = (x * dtype(3) + dtype(1)).astype(dtype)
        assert close(do.to_numpy(), want, dtype), (n, "map")
        zp.launch([dx, dy, do], n=n)
        with np.errstate(over="ignore"):
            want = (x - y).astype(dtype)
        assert close(do.to_numpy(), want, dtype), (n, "zip")


@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: np.dtype(t).name)
def test_reduce_scan_types(scl, dtype):
    t = S.CL_TYPE[np.dtype(dtype)]
    src = f"{t} func({t} x, {t} y){{ return x + y; }}"
    rp = S.Program(S.KIND_REDUCE, src, [t], identity="0")
    sp = S.Program(S.KIND_SCAN, src, [t], identity="0")
    acc = np.float64 if np.issubdtype(dtype, np.floating) else (np.uint64 if np.dtype(dtype).kind == "u" else np.int64)
    for n in SIZES:
        x = data(dtype, n, 3)
        dx, dr, ds = dev(x), S.DeviceArray(1, dtype), S.DeviceArray(n, dtype)
        rp.launch([dx, dr], n=n)
        total = x.astype(acc).sum(dtype=acc)
        assert close(dr.to_numpy(), np.array([total]).astype(dtype), dtype, n), (n, "reduce")
        for flags in (0, S.SHAPE_INCLUSIVE, S.SHAPE_REVERSE, S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE):
            sp.launch([dx, ds], n=n, flags=flags)
            v = x[::-1] if flags & S.SHAPE_REVERSE else x
            incl = np.cumsum(v.astype(acc), dtype=acc)
            res = incl if flags & S.SHAPE_INCLUSIVE else incl - v.astype(acc)
            res = res[::-1] if flags & S.SHAPE_REVERSE else res
            assert close(ds.to_numpy(), res.astype(dtype), dtype, n), (n, flags)


@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: np.dtype(t).name)
def test_planned_segments_types_and_unaligned_views(scl, dtype):
    """Segmented Scan (all four forms) and Reduce with a segment plan over
    every element type, on views that start 0..3 elements past a 16-byte
    boundary: the window records' bulk-copied interiors and plain-loaded ends
    at every phase, vectors of one thread (<= 256 elements), of a warp and of
    the tiles, and empty ones."""
    t = S.CL_TYPE[np.dtype(dtype)]
    src = f"{t} func({t} x, {t} y){{ return x + y; }}"
    sp = S.Program(S.KIND_SCAN, src, [t], identity="0")
    rp = S.Program(S.KIND_REDUCE, src, [t], identity="0")
    rng = np.random.default_rng(40)
    lens = np.concatenate([rng.integers(0, 260, 3000), rng.integers(257, 4096, 60),
                           rng.integers(4097, 20_000, 4), [0, 1, 255, 256, 257, 4096, 0]])
    rng.shuffle(lens)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    n = int(off[-1])
    ids = np.repeat(np.arange(len(lens)), lens)
    doff = dev(off)
    for shift in range(4):
        x = data(dtype, n + shift, 41 + shift)
        base = dev(x)
        dx = base.view(shift, n)
        xs = x[shift:]
        dy, dr = S.DeviceArray(n, dtype), S.DeviceArray(len(lens), dtype)
        plan = S.SegPlan(doff, n)
        try:
            for flags in (0, 1, 2, 3):
                sp.launch([dx, dy], n=n, flags=flags, segments=plan)
                got = dy.to_numpy()
                inclusive, reverse = bool(flags & 1), bool(flags & 2)
                want = np.empty(n, dtype)
                for s in range(len(lens)):
                    lo, hi = int(off[s]), int(off[s + 1])
                    if lo == hi:
                        continue
                    seg = xs[lo:hi][::-1] if reverse else xs[lo:hi]
                    with np.errstate(over="ignore"):
                        c = np.cumsum(seg, dtype=dtype)
                        if not inclusive:
                            c = np.concatenate([[dtype(0)], c[:-1]]).astype(dtype)
                    want[lo:hi] = c[::-1] if reverse else c
                assert close(got, want, dtype, terms=int(lens.max())), (shift, flags)
            rp.launch([dx, dr], n=n, segments=plan)
            with np.errstate(over="ignore"):
                sums = np.zeros(len(lens), dtype)
                np.add.at(sums, ids, xs)
            assert close(dr.to_numpy(), sums, dtype, terms=int(lens.max())), (shift, "reduce")
        finally:
            plan.release()
