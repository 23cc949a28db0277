"""The launch autotuner: candidates are timed once per (program, skeleton,
size bucket), the winner is cached (memory and SKELCL_CACHE_DIR/autotune.tsv)
and reused; calls that are not repeatable (in place) are never tuned; every
candidate gives the same result."""
import ctypes
import os

import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu


@pytest.fixture
def tuning_on(scl, tmp_path):
    old = os.environ.get("SKELCL_CACHE_DIR")
    os.environ["SKELCL_CACHE_DIR"] = str(tmp_path)
    S.check(S.lib().scl_autotune_set(1))
    try:
        yield tmp_path
    finally:
        S.check(S.lib().scl_autotune_set(0))
        if old is None:
            os.environ.pop("SKELCL_CACHE_DIR", None)
        else:
            os.environ["SKELCL_CACHE_DIR"] = old


def test_map_is_tuned_once_and_cached(tuning_on, orc):
    n = (1 << 22) + 3
    x = orc.mod_i32(n, 1, 1001)
    p = S.Program(S.KIND_MAP, "int func(int x){ return x % 7; }", ["int", "int"])
    dx, dy = S.DeviceArray.from_numpy(x), S.DeviceArray(n, np.int32)
    c0 = S.launch_count()
    p.launch([dx, dy], n=n)
    first = S.launch_count() - c0
    assert np.array_equal(dy.to_numpy(), x % 7)
    c1 = S.launch_count()
    p.launch([dx, dy], n=n)
    assert S.launch_count() - c1 == 1  # cached: one launch
    assert first > 9                   # nine candidates were timed
    lines = (tuning_on / "autotune.tsv").read_text().splitlines()
    assert any("|map|22" in ln for ln in lines), lines


def test_in_place_map_is_not_tuned(tuning_on, orc):
    n = 1 << 20
    x = orc.mod_i32(n, 2, 1001)
    p = S.Program(S.KIND_MAP, "int func(int x){ return x + 1; }", ["int", "int"])
    d = S.DeviceArray.from_numpy(x)
    c0 = S.launch_count()
    p.launch([d, d], n=n)
    assert S.launch_count() - c0 == 1
    assert np.array_equal(d.to_numpy(), x + 1)  # applied exactly once


@pytest.mark.parametrize("segmented", [False, True])
def test_scan_and_reduce_tuned_results_exact(tuning_on, orc, segmented):
    n = 3_000_017
    x = orc.mod_i32(n, 3, 1001) - 500
    off = np.array([0, 5, 1_000_000, 1_000_001, n], np.uint64) if segmented else None
    seg = S.DeviceArray.from_numpy(off) if segmented else None
    sp = S.Program(S.KIND_SCAN, "int func(int x, int y){ return x + y; }", ["int"], identity="0")
    rp = S.Program(S.KIND_REDUCE, "int func(int x, int y){ return x + y; }", ["int"], identity="0")
    dx, dy = S.DeviceArray.from_numpy(x), S.DeviceArray(n, np.int32)
    nout = len(off) - 1 if segmented else 1
    dr = S.DeviceArray(nout, np.int32)
    for _ in range(2):  # tuned, then cached
        sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, segments=seg)
        rp.launch([dx, dr], n=n, segments=seg)
        x64 = x.astype(np.int64)
        if segmented:
            ref_scan = np.concatenate([np.cumsum(x64[int(a):int(b)]) for a, b in zip(off[:-1], off[1:])])
            ref_red = [int(x64[int(a):int(b)].sum()) for a, b in zip(off[:-1], off[1:])]
        else:
            ref_scan, ref_red = np.cumsum(x64), [int(x64.sum())]
        assert np.array_equal(dy.to_numpy(), ref_scan.astype(np.int32))
        assert list(dr.to_numpy()) == [np.int32(np.int64(v).astype(np.int32)) for v in ref_red]
    lines = (tuning_on / "autotune.tsv").read_text()
    assert ("|scan_seg|" in lines) == segmented and ("|reduce_seg|" in lines) == segmented


def test_mapoverlap_tuned(tuning_on, orc):
    rows, cols = 700, 1024
    img = orc.uniform_f32(rows * cols, 5, 0.0, 255.0)
    src = "float func(input_matrix_t m){ return getData(m, -1, 0) + getData(m, 1, 2); }"
    p = S.Program(S.KIND_MAPOVERLAP, src, ["float", "float"], overlap_range=2, padding=S.PAD_NEAREST)
    di, do = S.DeviceArray.from_numpy(img), S.DeviceArray(rows * cols, np.float32)
    p.launch([di, do], rows=rows, cols=cols)
    m = img.reshape(rows, cols)
    ys, xs = np.arange(rows), np.arange(cols)
    ref = m[ys][:, np.clip(xs - 1, 0, cols - 1)] + m[np.clip(ys + 2, 0, rows - 1)][:, np.clip(xs + 1, 0, cols - 1)]
    assert np.array_equal(do.to_numpy().reshape(rows, cols), ref)
    assert "|mapoverlap|" in (tuning_on / "autotune.tsv").read_text()
