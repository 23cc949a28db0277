"""Host logic of segment plans, no device: the window records a plan makes
of its short vectors.  Every vector of at most short_max elements (empty
ones included) belongs to exactly one record and every longer one to none
(the tiles take those); records are ordered, their vectors consecutive and
starting in one window of short_max elements; a record's elements are
exactly its vectors' and span at most 2 * short_max (one staged tile)."""
import numpy as np
import pytest

import skelcl_gb300 as S


def check_records(off, short_max):
    off = np.asarray(off, np.uint64)
    n_seg = len(off) - 1
    rec = S.window_records(off, short_max)
    lens = (off[1:] - off[:-1]).astype(np.int64)
    owner = np.full(n_seg, -1)
    prev_end = 0
    for r, (first, end, e0, ln) in enumerate(rec.astype(np.int64)):
        assert prev_end <= first < end <= n_seg, (r, first, end)
        prev_end = end
        assert np.all(owner[first:end] == -1)
        owner[first:end] = r
        w = off[first] // short_max
        assert np.all(off[first:end] // short_max == w), "vectors start in one window"
        assert np.all(lens[first:end] <= short_max)
        assert e0 == off[first] and ln == off[end] - off[first], (r, e0, ln)
        assert ln <= 2 * short_max
    short = lens <= short_max
    assert np.all(owner[short] >= 0), np.nonzero(short & (owner < 0))[0][:5]
    assert np.all(owner[~short] == -1)
    return rec


@pytest.mark.parametrize("short_max", [1, 7, 4096])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_window_records_random(built, seed, short_max):
    rng = np.random.default_rng(seed)
    lens = np.concatenate([rng.integers(0, 3 * short_max + 2, 4000),
                           np.zeros(50, np.int64), [short_max, short_max + 1, 2 * short_max]])
    rng.shuffle(lens)
    off = np.concatenate([[0], np.cumsum(lens)])
    check_records(off, short_max)


def test_window_records_edges(built):
    sm = 4096
    # all empty: one record holding every vector
    rec = check_records(np.zeros(11, np.uint64), sm)
    assert rec.tolist() == [[0, 10, 0, 0]]
    # one long vector: no record
    assert len(check_records([0, 3 * sm], sm)) == 0
    # short vectors filling a window exactly, then one that starts the next
    rec = check_records([0, sm // 2, sm, sm + 1], sm)
    assert rec.tolist() == [[0, 2, 0, sm], [2, 3, sm, 1]]
    # a short vector, then a long one starting in the same window
    rec = check_records([0, 10, 10 + 2 * sm], sm)
    assert rec.tolist() == [[0, 1, 0, 10]]
    # a vector reaching into the next window ends its record there
    rec = check_records([0, sm - 1, 2 * sm - 2, 2 * sm], sm)
    assert rec.tolist() == [[0, 2, 0, 2 * sm - 2], [2, 3, 2 * sm - 2, 2]]


def test_window_records_bad_arguments(built):
    import ctypes
    cnt = ctypes.c_uint64(0)
    off = np.array([0, 5], np.uint64)
    assert S.lib().scl_debug_window_records(off.ctypes.data, 1, 0, None, 0, ctypes.byref(cnt)) == S.ERR_ARG
    rec = np.zeros((1, 4), np.uint64)
    off = np.array([0, 1, 5000, 5001], np.uint64)
    assert S.lib().scl_debug_window_records(off.ctypes.data, 3, 4096, rec.ctypes.data, 1,
                                            ctypes.byref(cnt)) == S.ERR_ARG
