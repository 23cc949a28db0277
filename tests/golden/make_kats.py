"""Collect the reference's known-answer tests for the skeleton path into
reference_kats.json.

The reference (SkelCL) computes every expectation inside its gtest files; it
ships no fixture files.  This script reads those test files, checks that each
known answer used here is literally present at the cited line, and writes the
cases as data, so the oracle and the GPU path can be pinned against them on a
machine without the reference sources.

Run: python tests/golden/make_kats.py [path-to-reference]
     (default: the directory SKELCL_REFERENCE_DIR names)
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

# (id, file, line, anchor text that must appear on that line, case data)
CASES = [
    ("reduce_float_sum_0_99", "test/ReduceTests.cpp", 89, "EXPECT_EQ(4950, output[0]);",
     {"skeleton": "reduce", "type": "float", "source": "float func(float x, float y){ return x+y; }",
      "input": {"arange": 100}, "expected": 4950}),
    ("reduce_float_extra_arg", "test/ReduceTests.cpp", 102, "r(input, 1.0f)",
     {"skeleton": "reduce", "type": "float",
      "source": "float func(float x, float y, float a){ return a*(x+y); }",
      "input": {"arange": 100}, "extra": [1.0], "expected": 4950}),
    ("reduce_int_sum_0_1586", "test/ReduceTests.cpp", 120, "EXPECT_EQ(1258491, output[0]);",
     {"skeleton": "reduce", "type": "int", "source": "int func(int x, int y){ return x+y; }",
      "input": {"arange": 1587}, "expected": 1258491}),
    ("reduce_int_1e8_ones", "test/ReduceTests.cpp", 135, "EXPECT_EQ(100000000, output[0]);",
     {"skeleton": "reduce", "type": "int", "source": "int func(int x, int y){ return x+y; }",
      "input": {"ones": 100000000}, "expected": 100000000}),
    ("reduce_float_sizes_1_255", "test/ReduceTests.cpp", 147, "for (int i = 1; i < N; ++i) {",
     {"skeleton": "reduce", "type": "float", "source": "float func(float x, float y){ return x+y; }",
      "input": {"ones_sizes": [1, 256]}, "expected": "size"}),
    ("reduce_float_sizes_8192_8447", "test/ReduceTests.cpp", 164, "for (int i = 8192; i < (8192 + N); ++i) {",
     {"skeleton": "reduce", "type": "float", "source": "float func(float x, float y){ return x+y; }",
      "input": {"ones_sizes": [8192, 8448]}, "expected": "size"}),
    ("scan_int_1024_ones", "test/ScanTests.cpp", 74, "skelcl::Vector<int> input(1024);",
     {"skeleton": "scan", "type": "int", "source": "int func(int x, int y){ return x+y; }",
      "identity": "0", "input": {"ones": 1024}, "expected": "index"}),
    ("scan_int_10_ones", "test/ScanTests.cpp", 93, "skelcl::Vector<int> input(10);",
     {"skeleton": "scan", "type": "int", "source": "int func(int x, int y){ return x+y; }",
      "identity": "0", "input": {"ones": 10}, "expected": "index"}),
    ("sha1_empty", "test/SHA1Tests.cpp", 60, "da39a3ee5e6b4b0d3255bfef95601890afd80709",
     {"text": "", "expected": "da39a3ee5e6b4b0d3255bfef95601890afd80709"}),
    ("sha1_lazy_dog", "test/SHA1Tests.cpp", 67, "2fd4e1c67a2d28fced849ee1bb76e7391b93eb12",
     {"text": "The quick brown fox jumps over the lazy dog",
      "expected": "2fd4e1c67a2d28fced849ee1bb76e7391b93eb12"}),
    ("sha1_lazy_cog", "test/SHA1Tests.cpp", 74, "de9f2c7fd25e1b3afad3e85a0bd17d9b100db4b3",
     {"text": "The quick brown fox jumps over the lazy cog",
      "expected": "de9f2c7fd25e1b3afad3e85a0bd17d9b100db4b3"}),
    ("mapoverlap_right_shift_1024", "test/MapOverlapTests.cpp", 189, "getData(f, -1, 0)",
     {"skeleton": "mapoverlap", "type": "int", "range": 1, "dx": -1, "dy": 0, "size": 1024,
      "fill": "i*j+i", "padding": "NEAREST"}),
    ("mapoverlap_two_right_shift_100", "test/MapOverlapTests.cpp", 222, "getData(f, -2, 0)",
     {"skeleton": "mapoverlap", "type": "int", "range": 2, "dx": -2, "dy": 0, "size": 100,
      "fill": "j", "padding": "NEAREST"}),
    ("mapoverlap_left_shift_100", "test/MapOverlapTests.cpp", 253, "getData(f, +1, 0)",
     {"skeleton": "mapoverlap", "type": "int", "range": 1, "dx": 1, "dy": 0, "size": 100,
      "fill": "j", "padding": "NEAREST"}),
    ("mapoverlap_two_left_shift_100", "test/MapOverlapTests.cpp", 287, "getData(f, +2, 0)",
     {"skeleton": "mapoverlap", "type": "int", "range": 2, "dx": 2, "dy": 0, "size": 100,
      "fill": "j", "padding": "NEAREST"}),
    ("mapoverlap_down_shift_1024", "test/MapOverlapTests.cpp", 319, "getData(f, 0, -1)",
     {"skeleton": "mapoverlap", "type": "int", "range": 1, "dx": 0, "dy": -1, "size": 1024,
      "fill": "i", "padding": "NEAREST"}),
    ("mapoverlap_two_down_shift_100", "test/MapOverlapTests.cpp", 352, "getData(f, 0, -2)",
     {"skeleton": "mapoverlap", "type": "int", "range": 2, "dx": 0, "dy": -2, "size": 100,
      "fill": "i", "padding": "NEAREST"}),
    ("mapoverlap_up_shift_1024", "test/MapOverlapTests.cpp", 385, "getData(f, 0, +1)",
     {"skeleton": "mapoverlap", "type": "int", "range": 1, "dx": 0, "dy": 1, "size": 1024,
      "fill": "i", "padding": "NEAREST"}),
    ("mapoverlap_two_up_shift_100", "test/MapOverlapTests.cpp", 419, "getData(f, 0, +2)",
     {"skeleton": "mapoverlap", "type": "int", "range": 2, "dx": 0, "dy": 2, "size": 100,
      "fill": "i", "padding": "NEAREST"}),
    ("allpairs_matmul_64x64x64", "test/AllPairsTests.cpp", 80, "testAllPairsWithMatrices(64, 64, 64);",
     {"skeleton": "allpairs", "height": 64, "dim": 64, "width": 64, "left_mod": 100, "right_mod": 101}),
    ("allpairs_matmul_32x128x32", "test/AllPairsTests.cpp", 85, "testAllPairsWithMatrices(32, 128, 32);",
     {"skeleton": "allpairs", "height": 32, "dim": 128, "width": 32, "left_mod": 100, "right_mod": 101}),
    ("allpairs_matmul_100x60x11", "test/AllPairsTests.cpp", 90, "testAllPairsWithMatrices(100, 60, 11);",
     {"skeleton": "allpairs", "height": 100, "dim": 60, "width": 11, "left_mod": 100, "right_mod": 101}),
    ("allpairs_extra_args_reduce_first", "test/AllPairsTests.cpp", 160, "allpairs(left, right, b, a)",
     {"skeleton": "allpairs", "height": 64, "dim": 64, "width": 64, "zip": "x*y+a", "reduce": "x+y+b",
      "a": 5.0, "b": 6.0}),
    ("index_vector_map", "test/IndexVectorTests.cpp", 86, "int func(Index i) { return i; }",
     {"skeleton": "map_index", "size": 1023, "expected": "index"}),
    ("index_matrix_map", "test/IndexMatrixTests.cpp", 89, "return i.y+i.x;",
     {"skeleton": "map_point", "rows": 32, "cols": 128, "expected": "y+x"}),
]


def main(ref_root: Path) -> None:
    out = []
    for cid, f, line, anchor, data in CASES:
        lines = (ref_root / f).read_text(errors="replace").splitlines()
        window = "\n".join(lines[max(0, line - 3):line + 2])
        if anchor not in window:
            raise SystemExit(f"{cid}: anchor {anchor!r} not found near {f}:{line}")
        out.append({"id": cid, "ref": f"{f}:{line}", **data})
    path = HERE / "reference_kats.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {len(out)} cases to {path}")


if __name__ == "__main__":
    import os
    where = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SKELCL_REFERENCE_DIR")
    if not where:
        raise SystemExit("usage: make_kats.py PATH-TO-REFERENCE (or set SKELCL_REFERENCE_DIR)")
    main(Path(where))
