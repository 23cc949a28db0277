"""Program binary cache on the GPU: a process that loads its cubins from
SKELCL_CACHE_DIR (SKELCL_LOAD_BINARY=YES) runs them without NVRTC and gets
the same bits as the process that compiled and saved them
(SKELCL_SAVE_BINARY=YES); with every file damaged, a third process compiles
again and still gets the same bits (src/Program.cpp:136-175, 252-281)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import hashlib, json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import oracle
import skelcl_gb300 as S
S.init(0)
n = (1 << 20) + 3
x = oracle.mod_i32(n, 3, 1001)
f = oracle.uniform_f32(n, 4, -1.0, 1.0)
scan = S.Program(S.KIND_SCAN, "int func(int x, int y){ return x + y; }", ["int"], identity="0")
red = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x + y; }", ["float"], identity="0")
dx, dy = S.DeviceArray.from_numpy(x), S.DeviceArray(n, np.int32)
df, dr = S.DeviceArray.from_numpy(f), S.DeviceArray(1, np.float32)
scan.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE)
# a lazily compiled variant: the register-tile scan with 4 rows
scan.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE,
            tuning=S.Tuning(variant=S.VARIANT_VECTOR, items=4, tile_w=4))
rev = dy.to_numpy()
scan.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE)
red.launch([df, dr], n=n)
h = hashlib.sha1(dy.to_numpy().tobytes() + rev.tobytes() + dr.to_numpy().tobytes()).hexdigest()
ok = bool(np.array_equal(dy.to_numpy(), np.cumsum(x, dtype=np.int32)))
print(json.dumps({"stats": S.cache_stats(), "digest": h, "scan_exact": ok}))
"""


def run_child(cache_dir, **env):
    e = dict(os.environ)
    for k in ("SKELCL_SAVE_BINARY", "SKELCL_LOAD_BINARY", "SKELCL_COMPILE_ALL"):
        e.pop(k, None)
    e["SKELCL_CACHE_DIR"] = str(cache_dir)
    e.update(env)
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=e, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_cached_cubins_run_bit_identical(built, tmp_path):
    saved = run_child(tmp_path, SKELCL_SAVE_BINARY="YES")
    assert saved["scan_exact"]
    assert saved["stats"]["nvrtc_compiles"] >= 3  # scan, reduce, the lazy variant
    assert saved["stats"]["disk_saves"] == saved["stats"]["nvrtc_compiles"]

    loaded = run_child(tmp_path, SKELCL_LOAD_BINARY="YES")
    assert loaded["stats"]["nvrtc_compiles"] == 0
    assert loaded["stats"]["disk_loads"] == saved["stats"]["disk_saves"]
    assert loaded["digest"] == saved["digest"]

    for f in Path(tmp_path).glob("*.skelcl"):
        b = f.read_bytes()
        f.write_bytes(b[: len(b) // 2])  # every entry truncated
    damaged = run_child(tmp_path, SKELCL_LOAD_BINARY="YES")
    assert damaged["stats"]["disk_rejects"] == saved["stats"]["disk_saves"]
    assert damaged["stats"]["nvrtc_compiles"] == saved["stats"]["nvrtc_compiles"]
    assert damaged["digest"] == saved["digest"]
