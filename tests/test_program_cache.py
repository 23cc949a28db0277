"""Program binary cache (SKELCL_SAVE_BINARY / SKELCL_LOAD_BINARY, the
reference's switches in src/Program.cpp:136-175, 252-281), across processes.

Each step runs in a fresh Python process (the in-process cache would
otherwise answer first) and reports the library's cache counters: a process
that saves compiles with NVRTC and writes one file per compilation; a later
process that loads compiles nothing; truncated, garbled, foreign-key and
old-format files are rejected and compiled again.  CPU only: compile-only
programs go through the same cache, keyed without a device."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import skelcl_gb300 as S
S.compile_only(S.KIND_SCAN, "int func(int x, int y){ return x + y; }", ["int"], identity="0")
S.compile_only(S.KIND_MAP, "float func(float x){ return x * 2.0f; }", ["float", "float"])
S.compile_only(S.KIND_REDUCE, "float func(float x, float y){ return x + y; }", ["float"], identity="0")
print(json.dumps(S.cache_stats()))
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


def entries(cache_dir):
    return sorted(Path(cache_dir).glob("*.skelcl"))


def test_save_then_load_skips_nvrtc(built, tmp_path):
    saved = run_child(tmp_path, SKELCL_SAVE_BINARY="YES")
    assert saved["nvrtc_compiles"] >= 3 and saved["disk_saves"] == saved["nvrtc_compiles"]
    assert len(entries(tmp_path)) == saved["disk_saves"]
    loaded = run_child(tmp_path, SKELCL_LOAD_BINARY="YES")
    assert loaded == {"nvrtc_compiles": 0, "disk_loads": saved["disk_saves"], "disk_rejects": 0,
                      "disk_saves": 0}
    # without the switch the files are not read
    plain = run_child(tmp_path)
    assert plain["disk_loads"] == 0 and plain["nvrtc_compiles"] == saved["nvrtc_compiles"]


def test_damaged_files_are_compiled_again(built, tmp_path):
    saved = run_child(tmp_path, SKELCL_SAVE_BINARY="YES")
    files = entries(tmp_path)
    assert len(files) >= 3
    data = [f.read_bytes() for f in files]
    files[0].write_bytes(data[0][: len(data[0]) - 100])        # truncated cubin
    garbled = bytearray(data[1])
    garbled[-50] ^= 0xFF                                         # one byte of the cubin flipped
    files[1].write_bytes(bytes(garbled))
    files[2].write_bytes(data[0])                                # another program's entry
    damaged = run_child(tmp_path, SKELCL_LOAD_BINARY="YES", SKELCL_SAVE_BINARY="YES")
    assert damaged["disk_rejects"] == 3
    assert damaged["nvrtc_compiles"] == 3 and damaged["disk_saves"] == 3
    assert damaged["disk_loads"] == saved["disk_saves"] - 3
    # the rewritten files load again
    again = run_child(tmp_path, SKELCL_LOAD_BINARY="YES")
    assert again["nvrtc_compiles"] == 0 and again["disk_rejects"] == 0


def test_old_format_and_extra_bytes_are_rejected(built, tmp_path):
    run_child(tmp_path, SKELCL_SAVE_BINARY="YES")
    files = entries(tmp_path)
    first = files[0].read_bytes()
    files[0].write_bytes(first.replace(b"SCLBIN2\n", b"SCLBIN1\n", 1))
    files[1].write_bytes(files[1].read_bytes() + b"\0")
    r = run_child(tmp_path, SKELCL_LOAD_BINARY="YES")
    assert r["disk_rejects"] == 2 and r["nvrtc_compiles"] == 2
