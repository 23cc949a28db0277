"""Examples as drivers: the reference's example programs compile and link
unchanged against include/SkelCL, include/pvsutil and libskelcl_cuda.so
(CPU; SKELCL_REFERENCE_DIR names the reference checkout, and these cases skip
without it); this repository's examples/ build and, on the GPU, run with
--check against host loops."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path(os.environ["SKELCL_REFERENCE_DIR"]) if os.environ.get("SKELCL_REFERENCE_DIR") else None
HAVE_REF = REF is not None and (REF / "examples").is_dir()
CXX = shutil.which("g++") or "g++"
OURS = ["dot_product", "saxpy", "gauss", "matrix_mult", "mandelbrot"]
RUN_ARGS = {"dot_product": ["-n", "1000003"], "saxpy": ["-n", "100003"], "gauss": ["-r", "5"],
            "matrix_mult": ["-n", "512", "-k", "256"], "mandelbrot": ["-w", "640", "-h", "480"]}


def build(name: str, out: Path) -> None:
    lib = ROOT / "skelcl_gb300"
    r = subprocess.run([CXX, "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(ROOT / "examples" / f"{name}.cpp"),
                        f"-L{lib}", "-lskelcl_cuda", f"-Wl,-rpath,{lib}", "-o", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.skipif(not HAVE_REF, reason="SKELCL_REFERENCE_DIR does not name the reference sources")
@pytest.mark.parametrize("example", ["dot_product", "gauss", "mandelbrot", "matrix_mult", "montecarlo", "saxpy"])
def test_reference_example_links_unchanged(built, tmp_path, example):
    lib = ROOT / "skelcl_gb300"
    r = subprocess.run([CXX, "-std=c++17", "-O0", f"-I{ROOT / 'include'}",
                        str(REF / "examples" / example / "main.cpp"), f"-L{lib}", "-lskelcl_cuda",
                        f"-Wl,-rpath,{lib}", "-o", str(tmp_path / example)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.parametrize("example", OURS)
def test_example_builds(built, tmp_path, example):
    build(example, tmp_path / example)


def test_command_line_parser(built, tmp_path):
    build("saxpy", tmp_path / "saxpy")
    r = subprocess.run([str(tmp_path / "saxpy"), "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--alpha" in r.stdout and "(default: 2.5)" in r.stdout, r.stdout
    r = subprocess.run([str(tmp_path / "saxpy"), "--no-such-flag"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0


@pytest.mark.gpu
@pytest.mark.parametrize("example", OURS)
def test_example_runs_and_checks(built, tmp_path, example):
    exe = tmp_path / example
    build(example, exe)
    env = dict(os.environ, SKELCL_CACHE_DIR=str(tmp_path))
    r = subprocess.run([str(exe), "--check"] + RUN_ARGS[example], capture_output=True, text=True,
                       timeout=600, cwd=str(tmp_path), env=env)
    out = r.stdout[-4000:] + r.stderr[-2000:]
    assert r.returncode == 0 and "PASSED" in r.stdout, out
