"""The drop-in C++ API (include/SkelCL): the reference's own gtest sources
for the skeleton path compile unchanged against these headers (CPU, when the
reference sources are present), and the known-answer port in
tests/cpp/skelcl_api_tests.cpp builds here and passes on the GPU."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path("/root/reference")
CXX = shutil.which("g++") or "g++"
HOT_PATH_SUITES = ["MapTests", "ZipTests", "ReduceTests", "ScanTests", "MapOverlapTests",
                   "AllPairsTests", "IndexVectorTests", "IndexMatrixTests", "SHA1Tests",
                   "VectorTests", "MatrixTests", "DistributionTests"]


def build_port(out: Path, source: str = "skelcl_api_tests.cpp") -> None:
    lib = ROOT / "skelcl_gb300"
    cmd = [CXX, "-std=c++17", "-O1", f"-I{ROOT / 'include'}", f"-I{ROOT / 'tests' / 'cpp'}",
           str(ROOT / "tests" / "cpp" / source), f"-L{lib}", "-lskelcl_cuda",
           f"-Wl,-rpath,{lib}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.skipif(not REF.exists(), reason="reference sources not present")
@pytest.mark.parametrize("suite", HOT_PATH_SUITES)
def test_reference_suite_compiles_unchanged(built, suite):
    src = REF / "test" / f"{suite}.cpp"
    r = subprocess.run([CXX, "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'include'}",
                        f"-I{ROOT / 'tests' / 'cpp'}", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_api_port_builds(built, tmp_path):
    build_port(tmp_path / "skelcl_api_tests")


@pytest.mark.gpu
def test_api_port_passes_on_gpu(built, tmp_path):
    exe = tmp_path / "skelcl_api_tests"
    build_port(exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900,
                       cwd=str(tmp_path), env=dict(os.environ))
    tail = r.stdout[-6000:] + r.stderr[-2000:]
    assert r.returncode == 0, tail
    assert " 0 failed." in r.stdout, tail


def test_adjoint_tape_builds(built, tmp_path):
    build_port(tmp_path / "adjoint_tests", "adjoint_tests.cpp")


@pytest.mark.gpu
def test_adjoint_tape_passes_on_gpu(built, tmp_path):
    """The reverse-mode tape (include/SkelCL/Adjoint.h): gradients against FP64
    finite differences and against gradients composed from forward skeletons."""
    exe = tmp_path / "adjoint_tests"
    build_port(exe, "adjoint_tests.cpp")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900,
                       cwd=str(tmp_path), env=dict(os.environ))
    tail = r.stdout[-6000:] + r.stderr[-2000:]
    assert r.returncode == 0, tail
    assert " 0 failed." in r.stdout, tail


def test_extensions_build(built, tmp_path):
    build_port(tmp_path / "extensions_tests", "extensions_tests.cpp")


@pytest.mark.gpu
def test_extensions_pass_on_gpu(built, tmp_path):
    """Segmented Scan/Reduce, graph replay and autotuning through the C++ API."""
    exe = tmp_path / "extensions_tests"
    build_port(exe, "extensions_tests.cpp")
    env = dict(os.environ, SKELCL_CACHE_DIR=str(tmp_path))
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900, cwd=str(tmp_path), env=env)
    tail = r.stdout[-6000:] + r.stderr[-2000:]
    assert r.returncode == 0, tail
    assert " 0 failed." in r.stdout, tail
