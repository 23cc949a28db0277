"""The drop-in C++ API (include/SkelCL): the reference's own gtest sources
for the skeleton path compile and link unchanged against these headers and
libskelcl_cuda.so (CPU; SKELCL_REFERENCE_DIR names the reference checkout,
and these cases skip without it), its SHA-1 suite runs unchanged here, and
the known-answer port in tests/cpp/skelcl_api_tests.cpp builds here and
passes on the GPU."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path(os.environ["SKELCL_REFERENCE_DIR"]) if os.environ.get("SKELCL_REFERENCE_DIR") else None
HAVE_REF = REF is not None and (REF / "test").is_dir()
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


def link_reference_suite(suite: str, out: Path) -> None:
    """One unchanged reference test file + the gtest-compatible harness's
    main(), linked against libskelcl_cuda.so: a symbol the headers declare
    but nothing defines fails here, as it would in the reference's build
    (test/CMakeLists.txt:12-33 links each suite with gtest_main)."""
    lib = ROOT / "skelcl_gb300"
    cmd = [CXX, "-std=c++17", "-O0", f"-I{ROOT / 'include'}", f"-I{ROOT / 'tests' / 'cpp'}",
           str(REF / "test" / f"{suite}.cpp"), str(ROOT / "tests" / "cpp" / "gtest_main.cpp"),
           f"-L{lib}", "-lskelcl_cuda", f"-Wl,-rpath,{lib}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.skipif(not HAVE_REF, reason="SKELCL_REFERENCE_DIR does not name the reference sources")
@pytest.mark.parametrize("suite", HOT_PATH_SUITES)
def test_reference_suite_links_unchanged(built, tmp_path, suite):
    link_reference_suite(suite, tmp_path / suite)


@pytest.mark.skipif(not HAVE_REF, reason="SKELCL_REFERENCE_DIR does not name the reference sources")
def test_reference_sha1_suite_passes_unchanged(built, tmp_path):
    """The one suite that needs no device runs here, unchanged."""
    exe = tmp_path / "SHA1Tests"
    link_reference_suite("SHA1Tests", exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "3 tests ran, 0 failed." in r.stdout, r.stdout + r.stderr


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
