"""Build libskelcl_cuda.so (sm_103a) and the CPU oracle library.

The CUDA library is compiled in-tree with nvcc for sm_103a only.  The
skeleton templates under csrc/templates are embedded into the library as
string literals; NVRTC compiles them, with the user function spliced in, when
a skeleton is constructed.

Usage: python -m skelcl_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
TPL = CSRC / "templates"
BUILD = PKG / "_build"
LIB = PKG / "libskelcl_cuda.so"
INCLUDE = ROOT / "include"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
TEMPLATES = ["prelude", "elementwise", "reduce", "scan", "mapoverlap_pre", "mapoverlap",
             "allpairs_pre", "allpairs"]
SOURCES = ["runtime.cu", "program.cpp", "splicer.cpp", "launch.cpp", "allpairs_tc.cu", "noalloc.cu", "adjoint.cu", "segments.cu", "tune.cpp"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _nvcc() -> str:
    p = _cuda_home() / "bin" / "nvcc"
    return str(p) if p.exists() else "nvcc"


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def _gen_templates() -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / "templates_gen.cpp"
    deps = [TPL / f"{n}.cuh" for n in TEMPLATES]
    if _newer(out, deps + [Path(__file__)]):
        return out
    lines = ["// generated from skelcl_gb300/csrc/templates by build.py; do not edit"]
    for n in TEMPLATES:
        text = (TPL / f"{n}.cuh").read_text()
        if ")SCLTPL\"" in text:
            raise RuntimeError(f"template {n} contains the raw-string delimiter")
        lines.append(f'extern const char* scl_tpl_{n};')
        lines.append(f'const char* scl_tpl_{n} = R"SCLTPL({text})SCLTPL";')
    out.write_text("\n".join(lines) + "\n")
    return out


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    gen = _gen_templates()
    headers = list(CSRC.glob("*.h")) + [INCLUDE / "skelcl_cuda.h"]
    srcs = [CSRC / s for s in SOURCES] + [gen]
    objs = []
    jobs = []
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo",
              f"-I{INCLUDE}", f"-I{CSRC}"]
    for s in srcs:
        o = BUILD / (s.name + ".o")
        objs.append(o)
        if not force and _newer(o, [s] + headers + [Path(__file__)]):
            continue
        cmd = [_nvcc(), *ARCH, *common, "-c", str(s), "-o", str(o)]
        jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr)
    if force or jobs or not _newer(LIB, objs):
        cuda_lib = _cuda_home() / "lib64"
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs),
               f"-L{cuda_lib}", "-lnvrtc", "-Xlinker", f"-rpath,{cuda_lib}"]
        _run(cmd)
    return LIB


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "oracle.c"
    hdr = ORACLE_DIR / "oracle.h"
    if not force and _newer(ORACLE_LIB, [src, hdr]):
        return ORACLE_LIB
    cc = shutil.which("gcc") or shutil.which("cc") or "cc"
    _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-fno-fast-math", "-ffp-contract=off",
          "-o", str(ORACLE_LIB), str(src), "-lpthread", "-lm"])
    return ORACLE_LIB


def build(force: bool = False, verbose: bool = False) -> None:
    build_cuda(force=force, verbose=verbose)
    build_oracle(force=force)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
