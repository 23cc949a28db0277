"""CPU tests of the C ABI: the library loads and exports every declared
entry point, SHA-1 matches the reference's known answers, and the user
functions from the reference's tests splice and compile with NVRTC for
sm_103a (no device needed)."""
import json
import re
from pathlib import Path

import pytest

import skelcl_gb300 as s

ROOT = Path(__file__).resolve().parent.parent
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def declared_symbols():
    text = (ROOT / "include" / "skelcl_cuda.h").read_text()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(scl_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol(built):
    L = s.lib()
    names = declared_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(s.SIGNATURES), set(names) - set(s.SIGNATURES)
    assert L.scl_abi_version() == 1


def test_calls_before_init_fail_cleanly(built):
    import ctypes
    L = s.lib()
    if L.scl_is_initialized():
        pytest.skip("already initialised in this process")
    p = ctypes.c_void_p()
    assert L.scl_alloc(16, ctypes.byref(p)) == s.ERR_NOT_INIT
    assert b"scl_init" in L.scl_last_error_string()


@pytest.mark.parametrize("k", [k for k in KATS if k["id"].startswith("sha1")], ids=lambda k: k["id"])
def test_sha1_kats(built, k):
    assert s.sha1_hex(k["text"].encode()) == k["expected"]


def test_sha1_lengths(built):
    import hashlib
    for n in (55, 56, 63, 64, 65, 119, 120, 1000):
        data = bytes(range(256)) * 4
        assert s.sha1_hex(data[:n]) == hashlib.sha1(data[:n]).hexdigest()


# User functions from the reference's test suite (test/*.cpp), by skeleton.
REF_FUNCS = [
    (s.KIND_MAP, "float func(float f){ return -f; }", ["float", "float"], {}),
    (s.KIND_MAP, "float func(float f, float add, float add2) { return f+add+add2; }", ["float", "float"], {}),
    (s.KIND_MAP, "int func(float f) { return skelcl_get_device_id(); }", ["float", "int"], {}),
    (s.KIND_MAP_VOID, "void func(float f, __global float* out) { out[get_global_id(0)] = f; }", ["float"], {}),
    (s.KIND_MAP, "float func( float f, float_matrix_t mat, float add2, int_matrix_t mat2 )\n"
                 "{ return f + get(mat, 1, 1) + add2 + get(mat2, 1, 2); }", ["float", "float"], {}),
    (s.KIND_MAP, "int func(int i, __local int* lp) { lp[0] = i; barrier(CLK_LOCAL_MEM_FENCE); return -lp[0]; }",
     ["int", "int"], {}),
    (s.KIND_MAP, "float4 func(float4 f) { return -f; }", ["float4", "float4"], {}),
    (s.KIND_MAP, "double4 func(double4 f) { return -f; }", ["double4", "double4"], {}),
    (s.KIND_MAP, "int func(int i) { return -i; }", ["int", "int"], {}),
    (s.KIND_ZIP, "float func(float x, float y){ return x+y; }", ["float", "float", "float"], {}),
    (s.KIND_ZIP, "float func(float x, float y, float add, float add2) { return (x*y)+add+add2; }",
     ["float", "float", "float"], {}),
    (s.KIND_ZIP, "float func(float x, float y) { return x; }", ["float", "float", "float"], {}),
    (s.KIND_ZIP_VOID, "void func(float x, float y, __global float* out) { out[get_global_id(0)] = x*y; }",
     ["float", "float"], {}),
    (s.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], {"identity": "0"}),
    (s.KIND_REDUCE, "float func(float x, float y, float a){ return a*(x+y); }", ["float"], {"identity": "0"}),
    (s.KIND_REDUCE, "int func(int x, int y){ return x+y; }", ["int"], {"identity": "0"}),
    (s.KIND_SCAN, "int func(int x, int y){ return x+y; }", ["int"], {"identity": "0"}),
    (s.KIND_SCAN, "float func(float x, float y){ return x+y; }", ["float"], {"identity": "0.0f"}),
    (s.KIND_MAPOVERLAP, "int func(input_matrix_t f){ return getData(f, -1, 0); }", ["int", "int"],
     {"overlap_range": 1}),
    (s.KIND_MAPOVERLAP, "int func(input_matrix_t img, __global float* kernelVec, int range)\n"
                        "{ float sum = 0.0f; float norm = 0.0f;\n"
                        "  for (int i = -range; i <= range; i++) for (int j = -range; j <= range; j++) {\n"
                        "    sum += getData(img, i, j) * kernelVec[(i + j) / 2 + range];\n"
                        "    norm += kernelVec[(i + j) / 2 + range]; }\n"
                        "  float v = sum / norm; return (v > 255) ? 255 : ((v < 0) ? 0 : v); }",
     ["int", "int"], {"overlap_range": 5}),
    (s.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float", "float", "float"],
     {"source2": "float func(float x, float y){ return x*y; }", "identity": "0"}),
    (s.KIND_ALLPAIRS, "float func(float x, float y, float b){ return x+y+b; }", ["float", "float", "float"],
     {"source2": "float func(float x, float y, float a){ return x*y+a; }", "identity": "0"}),
    (s.KIND_ALLPAIRS_GENERIC,
     "float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim) {"
     "float res = 0; for (int i = 0; i < dim; ++i) {"
     "  res += getElementFromRow(row, i) * getElementFromColumn(col, i); } return res; }",
     ["float", "float", "float"], {}),
    (s.KIND_ALLPAIRS_GENERIC,
     "float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim, int start) {"
     "float res = start; for (int i = 0; i < dim; ++i) {"
     "  res += getElementFromRow(row, i) * getElementFromColumn(col, i); } return res; }",
     ["float", "float", "float"], {}),
    (s.KIND_MAP_INDEX, "int func(Index i) { return i; }", ["int"], {}),
    (s.KIND_MAP_INDEX_VOID, "void func(Index i, __global int* out) { out[i] = i; }", [], {}),
    (s.KIND_MAP_POINT, "int func(IndexPoint i) { return i.y+i.x; }", ["int"], {}),
    (s.KIND_MAP_POINT_VOID, "void func(IndexPoint ip, int_matrix_t out) { set(out, ip.y, ip.x, ip.y+ip.x); }",
     [], {}),
]


@pytest.mark.parametrize("kind,src,types,kw", REF_FUNCS)
def test_reference_user_functions_compile(built, kind, src, types, kw):
    s.compile_only(kind, src, types, **kw)


# Every kernel variant of each skeleton kind (those compiled on first use
# included), so that a template error shows without a GPU.
STENCIL3 = ("float func(input_matrix_t m, __global float* w) { float s = 0.0f;"
            " for (int dy = -1; dy <= 1; ++dy) for (int dx = -1; dx <= 1; ++dx)"
            "  s += getData(m, dx, dy) * w[(dy + 1) * 3 + (dx + 1)]; return s; }")
ALL_VARIANTS = [
    (s.KIND_MAP, "float func(float f){ return -f; }", ["float", "float"], {}),
    (s.KIND_MAP, "int func(int i, __local int* lp) { lp[0] = i; return -lp[0]; }", ["int", "int"], {}),
    (s.KIND_ZIP, "float func(float x, float y){ return x*y; }", ["float"] * 3, {}),
    (s.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], {"identity": "0"}),
    (s.KIND_REDUCE, "double func(double x, double y){ return x+y; }", ["double"], {"identity": "0"}),
    (s.KIND_REDUCE, "unsigned char func(unsigned char x, unsigned char y){ return x > y ? x : y; }",
     ["unsigned char"], {"identity": "0"}),
    (s.KIND_SCAN, "int func(int x, int y){ return x+y; }", ["int"], {"identity": "0"}),
    (s.KIND_SCAN, "float func(float x, float y){ return x+y; }", ["float"], {"identity": "0"}),
    (s.KIND_SCAN, "long func(long x, long y){ return x+y; }", ["long"], {"identity": "0"}),
    (s.KIND_MAPOVERLAP, STENCIL3, ["float", "float"], {"overlap_range": 1}),
    (s.KIND_MAPOVERLAP, STENCIL3, ["float", "float"], {"overlap_range": 1, "flags": s.PROG_STENCIL_COLS2}),
    (s.KIND_MAPOVERLAP, STENCIL3, ["float", "float"], {"overlap_range": 1, "flags": s.PROG_STENCIL_COLS1}),
    (s.KIND_MAPOVERLAP, "unsigned char func(input_matrix_t m){ return getData(m, 1, -1); }",
     ["unsigned char", "unsigned char"], {"overlap_range": 1, "padding": s.PAD_NEAREST}),
    (s.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
     {"source2": "float func(float x, float y){ return x*y; }", "identity": "0"}),
    (s.KIND_ALLPAIRS, "double func(double x, double y){ return x+y; }", ["double"] * 3,
     {"source2": "double func(double x, double y){ return fabs(x-y); }", "identity": "0"}),
    (s.KIND_ALLPAIRS_GENERIC,
     "float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim) { float r = 0;"
     " for (unsigned int i = 0; i < dim; ++i) r += getElementFromRow(row, i) * getElementFromColumn(col, i);"
     " return r; }", ["float"] * 3, {}),
    (s.KIND_ZIP_REDUCE, "float func(float x, float y){ return x+y; }", ["float"] * 3,
     {"source2": "float m(float x, float y){ return x*y; }", "func2": "m", "identity": "0"}),
    (s.KIND_SCAN_MAP, "int func(int x, int y){ return x+y; }", ["int", "int"],
     {"source2": "int m(int x){ return x % 7; }", "func2": "m", "identity": "0"}),
    (s.KIND_MAP_ADJOINT, "float d(float x, float g){ return 2.0f*x*g; }", ["float", "float"], {"func": "d"}),
    (s.KIND_ZIP_ADJOINT, "float dl(float x, float y, float g){ return y*g; }\n"
                         "float dr(float x, float y, float g){ return x*g; }", ["float"] * 3,
     {"func": "dl", "func2": "dr"}),
]


@pytest.mark.parametrize("kind,src,types,kw", ALL_VARIANTS)
def test_every_kernel_variant_compiles(built, kind, src, types, kw):
    kw = dict(kw)
    kw["flags"] = kw.get("flags", 0) | s.PROG_COMPILE_ALL
    s.compile_only(kind, src, types, **kw)


def test_splice_forwards_extra_params_in_order(built):
    src = "float func(float f, float_matrix_t mat, float add2, int_matrix_t mat2, __local int* lp)" \
          "{ return f + get(mat, 1, 1) + add2 + get(mat2, 1, 2) + lp[0]; }"
    gen = s.generated_source(s.KIND_MAP, src, ["float", "float"])
    m = re.search(r"#define SCL_EXTRA_PARAMS (.*)", gen).group(1)
    assert m.split(",")[1:] == [" float* scl_x0_d", " unsigned int scl_x0_c", " float scl_x1",
                                " int* scl_x2_d", " unsigned int scl_x2_c", " unsigned int scl_x3_o"]
    assert "#define SCL_EXTRA_ARGS , scl_x0, scl_x1, scl_x2, scl_x3" in gen
    assert "SCL_FUNC(float f" in gen  # renamed user function


def test_allpairs_extra_order_reduce_then_zip(built):
    gen = s.generated_source(s.KIND_ALLPAIRS, "float func(float x, float y, float b){ return x+y+b; }",
                             ["float", "float", "float"],
                             source2="float func(float x, float y, float a){ return x*y+a; }",
                             identity="0")
    assert "#define SCL_REDUCE_ARGS , scl_x0" in gen
    assert "#define SCL_ZIP_ARGS , scl_x1" in gen
    assert "USR_REDUCE(float x" in gen and "USR_ZIP(float x" in gen


def test_float_reduce_gets_fp64_carry_twin(built):
    gen = s.generated_source(s.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"],
                             identity="0")
    assert "double SCL_FUNC_C(double x, double y)" in gen
    assert "typedef double SCL_CARRY_T;" in gen
    gen_i = s.generated_source(s.KIND_REDUCE, "int func(int x, int y){ return x+y; }", ["int"], identity="0")
    assert "typedef SCL_TYPE_0 SCL_CARRY_T;" in gen_i


def test_compile_errors_are_reported(built):
    with pytest.raises(s.SclError) as e:
        s.compile_only(s.KIND_MAP, "float func(float f){ return f + ; }", ["float", "float"])
    assert e.value.status == s.ERR_COMPILE and "error" in e.value.message
    with pytest.raises(s.SclError) as e:
        s.compile_only(s.KIND_MAP, "float other(float f){ return f; }", ["float", "float"])
    assert e.value.status == s.ERR_COMPILE and "func" in e.value.message
    with pytest.raises(s.SclError) as e:
        s.compile_only(s.KIND_ZIP, "float func(float f){ return f; }", ["float", "float", "float"])
    assert e.value.status == s.ERR_COMPILE
    with pytest.raises(s.SclError) as e:
        s.compile_only(s.KIND_MAP, "   ", ["float", "float"])
    assert e.value.status == s.ERR_ARG


def test_custom_func_name_and_comments(built):
    src = "/* helper */ float sq(float v) { return v*v; }\n// the entry\nfloat myfn(float f) { return sq(f) + 1.0f; }"
    s.compile_only(s.KIND_MAP, src, ["float", "float"], func="myfn")


def test_every_template_kernel_waits_for_its_predecessor():
    """Skeleton kernels are launched with programmatic stream serialization,
    which is only safe when each kernel's first statement waits for the
    previous grid: every __global__ in the templates must open with
    SCL_EXTRA_SETUP, and the generated SCL_EXTRA_SETUP must begin with the
    griddepcontrol.wait of the prelude."""
    tdir = ROOT / "skelcl_gb300" / "csrc" / "templates"
    kernels = 0
    for f in sorted(tdir.glob("*.cuh")):
        text = f.read_text()
        for m in re.finditer(r"__global__", text):
            body = text.index("{", m.end())
            first = text[body + 1:body + 400].strip().splitlines()[0].strip()
            line = text[:m.start()].count("\n") + 1
            assert first.startswith("SCL_EXTRA_SETUP"), f"{f.name}:{line} opens with {first!r}"
            kernels += 1
    assert kernels >= 25
    prelude = (tdir / "prelude.cuh").read_text()
    assert re.search(r'#define SCL_GRID_DEPENDENCY_WAIT asm volatile\("griddepcontrol\.wait;"', prelude)
    prog = (ROOT / "skelcl_gb300" / "csrc" / "program.cpp").read_text()
    assert '"#define SCL_EXTRA_SETUP SCL_GRID_DEPENDENCY_WAIT "' in prog
