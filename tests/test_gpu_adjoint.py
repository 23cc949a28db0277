"""Adjoint skeletons on the GPU, through the C ABI: each gradient against the
FP64 oracle and against FP64 central finite differences of the forward
(h = 1e-3 * max(1, |x|)) on 64 seeded coordinates."""
import numpy as np
import pytest

import skelcl_gb300 as S

pytestmark = pytest.mark.gpu

MAP_D = "float dfunc(float x, float g){ return 2.0f*x*g; }"   # of x*x + 1
ZIP_D = ("float dl(float x, float y, float g){ return y*g; }\n"
         "float dr(float x, float y, float g){ return x*g; }")  # of x*y
ADD = "float func(float x, float y){ return x + y; }"
GAUSS_SRC = ("float func(input_matrix_t img, __global float* w) { float s = 0.0f;"
             " for (int dy = -5; dy <= 5; ++dy) for (int dx = -5; dx <= 5; ++dx)"
             "  s += getData(img, dx, dy) * w[(dy + 5) * 11 + (dx + 5)]; return s; }")


def dev(a):
    return S.DeviceArray.from_numpy(np.ascontiguousarray(a))


def coords(n, k=64, seed=4):
    return np.random.default_rng(seed).choice(n, size=min(k, n), replace=False)


def fd(loss, x, j):
    """FP64 central difference of loss at coordinate j (x float32, flat)."""
    h = 1e-3 * max(1.0, abs(float(x.flat[j])))
    xp, xm = x.copy(), x.copy()
    xp.flat[j] = x.flat[j] + h
    xm.flat[j] = x.flat[j] - h
    hh = (float(xp.flat[j]) - float(xm.flat[j])) / 2.0  # the step float32 actually took
    return (loss(xp) - loss(xm)) / (2.0 * hh)


# ---- Map / Zip -------------------------------------------------------------------
def test_map_adjoint(scl, orc):
    n = (1 << 20) + 3
    x = orc.uniform_f32(n, 2, -1.0, 1.0)
    g = orc.uniform_f32(n, 3, -1.0, 1.0)
    p = S.Program(S.KIND_MAP_ADJOINT, MAP_D, ["float", "float"], func="dfunc")
    dx, dg, dgx = dev(x), dev(g), S.DeviceArray(n, np.float32)
    p.launch([dx, dg, dgx], n=n)
    gx = dgx.to_numpy()
    ref = 2.0 * x.astype(np.float64) * g
    assert np.abs(gx - ref).max() <= 1e-6  # two FP32 roundings of values <= 2
    g64 = g.astype(np.float64)
    loss = lambda v: float(np.dot(g64, v.astype(np.float64) ** 2 + 1.0))
    for j in coords(n):
        assert abs(fd(loss, x, j) - gx[j]) <= 1e-5 * max(1.0, abs(gx[j])), j
    # a second contribution adds
    p.launch([dx, dg, dgx], n=n, flags=S.SHAPE_ACCUMULATE)
    assert np.array_equal(dgx.to_numpy(), gx + gx)


@pytest.mark.parametrize("which", ["both", "left", "right"])
def test_zip_adjoint(scl, orc, which):
    n = 777_777
    x = orc.uniform_f32(n, 5, -1.0, 1.0)
    y = orc.uniform_f32(n, 6, -1.0, 1.0)
    g = orc.uniform_f32(n, 7, -1.0, 1.0)
    p = S.Program(S.KIND_ZIP_ADJOINT, ZIP_D, ["float"] * 3, func="dl", func2="dr")
    dgx = S.DeviceArray(n, np.float32) if which != "right" else None
    dgy = S.DeviceArray(n, np.float32) if which != "left" else None
    p.launch([dev(x), dev(y), dev(g), dgx, dgy], n=n)
    if dgx is not None:
        assert np.array_equal(dgx.to_numpy(), y * g)
    if dgy is not None:
        assert np.array_equal(dgy.to_numpy(), x * g)
    if which == "both":
        p.launch([dev(x), dev(y), dev(g), dgx, dgy], n=n, flags=S.SHAPE_ACCUMULATE_RIGHT)
        assert np.array_equal(dgx.to_numpy(), y * g)          # overwritten
        assert np.array_equal(dgy.to_numpy(), x * g + x * g)  # added


def test_zip_adjoint_needs_right_derivative_for_right_gradient(scl):
    p = S.Program(S.KIND_ZIP_ADJOINT, "float dl(float x, float y, float g){ return y*g; }",
                  ["float"] * 3, func="dl")
    a = S.DeviceArray(16, np.float32)
    with pytest.raises(S.SclError):
        p.launch([a, a, a, None, S.DeviceArray(16, np.float32)], n=16)


def test_zip_adjoint_float4_with_extra(scl, orc):
    n = 4096
    x = orc.uniform_f32(4 * n, 8, -1.0, 1.0)
    y = orc.uniform_f32(4 * n, 9, -1.0, 1.0)
    g = orc.uniform_f32(4 * n, 10, -1.0, 1.0)
    src = ("float4 dl(float4 x, float4 y, float4 g, float a){ return a * y * g; }\n"
           "float4 dr(float4 x, float4 y, float4 g, float a){ return a * x * g; }")
    p = S.Program(S.KIND_ZIP_ADJOINT, src, ["float4"] * 3, func="dl", func2="dr")
    dgx, dgy = S.DeviceArray(4 * n, np.float32), S.DeviceArray(4 * n, np.float32)
    p.launch([dev(x), dev(y), dev(g), dgx, dgy], n=n, extra=S.value(np.float32(0.5)))
    assert np.allclose(dgx.to_numpy(), 0.5 * y * g, rtol=1e-6, atol=1e-7)
    assert np.allclose(dgy.to_numpy(), 0.5 * x * g, rtol=1e-6, atol=1e-7)


# ---- Reduce(+): broadcast; accumulation -----------------------------------------------
@pytest.mark.parametrize("dtype,code", [(np.float32, S.DTYPE_F32), (np.float64, S.DTYPE_F64)])
@pytest.mark.parametrize("n", [1, 7, 4096, 1_000_001])
def test_broadcast(scl, dtype, code, n):
    g = dev(np.array([1.25], dtype))
    out = dev(np.zeros(n + 1, dtype))
    view = out.view(1, n)  # an unaligned destination too
    S.check(S.lib().scl_adjoint_broadcast(g.ptr, out.ptr, n, code, 0))
    assert np.all(out.to_numpy()[:n] == dtype(1.25))
    S.check(S.lib().scl_adjoint_broadcast(g.ptr, view.ptr, n, code, 1))
    got = out.to_numpy()
    assert got[0] == dtype(1.25) and np.all(got[1:n] == dtype(2.5)) and got[n] == dtype(1.25)


@pytest.mark.parametrize("dtype,code", [(np.float32, S.DTYPE_F32), (np.float64, S.DTYPE_F64)])
def test_accumulate(scl, orc, dtype, code):
    n = 1_000_003
    a = orc.uniform_f32(n, 11, -1.0, 1.0).astype(dtype)
    b = orc.uniform_f32(n, 12, -1.0, 1.0).astype(dtype)
    da, db = dev(a), dev(b)
    S.check(S.lib().scl_adjoint_accumulate(da.ptr, db.ptr, n, code))
    assert np.array_equal(da.to_numpy(), a + b)


def test_reduce_sum_gradient_fd(scl, orc):
    """d/dx sum(x) = 1 for every coordinate: broadcast of the seed 1."""
    n = 100_003
    x = orc.uniform_f32(n, 13, -1.0, 1.0)
    seed = dev(np.array([1.0], np.float32))
    gx = S.DeviceArray(n, np.float32)
    S.check(S.lib().scl_adjoint_broadcast(seed.ptr, gx.ptr, n, S.DTYPE_F32, 0))
    got = gx.to_numpy()
    loss = lambda v: float(v.astype(np.float64).sum())
    for j in coords(n):
        assert abs(fd(loss, x, j) - got[j]) <= 1e-6


# ---- Scan(+): reverse scan ------------------------------------------------------------
def reverse_tol(n):
    # as the forward float scan tests: 1e-5 * (1 + sqrt(number of summed terms))
    return 1e-5 * (1.0 + np.sqrt(np.arange(n, 0, -1, dtype=np.float64)))


@pytest.mark.parametrize("inclusive", [False, True])
def test_scan_adjoint_fd(scl, orc, inclusive):
    n = (1 << 20) + 5
    x = orc.uniform_f32(n, 2, -1.0, 1.0)
    g = orc.uniform_f32(n, 3, -1.0, 1.0)
    p = S.Program(S.KIND_SCAN, ADD, ["float"], identity="0")
    dgx = S.DeviceArray(n, np.float32)
    flags = S.SHAPE_REVERSE | (S.SHAPE_INCLUSIVE if inclusive else 0)
    p.launch([dev(g), dgx], n=n, flags=flags)
    got = dgx.to_numpy().astype(np.float64)
    ref = orc.scan_f64(g, inclusive=inclusive, reverse=True)
    assert np.all(np.abs(got - ref) <= reverse_tol(n))
    g64 = g.astype(np.float64)
    loss = lambda v: float(np.dot(g64, orc.scan_f64(v, inclusive=inclusive)))
    for j in coords(n):
        assert abs(fd(loss, x, j) - got[j]) <= 1e-4 * max(1.0, abs(got[j])), j


def test_scan_adjoint_full_size(scl, orc):
    """The float scan workload at its full size (2^26, U[-1,1]): the reverse
    scan against the FP64 oracle, and against FP64 central differences of
    loss = g . Scan(x) on 64 seeded coordinates (each difference runs the
    whole FP64 forward twice)."""
    n = 1 << 26
    x = orc.uniform_f32(n, 2, -1.0, 1.0)
    g = orc.uniform_f32(n, 3, -1.0, 1.0)
    p = S.Program(S.KIND_SCAN, ADD, ["float"], identity="0")
    dgx = S.DeviceArray(n, np.float32)
    p.launch([dev(g), dgx], n=n, flags=S.SHAPE_REVERSE | S.SHAPE_INCLUSIVE)
    got = dgx.to_numpy().astype(np.float64)
    ref = orc.scan_f64(g, inclusive=True, reverse=True)
    assert np.all(np.abs(got - ref) <= reverse_tol(n))
    del ref
    g64 = g.astype(np.float64)
    loss = lambda v: float(np.dot(g64, orc.scan_f64(v, inclusive=True)))
    for j in coords(n):
        # in place: a copy of 2^26 floats per evaluation is not needed
        x0 = x[j]
        h = 1e-3 * max(1.0, abs(float(x0)))
        x[j] = x0 + h
        up, hp = loss(x), float(x[j])
        x[j] = x0 - h
        dn, hm = loss(x), float(x[j])
        x[j] = x0
        d = (up - dn) / (hp - hm)
        assert abs(d - got[j]) <= 1e-4 * max(1.0, abs(got[j])), j


# ---- MapOverlap (linear): transposed stencil ---------------------------------------------
def stencil_adjoint_gpu(fwd, R, g, w_extra, padding):
    """What the tape does: impulse-probe the transposed weights, run the
    zero-padded adjoint stencil, fold the edges for NEAREST."""
    rows, cols = g.shape
    W = 2 * R + 1
    imp = np.zeros((W, W), np.float32)
    imp[R, R] = 1.0
    ri, rz = S.DeviceArray(W * W, np.float32), S.DeviceArray(W * W, np.float32)
    fwd.launch([dev(imp), ri], rows=W, cols=W, extra=w_extra)
    fwd.launch([dev(np.zeros((W, W), np.float32)), rz], rows=W, cols=W, extra=w_extra)
    wt = (ri.to_numpy() - rz.to_numpy()).astype(np.float32)
    src = (f"float adj(input_matrix_t g, __global const float* w) {{ float s = 0.0f;"
           f" for (int dy = -{R}; dy <= {R}; ++dy) for (int dx = -{R}; dx <= {R}; ++dx)"
           f"  s += w[(dy + {R}) * {W} + (dx + {R})] * getData(g, dx, dy); return s; }}")
    adj = S.Program(S.KIND_MAPOVERLAP, src, ["float", "float"], func="adj", overlap_range=R,
                    padding=S.PAD_NEUTRAL, neutral="0.0f")
    dg, dwt, out = dev(g), dev(wt), S.DeviceArray(rows * cols, np.float32)
    adj.launch([dg, out], rows=rows, cols=cols, extra=S.buffer(dwt))
    if padding == S.PAD_NEAREST:
        S.check(S.lib().scl_mapoverlap_adjoint_edges(dg.ptr, dwt.ptr, out.ptr, rows, cols, R))
    return out.to_numpy().reshape(rows, cols), wt


@pytest.mark.parametrize("shape", [(300, 257), (64, 1000), (1000, 3), (1, 50)])
@pytest.mark.parametrize("padding", [S.PAD_NEUTRAL, S.PAD_NEAREST])
def test_mapoverlap_adjoint(scl, orc, shape, padding):
    rows, cols = shape
    img = orc.uniform_f32(rows * cols, 5, 0.0, 255.0).reshape(rows, cols)
    g = orc.uniform_f32(rows * cols, 6, -1.0, 1.0).reshape(rows, cols)
    w = orc.gaussian_weights(5, 2.0)
    dw = dev(w)
    fwd = S.Program(S.KIND_MAPOVERLAP, GAUSS_SRC, ["float", "float"], overlap_range=5,
                    padding=padding, neutral="0")
    got, wt = stencil_adjoint_gpu(fwd, 5, g, S.buffer(dw), padding)
    assert np.allclose(wt.reshape(11, 11), w.reshape(11, 11)[::-1, ::-1], atol=1e-7)
    ref = orc.stencil_adjoint_f64(g, 5, w, padding)
    # FP32 sums of <= 121 products per position; NEAREST corners fold up to 36 positions
    assert np.abs(got - ref).max() <= 2e-5 * max(1.0, np.abs(ref).max())
    g64 = g.astype(np.float64)
    loss = lambda v: float((g64 * orc.stencil_f64(v.reshape(rows, cols), 5, w, padding, 0.0)).sum())
    edge = [0, cols - 1, (rows - 1) * cols, rows * cols - 1]
    for j in list(coords(rows * cols, 60, seed=7)) + edge:
        assert abs(fd(loss, img.ravel(), j) - got.flat[j]) <= 1e-3 * max(1.0, abs(got.flat[j])), j


@pytest.mark.parametrize("padding", [S.PAD_NEUTRAL, S.PAD_NEAREST])
def test_mapoverlap_adjoint_full_size(scl, orc, padding):
    """The stencil workload at its full size: 8192 x 8192 U[0,255], 11 x 11
    Gaussian (sigma 2), loss = sum(out * w) with w U[-1,1].  The transposed
    stencil against the FP64 oracle's adjoint, and against FP64 central
    differences on 64 seeded pixels plus the four corners.  Moving pixel j
    changes only the outputs within R of it, which read inputs within 2R, so
    each difference evaluates the FP64 forward on that neighbourhood: the
    other outputs are identical in both evaluations."""
    rows = cols = 8192
    R = 5
    img = orc.uniform_f32(rows * cols, 5, 0.0, 255.0).reshape(rows, cols)
    g = orc.uniform_f32(rows * cols, 6, -1.0, 1.0).reshape(rows, cols)
    w = orc.gaussian_weights(R, 2.0)
    fwd = S.Program(S.KIND_MAPOVERLAP, GAUSS_SRC, ["float", "float"], overlap_range=R,
                    padding=padding, neutral="0")
    got, _ = stencil_adjoint_gpu(fwd, R, g, S.buffer(dev(w)), padding)
    ref = orc.stencil_adjoint_f64(g, R, w, padding)
    assert np.abs(got - ref).max() <= 2e-5 * max(1.0, np.abs(ref).max())
    del ref

    def local_loss(r, c):
        r0, r1 = max(0, r - 2 * R), min(rows, r + 2 * R + 1)
        c0, c1 = max(0, c - 2 * R), min(cols, c + 2 * R + 1)
        o0, o1 = max(0, r - R), min(rows, r + R + 1)
        p0, p1 = max(0, c - R), min(cols, c + R + 1)
        sub = np.ascontiguousarray(img[r0:r1, c0:c1])
        gbox = g[o0:o1, p0:p1].astype(np.float64)

        def loss(v):
            # the neighbourhood's own border is an image border wherever it
            # was clipped; elsewhere the box's outputs read only inside it
            out = orc.stencil_f64(v.reshape(sub.shape), R, w, padding, 0.0)
            return float((gbox * out[o0 - r0:o1 - r0, p0 - c0:p1 - c0]).sum())
        return sub, (r - r0) * (c1 - c0) + (c - c0), loss

    pix = [(int(j) // cols, int(j) % cols) for j in coords(rows * cols, 64, seed=7)]
    pix += [(0, 0), (0, cols - 1), (rows - 1, 0), (rows - 1, cols - 1)]
    for r, c in pix:
        sub, j, loss = local_loss(r, c)
        d = fd(loss, sub.ravel(), j)
        assert abs(d - got[r, c]) <= 1e-3 * max(1.0, abs(got[r, c])), (r, c)


# ---- AllPairs (x*y, +): two AllPairs with transposed operands -----------------------------
ZIP = "float func(float x, float y){ return x*y; }"


@pytest.mark.parametrize("variant", [S.VARIANT_AUTO, S.VARIANT_SIMT])
@pytest.mark.parametrize("shape", [(256, 192, 384), (300, 129, 257)])
def test_allpairs_adjoint(scl, orc, variant, shape):
    M, K, N = shape
    A = orc.normal_f32(M * K, 7).reshape(M, K)
    B = orc.normal_f32(K * N, 8).reshape(K, N)
    G = orc.normal_f32(M * N, 9).reshape(M, N)
    p = S.Program(S.KIND_ALLPAIRS, ADD, ["float"] * 3, source2=ZIP, identity="0")
    dA_, dB_, dG_ = dev(A), dev(B), dev(G)
    dA, dB = S.DeviceArray(M * K, np.float32), S.DeviceArray(K * N, np.float32)
    t = S.Tuning(variant=variant)
    p.launch([dG_, dB_, dA], rows=M, cols=K, dim=N, flags=S.SHAPE_TRANS_RIGHT, tuning=t)
    p.launch([dA_, dG_, dB], rows=K, cols=N, dim=M, flags=S.SHAPE_TRANS_LEFT, tuning=t)
    G64, A64, B64 = G.astype(np.float64), A.astype(np.float64), B.astype(np.float64)
    refA, refB = G64 @ B64.T, A64.T @ G64
    errA = np.abs(dA.to_numpy().reshape(M, K) - refA).max() / np.abs(refA).max()
    errB = np.abs(dB.to_numpy().reshape(K, N) - refB).max() / np.abs(refB).max()
    assert errA <= 1e-5 and errB <= 1e-5, (errA, errB)
    # FD of L = sum(G * (A B)) in FP64 at sampled entries of A and B
    loss_a = lambda v: float((G64 * (v.reshape(M, K).astype(np.float64) @ B64)).sum())
    loss_b = lambda v: float((G64 * (A64 @ v.reshape(K, N).astype(np.float64))).sum())
    ga, gb = dA.to_numpy(), dB.to_numpy()
    for j in coords(M * K, 16):
        assert abs(fd(loss_a, A.ravel(), j) - ga[j]) <= 1e-3 * max(1.0, abs(ga[j]))
    for j in coords(K * N, 16):
        assert abs(fd(loss_b, B.ravel(), j) - gb[j]) <= 1e-3 * max(1.0, abs(gb[j]))
