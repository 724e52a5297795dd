"""GPU parity: the engine against the oracle's FP64 direct sums (the reference
test suite's check, test/cuda/cufinufft{1,2,3}d_test.cu) and against the
oracle's FP64 restatement of the same algorithm with the same kernel (PSWF by
default, ES on request): a much tighter check of the kernels themselves, and
the bar for the error against the direct sum (the restatement's error plus
the plan precision's rounding). All calls go through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (dim, modes row-major, M) -- sizes of the reference's GPU test matrix
# (test/cuda/CMakeLists.txt:26-250), 3D enlarged so every spread path is exercised
CASES = {1: ((2000,), 4000), 2: ((100, 200), 20000), 3: ((10, 12, 16), 5000)}
# requested tol -> checktol of the reference suite (test/cuda/CMakeLists.txt:239-250)
PREC = {"complex64": (1e-4, 2e-3), "complex128": (1e-12, 1e-11)}


def _torch():
    import torch

    return torch


def _dev(a):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _pts(rng, dim, M, rdt):
    return rng.uniform(-np.pi, np.pi, (dim, M)).astype(rdt)


def _cx(rng, shape, cdt):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(cdt)


def _oracle_pts(pts):
    """python axis order (slowest first) -> oracle order (fastest first)"""
    return [p.astype(np.float64) for p in pts[::-1]]


def _kernel(plan):
    """the oracle's name of the plan's kernel form"""
    return "pswf" if plan.info().kernel_form == 2 else "es"


# floor of a single-precision result's error against the FP64 direct sum (the
# float arithmetic of spread, FFT and deconvolution: ~3e-6 measured for the
# CPU restatement in single precision on 2D grids at tol 1e-6), and of a double one
ROUND = {"complex64": 5e-6, "complex128": 5e-13}


def _bound(same_err, dtype):
    """accuracy bar for the engine: the error of the same algorithm in FP64 (the
    oracle's restatement, the kernel truncation alone) with 25% slack, plus the
    rounding floor of the plan's precision"""
    return 1.25 * same_err + ROUND[dtype]


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("method", [0, 1, 2, 3])
@pytest.mark.parametrize("form", [0, 1])
def test_type1(oracle, dtype, dim, method, form):
    """type 1 against the FP64 direct sum at the suite's checktol and against the
    same algorithm in FP64 (default PSWF kernel, form 0, and the ES kernel)"""
    import finufft_gb300 as fg

    tol, checktol = PREC[dtype]
    nm, M = CASES[dim]
    rng = np.random.default_rng(100 + dim)
    rdt = np.float32 if dtype == "complex64" else np.float64
    pts = _pts(rng, dim, M, rdt)
    c = _cx(rng, M, dtype)
    plan = fg.Plan(1, nm, eps=tol, dtype=dtype, isign=1, gpu_method=method, kernel_form=form)
    assert plan.info().kernel_form == (2 if form == 0 else 1)
    plan.setpts(*[_dev(p) for p in pts])
    f = plan.execute(_dev(c)).cpu().numpy()
    assert f.shape == nm
    ref = oracle.dirft1(_oracle_pts(pts), c, 1, nm[::-1]).reshape(nm)
    assert oracle.rel_l2(f, ref) < checktol
    same = oracle.nufft_es(1, _oracle_pts(pts), c, 1, tol, n_modes=nm[::-1],
                           is_float=dtype == "complex64", kernel=_kernel(plan)).reshape(nm)
    assert oracle.rel_l2(f, same) < (3e-5 if dtype == "complex64" else 1e-11)
    assert oracle.rel_l2(f, ref) < _bound(oracle.rel_l2(same, ref), dtype)


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("form", [0, 1])
def test_type2(oracle, dtype, dim, form):
    import finufft_gb300 as fg

    tol, checktol = PREC[dtype]
    nm, M = CASES[dim]
    rng = np.random.default_rng(200 + dim)
    rdt = np.float32 if dtype == "complex64" else np.float64
    pts = _pts(rng, dim, M, rdt)
    fk = _cx(rng, nm, dtype)
    plan = fg.Plan(2, nm, eps=tol, dtype=dtype, kernel_form=form)
    plan.setpts(*[_dev(p) for p in pts])
    c = plan.execute(_dev(fk)).cpu().numpy()
    ref = oracle.dirft2(_oracle_pts(pts), fk.ravel(), -1, nm[::-1])
    assert oracle.rel_l2(c, ref) < checktol
    same = oracle.nufft_es(2, _oracle_pts(pts), fk, -1, tol, n_modes=nm[::-1],
                           is_float=dtype == "complex64", kernel=_kernel(plan))
    assert oracle.rel_l2(c, same) < (3e-5 if dtype == "complex64" else 1e-11)
    assert oracle.rel_l2(c, ref) < _bound(oracle.rel_l2(same, ref), dtype)


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("form", [0, 1])
def test_type3(oracle, dtype, dim, form):
    import finufft_gb300 as fg

    tol = 1e-4 if dtype == "complex64" else 1e-9
    checktol = 2e-3 if dtype == "complex64" else 1e-7
    rng = np.random.default_rng(300 + dim)
    rdt = np.float32 if dtype == "complex64" else np.float64
    M, N = 3000, 1000
    half = [2.0, 3.0, 1.5][:dim]
    pts = np.stack([rng.uniform(-h, h, M) + 0.3 for h in half]).astype(rdt)
    freq = np.stack([rng.uniform(-s, s, N) for s in [40.0, 25.0, 30.0][:dim]]).astype(rdt)
    c = _cx(rng, M, dtype)
    plan = fg.Plan(3, dim, eps=tol, dtype=dtype, kernel_form=form)
    plan.setpts(*[_dev(p) for p in pts], **dict(zip('stu', [_dev(s) for s in freq])))
    f = plan.execute(_dev(c)).cpu().numpy()
    ref = oracle.dirft3(_oracle_pts(pts), c, 1, _oracle_pts(freq))
    assert oracle.rel_l2(f, ref) < checktol
    same = oracle.nufft_es(3, _oracle_pts(pts), c, 1, tol, ss=_oracle_pts(freq),
                           is_float=dtype == "complex64", kernel=_kernel(plan))
    # (double: both sit at errors near tol on either side of the direct sum)
    assert oracle.rel_l2(f, same) < (3e-5 if dtype == "complex64" else 3 * tol)
    if _kernel(plan) == "es":
        assert oracle.rel_l2(f, ref) < _bound(oracle.rel_l2(same, ref), dtype)
    else:
        # the CPU library's kernel: the accuracy contract against its algorithm
        # (the CPU restatement at the same upsampling factor and precision)
        cpu = oracle.CpuPlan(3, dim, 1, tol, dtype=dtype, sigma=plan.info().upsampfac)
        cpu.setpts(_oracle_pts(pts), _oracle_pts(freq))
        cpu_err = oracle.rel_l2(cpu.execute(c), ref)
        assert oracle.rel_l2(f, ref) < 2 * cpu_err


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("keys", [0, 2])
def test_sort_bit_exact(oracle, dtype, dim, keys):
    """setpts' device permutation and bin-local coordinates equal the host
    replica (stable counting sort with the engine's fold) bit for bit, with the
    engine's keys (bin and support start cell, 0) and with the reference's bin
    ordering (bin index x fastest, input order inside a bin, 2)."""
    import ctypes

    import finufft_gb300 as fg

    rdt = np.float32 if dtype == "complex64" else np.float64
    rng = np.random.default_rng(400 + dim)
    M = 30000
    pts = _pts(rng, dim, M, rdt)
    pts[:, :50] = rdt(np.pi)       # exactly on the seam
    pts[:, 50:100] = rdt(-np.pi)
    pts[0, 100:200] = rdt(1e4)     # far outside [-pi, pi): folded
    # a cluster: many points in one bin
    pts[:, 200:5200] = (0.01 * rng.standard_normal((dim, 5000))).astype(rdt)
    nm = CASES[dim][0]
    # even and odd kernel widths (odd ones sort by half cell)
    for tol in ((1e-5, 1e-6) if rdt == np.float32 else (1e-10, 1e-12)):
        plan = fg.Plan(1, nm, eps=tol, dtype=dtype, sort_keys=keys)
        plan.setpts(*[_dev(p) for p in pts])
        info = plan.info()
        perm = np.zeros(M, dtype=np.int32)
        loc = np.zeros(dim * M, dtype=rdt)
        fn = getattr(plan._lib, plan._pfx + "_get_sort")
        assert fn(plan._plan, perm.ctypes.data, loc.ctypes.data) == 0
        # the coordinates as the engine received them (float32 for complex64
        # plans, which take the single-precision fold), fastest axis first
        hperm, hloc = oracle.bin_sort([np.ascontiguousarray(p) for p in pts[::-1]],
                                      list(info.nf)[:dim], list(info.bins)[:dim], loc_dtype=rdt,
                                      ns=info.ns, bin_only=keys == 2)
        np.testing.assert_array_equal(perm, hperm)
        np.testing.assert_array_equal(loc.reshape(dim, M), hloc)


def _clustered(rng, dim, M, rdt):
    """half uniform, half in two tight clusters (long same-cell runs, dense bins)"""
    u = rng.uniform(-np.pi, np.pi, (dim, M - M // 2))
    cen = rng.uniform(-np.pi, np.pi, (2, dim, 1))
    k = rng.integers(0, 2, M // 2)
    cl = cen[k, :, 0].T + 0.05 * rng.standard_normal((dim, M // 2))
    cl = np.remainder(cl + np.pi, 2 * np.pi) - np.pi
    return np.concatenate([u, cl], axis=1).astype(rdt)


@pytest.mark.parametrize("dtype,tol", [("complex64", 1e-5), ("complex64", 1e-3),
                                       ("complex64", 3e-7), ("complex128", 1e-7)])
@pytest.mark.parametrize("bins", [None, (12, 4, 8)])
def test_spread_variants_3d(oracle, dtype, tol, bins):
    """3D type 1 through every tiled spread variant (0 per-point atomics, 1
    exclusive-warp tiles, 2 warp-aggregated runs, 3 runs with x slack): each
    equals the FP64 direct sum, and all agree with variant 0 to rounding."""
    import finufft_gb300 as fg

    rdt = np.float32 if dtype == "complex64" else np.float64
    rng = np.random.default_rng(77)
    nm, M, ntr = (14, 18, 22), 6000, 3
    pts = _clustered(rng, 3, M, rdt)
    c = _cx(rng, (ntr, M), dtype)
    kw = {} if bins is None else dict(gpu_binsizex=bins[0], gpu_binsizey=bins[1],
                                      gpu_binsizez=bins[2])
    outs = {}
    for v in (0, 1, 2, 3):
        plan = fg.Plan(1, nm, n_trans=ntr, eps=tol, dtype=dtype, isign=1, spread_variant=v, **kw)
        plan.setpts(*[_dev(p) for p in pts])
        outs[v] = plan.execute(_dev(c)).cpu().numpy()
        outs[v, "used"] = plan.info().spread_variant
    ref = oracle.dirft1(_oracle_pts(pts), c[1], 1, nm[::-1])
    same = oracle.nufft_es(1, _oracle_pts(pts), c[1], 1, tol, n_modes=nm[::-1],
                           is_float=dtype == "complex64", kernel=_kernel(plan))
    bound = _bound(oracle.rel_l2(same, ref), dtype)
    for v in (0, 1, 2, 3):
        got = outs[v][1].ravel()
        assert oracle.rel_l2(got, ref) < bound, (v, outs[v, "used"])
        if v:
            assert oracle.rel_l2(outs[v], outs[0]) < (2e-5 if dtype == "complex64" else 1e-12), v
    assert outs[3, "used"] == 3 or tol < 1e-6  # width 8 and below take variant 3


@pytest.mark.parametrize("tol", [1e-3, 1e-5])
@pytest.mark.parametrize("scale", [1.0, 1e25, 1e-20, 1e31])
def test_fixed_point_tile(oracle, tol, scale):
    """single-precision 3D spread with the int32 fixed-point tile (the default
    for ns <= 6) against the float tile and the FP64 direct sum, on clustered
    points with a few strong sources among weak ones, at strength scales far
    from 1 (the per-subproblem power-of-two scale follows them; at 1e31 the
    subproblems' strength sums exceed 2^100 and they add floats instead)"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(101)
    nm, M, ntr = (16, 20, 24), 8000, 2
    pts = _clustered(rng, 3, M, np.float32)
    c = _cx(rng, (ntr, M), "complex64")
    c[0, :50] *= 300.0  # a few strong sources among weak ones
    c = (c * np.float32(scale)).astype(np.complex64)
    outs = {}
    for ft in (0, 1):
        plan = fg.Plan(1, nm, n_trans=ntr, eps=tol, isign=1, spread_float_tile=ft)
        assert plan.info().spread_variant == 3
        plan.setpts(*[_dev(p) for p in pts])
        outs[ft] = plan.execute(_dev(c)).cpu().numpy()
    for k in range(ntr):
        ck = c[k].astype(np.complex128) / scale
        ref = oracle.dirft1(_oracle_pts(pts), ck, 1, nm[::-1])
        same = oracle.nufft_es(1, _oracle_pts(pts), ck, 1, tol, n_modes=nm[::-1],
                               kernel=_kernel(plan))
        got = outs[0][k].ravel().astype(np.complex128) / scale
        assert oracle.rel_l2(got, ref) < _bound(oracle.rel_l2(same, ref), "complex64"), k
        # the two tiles differ by float rounding only
        alt = outs[1][k].ravel().astype(np.complex128) / scale
        assert oracle.rel_l2(got, alt) < 3e-6, k


def test_fixed_point_tile_wide(oracle):
    """spread_float_tile=2 uses the fixed-point tile at widths 7 and 8 as well
    (a speed/accuracy trade): still within the suite's bound of the FP64 sum"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(103)
    nm, M = (16, 20, 24), 8000
    pts = _clustered(rng, 3, M, np.float32)
    c = _cx(rng, M, "complex64")
    ref = oracle.dirft1(_oracle_pts(pts), c.astype(np.complex128), 1, nm[::-1])
    for tol, ns in ((1e-6, 7), (1.2e-7, 8)):
        plan = fg.Plan(1, nm, eps=tol, isign=1, spread_float_tile=2)
        plan.setpts(*[_dev(p) for p in pts])
        info = plan.info()
        assert info.ns == ns and info.spread_fixed == 1
        got = plan.execute(_dev(c)).cpu().numpy().ravel()
        assert oracle.rel_l2(got, ref) < 1e-5, ns


def test_fixed_point_tile_nan_and_type3(oracle):
    """a NaN strength reaches the output as with float atomics (its subproblem
    keeps the float tile); type 3 spreads c times the pre-phase through the
    fixed-point tile"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(102)
    M = 4000
    pts = _clustered(rng, 3, M, np.float32)
    c = _cx(rng, M, "complex64")
    c[17] = np.nan
    plan = fg.Plan(1, (12, 12, 12), eps=1e-5, isign=1)
    plan.setpts(*[_dev(p) for p in pts])
    f = plan.execute(_dev(c)).cpu().numpy()
    assert np.isnan(f).any()
    s = rng.uniform(-8, 8, (3, 600)).astype(np.float32)
    c[17] = 1.0
    outs = {}
    for ft in (0, 1):
        p3 = fg.Plan(3, 3, eps=1e-5, isign=1, spread_float_tile=ft)
        p3.setpts(*[_dev(p) for p in pts], s=_dev(s[0]), t=_dev(s[1]), u=_dev(s[2]))
        outs[ft] = p3.execute(_dev(c)).cpu().numpy().ravel()
    ref = oracle.dirft3(_oracle_pts(pts), c.astype(np.complex128), 1, _oracle_pts(s))
    assert oracle.rel_l2(outs[0], ref) < 2e-4
    assert oracle.rel_l2(outs[0], outs[1]) < 3e-6


@pytest.mark.parametrize("v", [2, 3])
def test_spread_variants_type3(oracle, v):
    """type 3 (spread with the pre-phase factor) through the warp-aggregated variants"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(78)
    M, K = 5000, 400
    x = _clustered(rng, 3, M, np.float32)
    s = rng.uniform(-12, 12, (3, K)).astype(np.float32)
    c = _cx(rng, M, "complex64")
    plan = fg.Plan(3, 3, eps=1e-5, dtype="complex64", isign=1, spread_variant=v)
    plan.setpts(*[_dev(a) for a in x], s=_dev(s[0]), t=_dev(s[1]), u=_dev(s[2]))
    f = plan.execute(_dev(c)).cpu().numpy()
    ref = oracle.dirft3(_oracle_pts(x), c, 1, _oracle_pts(s))
    assert oracle.rel_l2(f.ravel(), ref) < 2e-4


@pytest.mark.parametrize("dim,dtype", [(2, "complex64"), (3, "complex64"), (2, "complex128"),
                                       (3, "complex128")])
def test_type2_tile_rounds(oracle, dim, dtype):
    """type 2 with 11 vectors (the tile-staged interpolation loads up to 8
    transforms' tiles per round, so several rounds run), clustered points;
    every vector equals its FP64 direct sum"""
    import finufft_gb300 as fg

    rdt = np.float32 if dtype == "complex64" else np.float64
    tol = 1e-5 if dtype == "complex64" else 1e-11
    rng = np.random.default_rng(90 + dim)
    nm = (40, 36) if dim == 2 else (12, 14, 10)
    M, ntr = 3000, 11
    pts = _clustered(rng, dim, M, rdt)
    fk = _cx(rng, (ntr,) + nm, dtype)
    plan = fg.Plan(2, nm, n_trans=ntr, eps=tol, dtype=dtype, isign=-1)
    plan.setpts(*[_dev(p) for p in pts])
    c = plan.execute(_dev(fk)).cpu().numpy()
    for k in (0, 5, 10):
        ref = oracle.dirft2(_oracle_pts(pts), fk[k].ravel(), -1, nm[::-1])
        same = oracle.nufft_es(2, _oracle_pts(pts), fk[k], -1, tol, n_modes=nm[::-1],
                               is_float=dtype == "complex64", kernel=_kernel(plan))
        assert oracle.rel_l2(c[k], ref) < _bound(oracle.rel_l2(same, ref), dtype), k


def test_type3_adjoint_tile(oracle):
    """the adjoint of type 3 interpolates with a post factor through the tile kernel"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(95)
    M, K = 3000, 500
    x = _clustered(rng, 3, M, np.float64)
    s = rng.uniform(-10, 10, (3, K))
    f = _cx(rng, K, "complex128")
    plan = fg.Plan(3, 3, eps=1e-10, dtype="complex128", isign=1)
    plan.setpts(*[_dev(a) for a in x], s=_dev(s[0]), t=_dev(s[1]), u=_dev(s[2]))
    c = plan.execute_adjoint(_dev(f)).cpu().numpy().ravel()
    # adjoint of f_k = sum_j c_j e^{+i s_k x_j} is c_j = sum_k f_k e^{-i s_k x_j}
    ref = oracle.dirft3(_oracle_pts(s), f, -1, _oracle_pts(x))
    assert oracle.rel_l2(c, ref) < 1e-8


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_type1_cell_edge_points(oracle, dim):
    """Float coordinates on, and one float step either side of, fine-grid cell
    edges (where the single-precision fold's rounding is decided), including a
    coordinate 1e-8 cells below an edge: every point must land within rounding
    of its true position (one point a cell off would put the error near 1e-2)."""
    import finufft_gb300 as fg

    rng = np.random.default_rng(60 + dim)
    nm = {1: (100,), 2: (40, 32), 3: (16, 20, 12)}[dim]
    plan = fg.Plan(1, nm, eps=1e-5, dtype="complex64", isign=1)
    nf = list(plan.info().nf)[:dim][::-1]  # row-major axis order (slowest first)
    M = 3000
    pts = []
    for d in range(dim):
        j = rng.integers(0, nf[d] + 1, M)
        e = (2 * np.pi * (j / nf[d] - 0.5)).astype(np.float32)
        step = rng.integers(-1, 2, M)
        e = np.where(step > 0, np.nextafter(e, np.float32(9)),
                     np.where(step < 0, np.nextafter(e, np.float32(-9)), e)).astype(np.float32)
        pts.append(e)
    pts = np.array(pts)
    pts[0, :5] = np.uint32([3158904795]).view(np.float32)[0]
    c = _cx(rng, M, "complex64")
    plan.setpts(*[_dev(p) for p in pts])
    f = plan.execute(_dev(c)).cpu().numpy()
    ref = oracle.dirft1(_oracle_pts(pts), c, 1, nm[::-1]).reshape(nm)
    assert oracle.rel_l2(f, ref) < 1e-4


@pytest.mark.parametrize("dtype,tol", [("complex64", 1e-5), ("complex64", 1e-6),
                                       ("complex128", 1e-12)])
def test_spread_variants_2d(oracle, dtype, tol):
    """2D type 1 through the tiled spread variants (0 per-point atomics, 1 one
    warp per tile with plain read-modify-writes, 2 eight warps with runs added
    by atomics): each equals the FP64 direct sum, all agree to rounding."""
    import finufft_gb300 as fg

    rdt = np.float32 if dtype == "complex64" else np.float64
    rng = np.random.default_rng(88)
    nm, M, ntr = (60, 44), 20000, 2
    pts = _clustered(rng, 2, M, rdt)
    c = _cx(rng, (ntr, M), dtype)
    outs = {}
    for v in (0, 1, 2):
        plan = fg.Plan(1, nm, n_trans=ntr, eps=tol, dtype=dtype, isign=1, spread_variant=v)
        plan.setpts(*[_dev(p) for p in pts])
        outs[v] = plan.execute(_dev(c)).cpu().numpy()
        assert plan.info().spread_variant == v
    ref = oracle.dirft1(_oracle_pts(pts), c[1], 1, nm[::-1])
    same = oracle.nufft_es(1, _oracle_pts(pts), c[1], 1, tol, n_modes=nm[::-1],
                           is_float=dtype == "complex64", kernel=_kernel(plan))
    bound = _bound(oracle.rel_l2(same, ref), dtype)
    for v in (0, 1, 2):
        assert oracle.rel_l2(outs[v][1].ravel(), ref) < bound, v
        if v:
            assert oracle.rel_l2(outs[v], outs[0]) < (2e-5 if dtype == "complex64" else 1e-12), v


@pytest.mark.parametrize("tol", [1e-7, 1e-9, 1e-12, 1e-14])
@pytest.mark.parametrize("scale", [1.0, 1e20, 1e200, 1e-200, 1e-290])
def test_fp64_fixed_point_tile(oracle, tol, scale):
    """double-precision 3D spread with the int64 fixed-point tile and integer
    products (variant 4, the default for widths above 5) against the
    double-atomic tile (variant 0) and the FP64 direct sum, on clustered points
    at strength scales the tile's power-of-two scale covers (1 to 1e-200) and
    one where a subproblem's sum needs a scale beyond 2^1000 and falls back to
    double atomics (1e-290)"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(104)
    nm, M = (14, 16, 12), 6000
    pts = _clustered(rng, 3, M, np.float64)
    c = _cx(rng, M, "complex128") * scale
    c[:40] *= 500.0  # strong sources among weak ones
    outs = {}
    for v in (-1, 0):
        plan = fg.Plan(1, nm, eps=tol, dtype="complex128", isign=1, spread_variant=v)
        outs[v, "used"] = plan.info().spread_variant
        plan.setpts(*[_dev(p) for p in pts])
        outs[v] = plan.execute(_dev(c)).cpu().numpy().ravel() / scale
    assert outs[-1, "used"] == (4 if plan.info().ns > 5 else 3)
    assert outs[0, "used"] == 0
    assert oracle.rel_l2(outs[-1], outs[0]) < 1e-13
    ref = oracle.dirft1(_oracle_pts(pts), c / scale, 1, nm[::-1])
    same = oracle.nufft_es(1, _oracle_pts(pts), c / scale, 1, tol, n_modes=nm[::-1],
                           is_float=False, kernel=_kernel(plan))
    assert oracle.rel_l2(outs[-1], ref) < _bound(oracle.rel_l2(same, ref), "complex128")


def test_fp64_fixed_point_tile_nan():
    """a NaN strength reaches the output (its subproblem sums doubles)"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(105)
    pts = _clustered(rng, 3, 3000, np.float64)
    c = _cx(rng, 3000, "complex128")
    c[7] = np.nan
    plan = fg.Plan(1, (12, 12, 12), eps=1e-12, dtype="complex128", isign=1)
    assert plan.info().spread_variant == 4
    plan.setpts(*[_dev(p) for p in pts])
    assert np.isnan(plan.execute(_dev(c)).cpu().numpy()).any()


@pytest.mark.parametrize("dim,dtype", [(2, "complex64"), (3, "complex64"), (2, "complex128"),
                                       (3, "complex128")])
@pytest.mark.parametrize("ntr", [1, 3, 8])
def test_interp_modes_agree(oracle, dim, dtype, ntr):
    """type 2 through the three interpolation schedules -- per-point gather (1),
    block-loaded tiles (2) and TMA-copied tiles with two buffers (3) -- on
    clustered points with subproblems larger than one pass of the block
    (maxsub 4096) and tiles on the periodic boundary: the same values to
    rounding, and the FP64 direct sum within the bar; no bounded wait gave up"""
    import ctypes

    import finufft_gb300 as fg

    rdt = np.float32 if dtype == "complex64" else np.float64
    tol = 1e-5 if dtype == "complex64" else 1e-11
    rng = np.random.default_rng(120 + dim + ntr)
    nm = (60, 52) if dim == 2 else (20, 18, 22)
    M = 30000
    pts = _clustered(rng, dim, M, rdt)
    pts[:, :200] = rdt(np.pi) - rdt(1e-3) * rng.random((dim, 200)).astype(rdt)  # seam tiles
    fk = _cx(rng, (ntr,) + nm, dtype)
    outs = {}
    for mode in (1, 2, 3):
        plan = fg.Plan(2, nm, n_trans=ntr, eps=tol, dtype=dtype, isign=-1, interp_mode=mode,
                       gpu_maxsubprobsize=4096, gpu_maxbatchsize=ntr)
        plan.setpts(*[_dev(p) for p in pts])
        outs[mode] = plan.execute(_dev(fk)).cpu().numpy().reshape(ntr, M)
    lib = fg.load_library()
    code = ctypes.c_int(-1)
    assert lib.gbnufft_device_error(0, ctypes.byref(code)) == 0 and code.value == 0
    agree = 2e-6 if dtype == "complex64" else 1e-13
    assert oracle.rel_l2(outs[3], outs[1]) < agree
    assert oracle.rel_l2(outs[2], outs[1]) < agree
    k = ntr - 1
    ref = oracle.dirft2(_oracle_pts(pts), fk[k].ravel(), -1, nm[::-1])
    same = oracle.nufft_es(2, _oracle_pts(pts), fk[k], -1, tol, n_modes=nm[::-1],
                           is_float=dtype == "complex64", kernel=_kernel(plan))
    assert oracle.rel_l2(outs[3][k], ref) < _bound(oracle.rel_l2(same, ref), dtype)


@pytest.mark.parametrize("dtype,tol", [("complex64", 1e-5), ("complex128", 1e-12)])
@pytest.mark.parametrize("ty", [1, 2])
def test_reference_bin_ordering_transforms(oracle, dtype, tol, ty):
    """3D plans sorted in the reference's bin ordering (sort_keys = 2, no
    support-cell refinement inside a bin) give the default plan's result to
    rounding and the FP64 direct sum within the bar"""
    import finufft_gb300 as fg

    rdt = np.float32 if dtype == "complex64" else np.float64
    rng = np.random.default_rng(108 + ty)
    nm, M = (14, 16, 12), 8000
    pts = _clustered(rng, 3, M, rdt)
    data = _cx(rng, M if ty == 1 else nm, dtype)
    outs = []
    for keys in (0, 2):
        plan = fg.Plan(ty, nm, eps=tol, dtype=dtype, isign=1 if ty == 1 else -1, sort_keys=keys)
        plan.setpts(*[_dev(p) for p in pts])
        outs.append(plan.execute(_dev(data)).cpu().numpy().ravel())
    # the orderings flush different register runs into the fixed-point tile,
    # each rounded to at most 2^-29 of its subproblem's strength sum
    assert oracle.rel_l2(outs[1], outs[0]) < (5e-6 if dtype == "complex64" else 1e-13)
    if ty == 1:
        ref = oracle.dirft1(_oracle_pts(pts), data, 1, nm[::-1])
        same = oracle.nufft_es(1, _oracle_pts(pts), data, 1, tol, n_modes=nm[::-1],
                               is_float=dtype == "complex64", kernel=_kernel(plan))
    else:
        ref = oracle.dirft2(_oracle_pts(pts), data.ravel(), -1, nm[::-1])
        same = oracle.nufft_es(2, _oracle_pts(pts), data, -1, tol, n_modes=nm[::-1],
                               is_float=dtype == "complex64", kernel=_kernel(plan))
    assert oracle.rel_l2(outs[1], ref) < _bound(oracle.rel_l2(np.ravel(same), ref), dtype)
