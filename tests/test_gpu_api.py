"""GPU tests of the drop-in API: error codes that need the device
(test/cuda/test_makeplan.c), many-vector batches, mode ordering,
spread/interp-only mode, adjoints, the host-pointer finufft_* interface, the
simple interfaces, CUDA-graph replay and edge cases."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _cx(rng, shape, dt="complex64"):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dt)


def _mk(engine, pfx, ty, dim, modes, ntr=1, tol=1e-5, opts=None):
    p = ctypes.c_void_p()
    m = (ctypes.c_int64 * 3)(*modes)
    ier = getattr(engine, pfx + "_makeplan")(ty, dim, m, 1, ntr, tol, ctypes.byref(p),
                                             ctypes.byref(opts) if opts else None)
    if ier == 0:
        getattr(engine, pfx + "_destroy")(p)
    return ier


def test_makeplan_error_codes(engine):
    from finufft_gb300 import _lib

    N = (10, 20, 15)
    for dim in (1, 2, 3):
        assert _mk(engine, "cufinufftf", 1, dim, N) == 0
        assert _mk(engine, "cufinufftf", 4, dim, N) == 10  # FINUFFT_ERR_TYPE_NOTVALID
        assert _mk(engine, "cufinufftf", 1, dim, N, ntr=0) == 9  # FINUFFT_ERR_NTRANS_NOTVALID
    assert _mk(engine, "cufinufftf", 1, 1, (10, 0, 15)) == 0  # higher dims ignored
    o = _lib.default_opts()
    o.upsampfac, o.gpu_kerevalmeth = 0.9, 1
    assert _mk(engine, "cufinufftf", 1, 2, N, opts=o) == 8  # FINUFFT_ERR_HORNER_WRONG_BETA
    o.gpu_kerevalmeth = 0
    assert _mk(engine, "cufinufftf", 1, 2, N, opts=o) == 7  # FINUFFT_ERR_UPSAMPFAC_TOO_SMALL
    o.upsampfac = 4.5
    assert _mk(engine, "cufinufftf", 1, 2, N, opts=o) == 0  # only a warning
    o = _lib.default_opts()
    o.gpu_device_id = 999
    assert _mk(engine, "cufinufftf", 1, 2, N, opts=o) == 15  # FINUFFT_ERR_CUDA_FAILURE
    o = _lib.default_opts()
    o.gpu_method, o.gpu_binsizex, o.gpu_binsizey, o.gpu_binsizez = 2, 200, 200, 200
    assert _mk(engine, "cufinufftf", 1, 3, (64, 64, 64), opts=o) == 19  # INSUFFICIENT_SHMEM


def test_type3_null_targets(engine):
    import torch

    p = ctypes.c_void_p()
    assert engine.cufinufftf_makeplan(3, 2, None, 1, 1, 1e-5, ctypes.byref(p), None) == 0
    x = torch.zeros(10, device="cuda")
    ier = engine.cufinufftf_setpts(p, 10, x.data_ptr(), x.data_ptr(), None, 5, x.data_ptr(),
                                   None, None)
    assert ier == 21  # FINUFFT_ERR_INVALID_ARGUMENT
    assert engine.cufinufftf_destroy(p) == 0


@pytest.mark.parametrize("ty", [1, 2, 3])
def test_many_vectors_partial_batch(oracle, ty):
    """ntransf=5 with batches of 2 (last batch partial) equals 5 single transforms."""
    import finufft_gb300 as fg

    rng = np.random.default_rng(7)
    nm, M, nt = (24, 32), 3000, 5
    pts = rng.uniform(-np.pi, np.pi, (2, M)).astype(np.float32)
    freq = rng.uniform(-20, 20, (2, 700)).astype(np.float32)
    extra = dict(zip('stu', [_dev(f) for f in freq])) if ty == 3 else {}
    many = fg.Plan(ty, 2 if ty == 3 else nm, n_trans=nt, eps=1e-5, gpu_maxbatchsize=2)
    many.setpts(*[_dev(p) for p in pts], **extra)
    one = fg.Plan(ty, 2 if ty == 3 else nm, n_trans=1, eps=1e-5)
    one.setpts(*[_dev(p) for p in pts], **extra)
    data = _cx(rng, (nt, M) if ty != 2 else (nt,) + nm)
    out = many.execute(_dev(data)).cpu().numpy()
    for t in range(nt):
        ref = one.execute(_dev(data[t])).cpu().numpy()
        # type 3: the inner FFT plan's batch differs, so rounding differs slightly
        assert oracle.rel_l2(out[t], ref) < (3e-5 if ty == 3 else 1e-6)


def test_modeord_fft_order(oracle):
    import finufft_gb300 as fg

    rng = np.random.default_rng(8)
    nm, M = (15, 16), 2000
    pts = rng.uniform(-np.pi, np.pi, (2, M)).astype(np.float32)
    c = _cx(rng, M)
    p0 = fg.Plan(1, nm, eps=1e-5)
    p1 = fg.Plan(1, nm, eps=1e-5, modeord=1)
    for p in (p0, p1):
        p.setpts(*[_dev(q) for q in pts])
    f0 = p0.execute(_dev(c)).cpu().numpy()
    f1 = p1.execute(_dev(c)).cpu().numpy()
    np.testing.assert_allclose(np.fft.ifftshift(f0), f1, rtol=0, atol=1e-5 * np.abs(f0).max())
    # type 2 reads modes in FFT order
    fk = _cx(rng, nm)
    q0, q1 = fg.Plan(2, nm, eps=1e-5), fg.Plan(2, nm, eps=1e-5, modeord=1)
    for p in (q0, q1):
        p.setpts(*[_dev(q) for q in pts])
    a = q0.execute(_dev(fk)).cpu().numpy()
    b = q1.execute(_dev(np.fft.ifftshift(fk))).cpu().numpy()
    assert oracle.rel_l2(b, a) < 1e-6


@pytest.mark.parametrize("nm,dtype", [((64, 48), "complex128"), ((17, 23, 31), "complex64")])
def test_spreadinterponly(oracle, nm, dtype):
    """gpu_spreadinterponly: type 1 spreads onto the mode grid itself, type 2
    interpolates from it (no FFT, no deconvolution). The odd 3D grid makes
    pairs of x cells start at unaligned addresses in the tile write-back."""
    import finufft_gb300 as fg

    rng = np.random.default_rng(9)
    M = 4000
    f64 = dtype == "complex128"
    tol, chk = (1e-10, 1e-12) if f64 else (1e-5, 2e-5)
    pts = rng.uniform(-np.pi, np.pi, (len(nm), M)).astype(np.float64 if f64 else np.float32)
    c = _cx(rng, M, dtype)
    p = fg.Plan(1, nm, eps=tol, dtype=dtype, gpu_spreadinterponly=1)
    p.setpts(*[_dev(q) for q in pts])
    g = p.execute(_dev(c)).cpu().numpy()
    ns, beta = oracle.gpu_kernel(tol, 2.0, 1, not f64)
    ref = oracle._spread(_oracle_pts(pts), c, list(nm[::-1]), ns, beta)
    assert oracle.rel_l2(g, ref) < chk
    q = fg.Plan(2, nm, eps=tol, dtype=dtype, gpu_spreadinterponly=1)
    q.setpts(*[_dev(x) for x in pts])
    got = q.execute(_dev(ref.astype(dtype))).cpu().numpy()
    want = oracle._interp(_oracle_pts(pts), ref, list(nm[::-1]), ns, beta)
    assert oracle.rel_l2(got, want) < chk


def _oracle_pts(pts):
    return [p.astype(np.float64) for p in pts[::-1]]


@pytest.mark.parametrize("ty", [1, 2, 3])
@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_adjointness(ty, dtype):
    """<A x, y> = <x, A* y> (test/adjointness.cpp): tol 1e-6 float, 1e-12 double."""
    import finufft_gb300 as fg

    rng = np.random.default_rng(10 + ty)
    rdt = np.float32 if dtype == "complex64" else np.float64
    nm, M = (20, 16, 12), 2500
    pts = rng.uniform(-np.pi, np.pi, (3, M)).astype(rdt)
    freq = rng.uniform(-15, 15, (3, 900)).astype(rdt)
    extra = dict(zip('stu', [_dev(f) for f in freq])) if ty == 3 else {}
    tol = 1e-6 if dtype == "complex64" else 1e-12
    # float type 3 with sigma 1.25 loses digits to the large 1/phihat range
    # (the CPU library caps float widths at sigma < 1.4 for this reason)
    kw = {"upsampfac": 2.0} if (ty == 3 and dtype == "complex64") else {}
    p = fg.Plan(ty, 3 if ty == 3 else nm, eps=tol, dtype=dtype, **kw)
    p.setpts(*[_dev(q) for q in pts], **extra)
    nout = (900,) if ty == 3 else nm
    x = _cx(rng, (M,) if ty != 2 else nm, dtype)
    y = _cx(rng, nout if ty != 2 else (M,), dtype)
    ax = p.execute(_dev(x)).cpu().numpy().astype(np.complex128)
    aty = p.execute_adjoint(_dev(y)).cpu().numpy().astype(np.complex128)
    lhs = np.vdot(y.ravel(), ax.ravel())
    rhs = np.vdot(aty.ravel(), x.ravel())
    assert abs(lhs - rhs) / abs(lhs) < (1e-5 if dtype == "complex64" else 1e-11)


@pytest.mark.parametrize("prec", ["f", ""])
def test_host_pointer_api(oracle, engine, prec):
    """finufft[f]_makeplan/setpts/execute/execute_adjoint with host arrays."""
    from finufft_gb300 import _lib

    rdt = np.float32 if prec == "f" else np.float64
    cdt = np.complex64 if prec == "f" else np.complex128
    pfx = "finufft" + prec
    rng = np.random.default_rng(11)
    M, nm = 3000, (18, 14)  # C order: n_modes[0] fastest
    x, y = rng.uniform(-np.pi, np.pi, (2, M)).astype(rdt)
    c = _cx(rng, M, cdt)
    p = ctypes.c_void_p()
    tol = 1e-5 if prec == "f" else 1e-11
    m = (ctypes.c_int64 * 3)(nm[0], nm[1], 1)
    assert getattr(engine, pfx + "_makeplan")(1, 2, m, 1, 1, tol, ctypes.byref(p), None) == 0
    assert getattr(engine, pfx + "_setpts")(p, M, x.ctypes.data, y.ctypes.data, None, 0, None,
                                            None, None) == 0
    f = np.zeros(nm[0] * nm[1], dtype=cdt)
    assert getattr(engine, pfx + "_execute")(p, c.ctypes.data, f.ctypes.data) == 0
    ref = oracle.dirft1([x, y], c, 1, nm)
    # the accuracy contract: no worse than twice the CPU library's error at the
    # same tol (its algorithm restated in the oracle, same precision and inputs)
    cpu = oracle.CpuPlan(1, list(nm), 1, tol, dtype=cdt)
    cpu.setpts([x, y])
    cpu_err = oracle.rel_l2(cpu.execute(c).ravel(), ref)
    assert oracle.rel_l2(f, ref) < 2 * cpu_err
    # adjoint of type 1 = type 2 with the opposite sign, modes -> points
    g = _cx(rng, nm[0] * nm[1], cdt)
    cc = np.zeros(M, dtype=cdt)
    assert getattr(engine, pfx + "_execute_adjoint")(p, cc.ctypes.data, g.ctypes.data) == 0
    ref2 = oracle.dirft2([x, y], g, -1, nm)
    cpu2 = oracle.CpuPlan(2, list(nm), -1, tol, dtype=cdt)
    cpu2.setpts([x, y])
    cpu2_err = oracle.rel_l2(cpu2.execute(g), ref2)
    assert oracle.rel_l2(cc, ref2) < 2 * cpu2_err
    assert getattr(engine, pfx + "_destroy")(p) == 0


@pytest.mark.parametrize("ty", [1, 2, 3])
def test_host_pointer_pipelined_batches(oracle, engine, ty):
    """Host-pointer execute over several batches (input copy of batch k+1 and
    output copy of batch k-1 overlap batch k): 5 transforms in batches of 2,
    from pinned and from pageable host arrays, each equal to a direct sum."""
    import torch

    from finufft_gb300 import _lib

    rng = np.random.default_rng(40 + ty)
    M, nm, ntr, tol = 2500, (12, 10, 8), 5, 1e-5
    x, y, z = rng.uniform(-np.pi, np.pi, (3, M)).astype(np.float32)
    o = _lib.FinufftOpts()
    engine.finufft_default_opts(ctypes.byref(o))
    o.maxbatchsize = 2
    p = ctypes.c_void_p()
    m = (ctypes.c_int64 * 3)(*nm)
    assert engine.finufftf_makeplan(ty, 3, m, 1 if ty != 2 else -1, ntr, tol, ctypes.byref(p),
                                    ctypes.byref(o)) == 0
    K = 700
    s, t, u = (rng.uniform(-9, 9, (3, K)).astype(np.float32) if ty == 3 else (None,) * 3)
    ptr = (lambda a: a.ctypes.data if a is not None else None)
    assert engine.finufftf_setpts(p, M, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                  K if ty == 3 else 0, ptr(s), ptr(t), ptr(u)) == 0
    nout = K if ty == 3 else int(np.prod(nm))
    # bar: the same algorithm in FP64 (the plan's PSWF kernel) plus float rounding
    xo = [x.astype(np.float64), y.astype(np.float64), z.astype(np.float64)]

    def bar(k_in, ref):
        if ty == 1:
            same = oracle.nufft_es(1, xo, k_in, 1, tol, n_modes=nm, kernel="pswf").ravel()
        elif ty == 2:
            same = oracle.nufft_es(2, xo, k_in.reshape(nm[::-1]), -1, tol, n_modes=nm,
                                   kernel="pswf")
        else:
            same = oracle.nufft_es(3, xo, k_in, 1, tol, ss=[s, t, u], kernel="pswf")
        return 1.25 * oracle.rel_l2(same, ref) + 5e-6

    for pinned in (True, False):
        if ty == 2:
            fin = _cx(rng, (ntr, int(np.prod(nm))))
            cout = torch.zeros(ntr * M, dtype=torch.complex64, pin_memory=pinned).numpy()
            fh = torch.from_numpy(fin.ravel().copy())
            fh = fh.pin_memory() if pinned else fh
            assert engine.finufftf_execute(p, cout.ctypes.data, fh.numpy().ctypes.data) == 0
            for k in range(ntr):
                ref = oracle.dirft2([x, y, z], fin[k], -1, nm)
                assert oracle.rel_l2(cout[k * M:(k + 1) * M], ref) < bar(fin[k], ref)
        else:
            cin = _cx(rng, (ntr, M))
            ch = torch.from_numpy(cin.ravel().copy())
            ch = ch.pin_memory() if pinned else ch
            fout = torch.zeros(ntr * nout, dtype=torch.complex64, pin_memory=pinned).numpy()
            assert engine.finufftf_execute(p, ch.numpy().ctypes.data, fout.ctypes.data) == 0
            for k in range(ntr):
                if ty == 1:
                    ref = oracle.dirft1([x, y, z], cin[k], 1, nm)
                else:
                    ref = oracle.dirft3([x, y, z], cin[k], 1, [s, t, u])
                assert oracle.rel_l2(fout[k * nout:(k + 1) * nout], ref) < bar(cin[k], ref)
    assert engine.finufftf_destroy(p) == 0


def test_simple_interfaces(oracle, engine):
    import torch

    rng = np.random.default_rng(12)
    M = 2000
    x, y, z = rng.uniform(-np.pi, np.pi, (3, M)).astype(np.float32)
    c = _cx(rng, M)
    fk = torch.zeros(8 * 6 * 4, dtype=torch.complex64, device="cuda")
    d = [_dev(a) for a in (x, y, z, c)]
    ier = engine.cufinufftf3d1(ctypes.c_int64(M), ctypes.c_void_p(d[0].data_ptr()),
                               ctypes.c_void_p(d[1].data_ptr()), ctypes.c_void_p(d[2].data_ptr()),
                               ctypes.c_void_p(d[3].data_ptr()), 1, ctypes.c_float(1e-5),
                               ctypes.c_int64(8), ctypes.c_int64(6), ctypes.c_int64(4),
                               ctypes.c_void_p(fk.data_ptr()), None)
    assert ier == 0
    ref = oracle.dirft1([x, y, z], c, 1, (8, 6, 4))
    assert oracle.rel_l2(fk.cpu().numpy(), ref) < 2e-4
    out = torch.zeros(M, dtype=torch.complex64, device="cuda")
    ier = engine.cufinufftf1d2(ctypes.c_int64(M), ctypes.c_void_p(d[0].data_ptr()),
                               ctypes.c_void_p(out.data_ptr()), -1, ctypes.c_float(1e-5),
                               ctypes.c_int64(48), ctypes.c_void_p(fk.data_ptr()), None)
    assert ier == 0
    ref2 = oracle.dirft2([x], fk.cpu().numpy(), -1, (48,))
    assert oracle.rel_l2(out.cpu().numpy(), ref2) < 2e-4


def test_graph_replay_matches_execute(oracle):
    import torch

    import finufft_gb300 as fg

    rng = np.random.default_rng(13)
    nm, M = (32, 32, 32), 50000
    pts = rng.uniform(-np.pi, np.pi, (3, M)).astype(np.float32)
    s = torch.cuda.Stream()
    p = fg.Plan(1, nm, n_trans=3, eps=1e-5, gpu_stream=s.cuda_stream)
    p.setpts(*[_dev(q) for q in pts])
    c = _dev(_cx(rng, (3, M)))
    ref = p.execute(c)
    torch.cuda.synchronize()
    out = torch.zeros_like(ref)
    p.graph_capture(c, out)
    for _ in range(3):
        p.graph_launch()
    torch.cuda.synchronize()
    assert oracle.rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("ty", [1, 2])
def test_edge_cases(oracle, ty):
    """M=0 gives zeros, single mode, all points in one bin, tiny grids."""
    import torch

    import finufft_gb300 as fg

    rng = np.random.default_rng(14)
    p = fg.Plan(ty, (7, 5), eps=1e-5)
    e = torch.zeros(0, device="cuda")
    p.setpts(e, e)
    if ty == 1:
        out = p.execute(torch.zeros((1, 0), dtype=torch.complex64, device="cuda"))
        assert out.abs().max().item() == 0
    else:
        out = p.execute(_dev(_cx(rng, (7, 5))))
        assert out.numel() == 0
    # one mode, tiny grid, a dense cluster in one bin, points on the seam
    M = 20000
    pts = np.full((2, M), 0.5, np.float32) + 1e-3 * rng.standard_normal((2, M)).astype(np.float32)
    pts[:, :10] = np.float32(np.pi)
    for nm in [(1, 1), (2, 3), (64, 64)]:
        q = fg.Plan(ty, nm, eps=1e-5)
        q.setpts(*[_dev(a) for a in pts])
        if ty == 1:
            c = _cx(rng, M)
            f = q.execute(_dev(c)).cpu().numpy()
            ref = oracle.dirft1(_oracle_pts(pts), c, 1, nm[::-1]).reshape(nm)
        else:
            fk = _cx(rng, nm)
            f = q.execute(_dev(fk)).cpu().numpy()
            ref = oracle.dirft2(_oracle_pts(pts), fk.ravel(), -1, nm[::-1])
        assert oracle.rel_l2(f, ref) < 1e-3


@pytest.mark.parametrize("ty,nm", [(1, (24, 33)), (2, (24, 33)), (1, (10, 12, 15)),
                                   (2, (10, 12, 15))])
def test_fft_prune_matches_full_fft(oracle, ty, nm):
    """gbnufft_opts.fft_prune: the FFT as an x pass plus passes over the other
    dimensions on the retained modes' x columns (odd mode counts make the two
    column ranges unequal) gives the full FFT's result."""
    import finufft_gb300 as fg

    rng = np.random.default_rng(70 + ty + len(nm))
    M, ntr = 3000, 3
    pts = rng.uniform(-np.pi, np.pi, (len(nm), M)).astype(np.float32)
    outs = []
    data = _cx(rng, (ntr, M) if ty == 1 else (ntr,) + nm)
    for prune in (0, 1):
        p = fg.Plan(ty, nm, n_trans=ntr, eps=1e-5, isign=1 if ty == 1 else -1, fft_prune=prune,
                    gpu_maxbatchsize=2)
        p.setpts(*[_dev(q) for q in pts])
        outs.append(p.execute(_dev(data)).cpu().numpy())
    assert oracle.rel_l2(outs[1], outs[0]) < 1e-6
    xs = [q.astype(np.float64) for q in pts[::-1]]
    if ty == 1:
        ref = oracle.dirft1(xs, data[2], 1, nm[::-1]).reshape(nm)
    else:
        ref = oracle.dirft2(xs, data[2].ravel(), -1, nm[::-1])
    assert oracle.rel_l2(outs[1][2].ravel(), ref.ravel()) < 2e-4


@pytest.mark.parametrize("ty", [1, 3])
def test_repeated_setpts(oracle, ty):
    """setpts called again on one plan with more, then fewer points (the sort
    arrays grow, then are reused): each execute equals its direct sum; a graph
    captured before the new setpts is dropped (graph_launch refuses)."""
    import torch

    import finufft_gb300 as fg

    rng = np.random.default_rng(80 + ty)
    nm = (12, 10, 14)
    s = torch.cuda.Stream()
    kw = dict(eps=1e-5, isign=1, gpu_stream=s.cuda_stream)
    p = fg.Plan(ty, nm if ty == 1 else 3, **kw)
    for k, M in enumerate((5000, 60000, 100)):
        pts = rng.uniform(-np.pi, np.pi, (3, M)).astype(np.float32)
        c = _cx(rng, M)
        extra = {}
        if ty == 3:
            tg = rng.uniform(-8, 8, (3, 300 + 100 * k)).astype(np.float32)
            extra = dict(s=_dev(tg[0]), t=_dev(tg[1]), u=_dev(tg[2]))
        p.setpts(*[_dev(q) for q in pts], **extra)
        if k == 1:
            with pytest.raises(fg.NufftError):
                p.graph_launch()  # the graph captured for the previous points is gone
        dc = _dev(c)
        out = p.execute(dc)
        torch.cuda.synchronize()
        got = out.cpu().numpy().ravel()
        xs = [q.astype(np.float64) for q in pts[::-1]]
        if ty == 1:
            ref = oracle.dirft1(xs, c, 1, nm[::-1])
        else:
            ref = oracle.dirft3(xs, c, 1, [q.astype(np.float64) for q in tg[::-1]])
        assert oracle.rel_l2(got, ref) < 2e-4, M
        if k == 0:
            p.graph_capture(dc, out)


def test_trim_scratch_then_setpts(oracle, engine):
    """gbnufft_trim_scratch releases the setpts scratch pool; the next setpts
    allocates again and the transform is unchanged; a bad device is an error."""
    import finufft_gb300 as fg

    rng = np.random.default_rng(90)
    M, nm = 20000, (16, 16, 16)
    pts = rng.uniform(-np.pi, np.pi, (3, M)).astype(np.float32)
    c = _cx(rng, M)
    p = fg.Plan(1, nm, eps=1e-5, isign=1)
    p.setpts(*[_dev(q) for q in pts])
    a = p.execute(_dev(c)).cpu().numpy()
    assert engine.gbnufft_trim_scratch(0) == 0
    p.setpts(*[_dev(q) for q in pts])
    b = p.execute(_dev(c)).cpu().numpy()
    # the sort is deterministic; atomics add in any order (float rounding)
    assert oracle.rel_l2(b, a) < 1e-6
    assert engine.gbnufft_trim_scratch(999) != 0


def test_batch_cap_and_stage_times():
    """3D type-2 plans keep a batch's fine grids within half of L2 unless
    batch_cap = 1; 2D plans run gpu_maxbatchsize transforms per batch; the
    stage times of an execute in several batches cover every batch"""
    import torch

    import finufft_gb300 as fg

    l2 = torch.cuda.get_device_properties(0).L2_cache_size
    nt = 8
    nm3 = (64, 64, 64)
    p3 = fg.Plan(2, nm3, n_trans=nt, eps=1e-5, gpu_maxbatchsize=nt)
    gbytes = float(np.prod(p3.info().nf)) * 8
    expect = min(nt, max(1, int(l2 / (2 * gbytes)))) if 2 * gbytes <= l2 else nt
    assert p3.info().batchsize == expect
    assert fg.Plan(2, nm3, n_trans=nt, eps=1e-5, gpu_maxbatchsize=nt,
                   batch_cap=1).info().batchsize == nt
    assert fg.Plan(2, (512, 512), n_trans=nt, eps=1e-5,
                   gpu_maxbatchsize=nt).info().batchsize == nt
    # stage times against the execute's own duration, several batches
    rng = np.random.default_rng(106)
    M = 400_000
    pts = [_dev(rng.uniform(-np.pi, np.pi, M).astype(np.float32)) for _ in range(3)]
    p = fg.Plan(2, nm3, n_trans=nt, eps=1e-5, gpu_maxbatchsize=3, batch_cap=1)
    assert p.info().batchsize == 3
    p.setpts(*pts)
    fk = torch.randn(nt, *nm3, 2, device="cuda").view(torch.complex64)[..., 0]
    c = torch.empty(nt, M, dtype=torch.complex64, device="cuda")
    p.execute(fk, out=c)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    p.execute(fk, out=c)
    e1.record()
    torch.cuda.synchronize()
    whole = e0.elapsed_time(e1)
    p.stage_times(True)
    p.execute(fk, out=c)
    torch.cuda.synchronize()
    st = p.stage_times(False)
    # three batches: the last alone would be about a third of the whole
    assert st[3] > 0.7 * whole, (st, whole)
    assert abs(st[0] + st[1] + st[2] - st[3]) < 0.05 * st[3] + 0.05, st
