"""The accuracy contract on the benchmark workloads at reduced sizes: the
engine's relative l2 error against an FP64 direct sum on sampled outputs is no
worse than twice the error of the CPU library's algorithm (the oracle's
restatement of FINUFFT's CPU code, PSWF kernel, same precision) on the same
inputs at the same tol. All engine calls go through the C ABI."""
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clustered3(rng, M, rdt):
    """the metric's point mix: 80% from 8 wrapped Gaussians (sigma 0.3), 20% uniform"""
    ncl = int(0.8 * M)
    cen = rng.uniform(-np.pi, np.pi, (8, 3))
    cl = cen[rng.integers(0, 8, ncl)].T + 0.3 * rng.standard_normal((3, ncl))
    cl = np.remainder(cl + np.pi, 2 * np.pi) - np.pi
    u = rng.uniform(-np.pi, np.pi, (3, M - ncl))
    return np.concatenate([cl, u], axis=1).astype(rdt)


def _cx(rng, shape, cdt):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(cdt)


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("dtype,tol,nside,M", [("complex64", 1e-5, 128, 1_000_000),
                                               ("complex128", 1e-12, 64, 1_000_000)])
def test_c3_type1_clustered(oracle, dtype, tol, nside, M):
    """3D type 1 on the metric's clustered mix (FP32 at tol 1e-5, FP64 at tol 1e-12)"""
    import finufft_gb300 as fg

    rdt = np.float32 if dtype == "complex64" else np.float64
    rng = np.random.default_rng(31)
    pts = _clustered3(rng, M, rdt)
    c = _cx(rng, (2, M), dtype)
    nm = (nside,) * 3
    plan = fg.Plan(1, nm, n_trans=2, eps=tol, dtype=dtype, isign=1)
    plan.setpts(*[_dev(p) for p in pts])
    f = plan.execute(_dev(c)).cpu().numpy()
    cpu = oracle.CpuPlan(1, list(nm), +1, tol, dtype=dtype)
    cpu.setpts([pts[2], pts[1], pts[0]])
    kidx = np.random.default_rng(32).choice(nside ** 3, 1000, replace=False)
    for k in range(2):
        ref = oracle.dirft1([pts[2], pts[1], pts[0]], c[k], 1, nm, kidx=kidx)
        cpu_err = oracle.rel_l2(cpu.execute(c[k]).ravel()[kidx], ref)
        gpu_err = oracle.rel_l2(f[k].ravel()[kidx], ref)
        assert gpu_err <= 2 * cpu_err, (k, gpu_err, cpu_err)


def test_c2_type2_batched(oracle):
    """2D type 2, 16 vectors sharing 1e6 points, 256^2 modes, tol 1e-5"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(33)
    M, nt, N, tol = 1_000_000, 16, (256, 256), 1e-5
    x, y = rng.uniform(-np.pi, np.pi, (2, M)).astype(np.float32)
    fk = _cx(rng, (nt,) + N, np.complex64)
    plan = fg.Plan(2, N, n_trans=nt, eps=tol, isign=-1, gpu_maxbatchsize=nt)
    plan.setpts(_dev(x), _dev(y))
    c = plan.execute(_dev(fk)).cpu().numpy()
    cpu = oracle.CpuPlan(2, [N[1], N[0]], -1, tol, dtype=np.complex64)
    cpu.setpts([y, x])
    jidx = np.random.default_rng(34).choice(M, 1000, replace=False)
    for k in (0, nt - 1):
        ref = oracle.dirft2([y, x], fk[k].ravel(), -1, [N[1], N[0]], jidx=jidx)
        cpu_err = oracle.rel_l2(cpu.execute(fk[k])[jidx], ref)
        gpu_err = oracle.rel_l2(c[k][jidx], ref)
        assert gpu_err <= 2 * cpu_err, (k, gpu_err, cpu_err)


def test_c4_uneven_batch(oracle, engine):
    """256 uneven 2D type-1 problems (N/side log-uniform in [32,256], M
    log-uniform in [1e3,1e5]) in one batched plan at tol 1e-6"""
    import ctypes

    import torch

    from finufft_gb300 import _lib

    rng = np.random.default_rng(35)
    nprob, tol = 256, 1e-6
    Ns = np.round(np.exp(rng.uniform(np.log(32), np.log(256), (nprob, 2)))).astype(np.int64)
    Ms = np.round(np.exp(rng.uniform(np.log(1e3), np.log(1e5), nprob))).astype(np.int64)
    Mt = int(Ms.sum())
    xy = rng.uniform(-np.pi, np.pi, (2, Mt)).astype(np.float32)
    c = _cx(rng, Mt, np.complex64)
    nm = np.concatenate([Ns, np.ones((nprob, 1), np.int64)], axis=1).ravel()
    plan = ctypes.c_void_p()
    o = _lib.default_opts()
    i64p = ctypes.POINTER(ctypes.c_int64)
    assert engine.cufinufftf_batch_makeplan(1, 2, nprob, nm.ctypes.data_as(i64p), 1, tol,
                                            ctypes.byref(plan), ctypes.byref(o), None) == 0
    dx, dy, dc = _dev(xy[0]), _dev(xy[1]), _dev(c)
    assert engine.cufinufftf_batch_setpts(plan, Ms.ctypes.data_as(i64p), dx.data_ptr(),
                                          dy.data_ptr(), None) == 0
    nmodes = Ns[:, 0] * Ns[:, 1]
    fk = torch.empty(int(nmodes.sum()), dtype=torch.complex64, device="cuda")
    assert engine.cufinufftf_batch_execute(plan, dc.data_ptr(), fk.data_ptr()) == 0
    assert engine.cufinufftf_batch_destroy(plan) == 0
    fk = fk.cpu().numpy()
    off = np.concatenate([[0], np.cumsum(Ms)])
    moff = np.concatenate([[0], np.cumsum(nmodes)])
    got, want, cpu = [], [], []
    for p in np.random.default_rng(36).choice(nprob, 48, replace=False):
        a, b = off[p], off[p + 1]
        n0, n1 = int(Ns[p, 0]), int(Ns[p, 1])
        kidx = np.random.default_rng(int(p)).choice(n0 * n1, 20, replace=False)
        want.append(oracle.dirft1([xy[0, a:b], xy[1, a:b]], c[a:b], 1, [n0, n1], kidx=kidx))
        got.append(fk[moff[p]:moff[p + 1]][kidx])
        cp = oracle.CpuPlan(1, [n0, n1], +1, tol, dtype=np.complex64)
        cp.setpts([xy[0, a:b], xy[1, a:b]])
        cpu.append(cp.execute(c[a:b]).ravel()[kidx])
    want = np.concatenate(want)
    gpu_err = oracle.rel_l2(np.concatenate(got), want)
    cpu_err = oracle.rel_l2(np.concatenate(cpu), want)
    assert gpu_err <= 2 * cpu_err, (gpu_err, cpu_err)


def test_c5_type3(oracle):
    """3D type 3, M = K = 1e5, sources in the box (1,2,4), targets in (200,100,50)/4,
    tol 1e-6, error on 1e4 sampled targets"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(37)
    M = K = 100_000
    xs = (rng.uniform(-1, 1, (3, M)) * np.array([1.0, 2.0, 4.0])[:, None]).astype(np.float32)
    ss = (rng.uniform(-1, 1, (3, K)) * np.array([50.0, 25.0, 12.5])[:, None]).astype(np.float32)
    c = _cx(rng, M, np.complex64)
    plan = fg.Plan(3, 3, eps=1e-6, isign=1)
    plan.setpts(*[_dev(a) for a in xs], s=_dev(ss[0]), t=_dev(ss[1]), u=_dev(ss[2]))
    f = plan.execute(_dev(c)).cpu().numpy()
    sigma = plan.info().upsampfac
    kidx = np.random.default_rng(38).choice(K, 10000, replace=False)
    ref = oracle.dirft3(list(xs), c, 1, list(ss), kidx=kidx)
    cpu = oracle.CpuPlan(3, 3, +1, 1e-6, dtype=np.complex64, sigma=sigma)
    cpu.setpts(list(xs), list(ss))
    cpu_err = oracle.rel_l2(cpu.execute(c)[kidx], ref)
    gpu_err = oracle.rel_l2(f[kidx], ref)
    assert gpu_err <= 2 * cpu_err, (gpu_err, cpu_err)


def test_c1_type1_fp64(oracle):
    """1D type 1 in double precision at tol 1e-9 (M = N = 1e5)"""
    import finufft_gb300 as fg

    rng = np.random.default_rng(39)
    M = N = 100_000
    x = rng.uniform(-np.pi, np.pi, M)
    c = _cx(rng, M, np.complex128)
    plan = fg.Plan(1, (N,), eps=1e-9, dtype="complex128", isign=1)
    plan.setpts(_dev(x))
    f = plan.execute(_dev(c)).cpu().numpy()
    kidx = np.random.default_rng(40).choice(N, 1000, replace=False)
    ref = oracle.dirft1([x], c, 1, [N], kidx=kidx)
    cpu = oracle.CpuPlan(1, [N], +1, 1e-9, dtype=np.complex128)
    cpu.setpts([x])
    cpu_err = oracle.rel_l2(cpu.execute(c).ravel()[kidx], ref)
    gpu_err = oracle.rel_l2(f[kidx], ref)
    assert gpu_err <= 2 * cpu_err, (gpu_err, cpu_err)
