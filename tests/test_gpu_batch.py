"""GPU tests of uneven batches (cufinufft[f]_batch_*): many independent
transforms with different mode counts and point counts, executed by single
launches over all problems. Every problem must agree with a plan of its own
(to the tolerance: the batch rounds fine grids up to a size ladder) and with
the FP64 direct sum within the requested tolerance."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _make_batch(rng, dim, nprob, nlo, nhi, mlo, mhi):
    modes = [tuple(int(v) for v in rng.integers(nlo, nhi + 1, dim)) for _ in range(nprob)]
    Ms = [int(v) for v in rng.integers(mlo, mhi + 1, nprob)]
    return modes, Ms


@pytest.mark.parametrize("dim,ty,prec", [(2, 1, "f"), (2, 2, "f"), (3, 1, "f"), (1, 1, "f"),
                                         (2, 1, ""), (3, 1, ""), (3, 2, "f")])
def test_uneven_batch_matches_single_plans(oracle, engine, dim, ty, prec):
    import torch

    import finufft_gb300 as fg
    from finufft_gb300 import _lib

    rdt = np.float32 if prec == "f" else np.float64
    cdt = np.complex64 if prec == "f" else np.complex128
    tol = 1e-6 if prec == "f" else 1e-10
    rng = np.random.default_rng(31 + dim + 10 * ty)
    nprob = 24
    nrange = {1: (16, 200), 2: (8, 60), 3: (4, 16)}[dim]
    modes, Ms = _make_batch(rng, dim, nprob, nrange[0], nrange[1], 0, 3000)
    Ms[3] = 0  # an empty problem
    pts = [rng.uniform(-np.pi, np.pi, (dim, m)).astype(rdt) for m in Ms]
    # concatenated arrays (C order: coordinate d = dimension d, x fastest)
    xyz = [np.concatenate([p[d] for p in pts]) if sum(Ms) else np.zeros(0, rdt) for d in range(dim)]
    nm = np.array([list(m) + [1] * (3 - dim) for m in modes], dtype=np.int64).ravel()
    plan = ctypes.c_void_p()
    pfx = "cufinufft" + prec
    ier = getattr(engine, pfx + "_batch_makeplan")(
        ty, dim, nprob, nm.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), 1 if ty == 1 else -1,
        tol, ctypes.byref(plan), None, None)
    assert ier == 0
    dx = [_dev(a) for a in xyz] + [None] * (3 - dim)
    Ma = np.array(Ms, dtype=np.int64)
    ier = getattr(engine, pfx + "_batch_setpts")(
        plan, Ma.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        *[a.data_ptr() if a is not None else None for a in dx])
    assert ier == 0
    nmodes = [int(np.prod(m)) for m in modes]
    if ty == 1:
        cs = [(rng.standard_normal(m) + 1j * rng.standard_normal(m)).astype(cdt) for m in Ms]
        c = _dev(np.concatenate(cs))
        fk = torch.zeros(sum(nmodes), dtype=c.dtype, device="cuda")
    else:
        fks = [(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(cdt) for n in nmodes]
        fk = _dev(np.concatenate(fks))
        c = torch.zeros(sum(Ms), dtype=fk.dtype, device="cuda")
    assert getattr(engine, pfx + "_batch_execute")(plan, c.data_ptr(), fk.data_ptr()) == 0
    torch.cuda.synchronize()
    out = (fk if ty == 1 else c).cpu().numpy()
    assert getattr(engine, pfx + "_batch_destroy")(plan) == 0
    moff = np.concatenate([[0], np.cumsum(nmodes)])
    poff = np.concatenate([[0], np.cumsum(Ms)])
    for p in range(nprob):
        if Ms[p] == 0 and ty == 2:
            continue
        rowmajor = tuple(reversed(modes[p]))
        single = fg.Plan(ty, rowmajor, eps=tol, dtype="complex64" if prec == "f" else "complex128",
                         isign=1 if ty == 1 else -1)
        single.setpts(*[_dev(a) for a in pts[p][::-1]]) if Ms[p] else single.setpts(
            *[torch.zeros(0, dtype=torch.float32 if prec == "f" else torch.float64,
                          device="cuda")] * dim)
        if ty == 1:
            ref = single.execute(_dev(cs[p]).reshape(1, -1) if Ms[p] else
                                 torch.zeros((1, 0), dtype=c.dtype, device="cuda")).cpu().numpy().ravel()
            got = out[moff[p]:moff[p + 1]]
        else:
            ref = single.execute(_dev(fks[p].reshape(rowmajor))).cpu().numpy().ravel()
            got = out[poff[p]:poff[p + 1]]
        if np.linalg.norm(ref) == 0:
            assert np.abs(got).max() == 0
            continue
        # batched grids come from a size ladder (up to 25% finer than a single
        # plan's), so the two approximations agree to about tol, not bitwise
        assert oracle.rel_l2(got, ref) < (1e-5 if prec == "f" else 10 * tol), p
        if p < 3:  # and the truth, for a few problems
            if ty == 1:
                tru = oracle.dirft1([pts[p][d] for d in range(dim)], cs[p], 1, modes[p])
            else:
                tru = oracle.dirft2([pts[p][d] for d in range(dim)], fks[p], -1, modes[p])
            assert oracle.rel_l2(got, tru) < (1e-4 if prec == "f" else 1e-8)
