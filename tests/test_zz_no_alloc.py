"""GPU test of cufinufftf_spread_noalloc, the spread entry point that works in
a fixed scratch area compiled into the library, for callers that may not
allocate device memory. Its output must equal the regular entry point's
(a type-1 cufinufftf plan with gpu_spreadinterponly = 1), on two calls in a
row, so a second call that reuses the scratch left by the first is covered.
Kept in its own file, collected last, and valid in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _regular_spread(engine, nm_c, pts_c, c, tol):
    """the existing path: makeplan(type 1, spreadinterponly) + setpts + execute"""
    import torch

    from finufft_gb300 import _lib

    dim = len(nm_c)
    o = _lib.default_opts()
    o.gpu_spreadinterponly = 1
    p = ctypes.c_void_p()
    m = (ctypes.c_int64 * 3)(*(list(nm_c) + [1] * (3 - dim)))
    assert engine.cufinufftf_makeplan(1, dim, m, 1, 1, tol, ctypes.byref(p), ctypes.byref(o)) == 0
    ptr = [a.data_ptr() for a in pts_c] + [None] * (3 - dim)
    assert engine.cufinufftf_setpts(p, pts_c[0].numel(), *ptr, 0, None, None, None) == 0
    out = torch.zeros(int(np.prod(nm_c)), dtype=torch.complex64, device="cuda")
    assert engine.cufinufftf_execute(p, c.data_ptr(), out.data_ptr()) == 0
    torch.cuda.synchronize()
    assert engine.cufinufftf_destroy(p) == 0
    return out.cpu().numpy()


def _noalloc_spread(engine, nm_c, pts_c, c, tol):
    import torch

    dim = len(nm_c)
    grid = torch.full((int(np.prod(nm_c)),), 7.0 + 7.0j, dtype=torch.complex64, device="cuda")
    m = (ctypes.c_int64 * 3)(*(list(nm_c) + [1] * (3 - dim)))
    ptr = [a.data_ptr() for a in pts_c] + [None] * (3 - dim)
    ier = engine.cufinufftf_spread_noalloc(dim, m, pts_c[0].numel(), *ptr, c.data_ptr(),
                                           grid.data_ptr(), tol, None)
    assert ier == 0
    torch.cuda.synchronize()
    return grid.cpu().numpy()


@pytest.mark.parametrize("dim,nm_c,M", [(1, (4096,), 200000), (2, (256, 192), 300000),
                                        (3, (64, 48, 40), 500000)])
def test_noalloc_matches_regular_spread_twice(engine, dim, nm_c, M):
    import torch

    rng = np.random.default_rng(77 + dim)
    tol = 1e-5
    for call in range(2):  # the second call reuses the scratch left by the first
        pts = rng.uniform(-np.pi, np.pi, (dim, M)).astype(np.float32)
        pts[:, : M // 2] = (0.2 * rng.standard_normal((dim, M // 2))).astype(np.float32)
        c = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
        pts_c = [torch.from_numpy(p).cuda() for p in pts]
        cd = torch.from_numpy(c).cuda()
        want = _regular_spread(engine, nm_c, pts_c, cd, tol)
        got = _noalloc_spread(engine, nm_c, pts_c, cd, tol)
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < 1e-6, "call %d: rel diff %.3g" % (call, err)


def test_noalloc_rejects_oversize(engine):
    m = (ctypes.c_int64 * 3)(1 << 12, 1 << 12, 2)  # 2^25 cells > 2^24
    assert engine.cufinufftf_spread_noalloc(3, m, 10, None, None, None, None, None, 1e-5,
                                            None) == 2  # FINUFFT_ERR_MAXNALLOC
    m1 = (ctypes.c_int64 * 3)(1024, 1, 1)
    assert engine.cufinufftf_spread_noalloc(1, m1, (1 << 19) + 1, None, None, None, None, None,
                                            1e-5, None) == 2


def _free_bytes():
    import torch

    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_at_the_limits_against_the_oracle(engine, oracle):
    """3D at the declared limits (2^19 points, 2^24 grid cells, an odd kernel
    width whose start-cell sort keys are used too): the output equals the
    oracle's FP64 spread with the same ES kernel, and the call leaves the
    device's free memory unchanged (nothing allocated: the scratch is the fixed
    array, the library's setpts pool is trimmed first)"""
    import torch

    rng = np.random.default_rng(91)
    M = 1 << 19
    nm_c = (256, 256, 256)  # 2^24 cells, x fastest
    pts = rng.uniform(-np.pi, np.pi, (3, M)).astype(np.float32)
    pts[:, : M // 2] = (0.3 * rng.standard_normal((3, M // 2))).astype(np.float32)
    c = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    pts_c = [torch.from_numpy(p).cuda() for p in pts]
    cd = torch.from_numpy(c).cuda()
    grid = torch.empty(1 << 24, dtype=torch.complex64, device="cuda")
    m = (ctypes.c_int64 * 3)(*nm_c)
    for tol in (1e-5, 1e-4):  # widths 6 and 5
        assert engine.cufinufftf_spread_noalloc(3, m, M, *[a.data_ptr() for a in pts_c],
                                                cd.data_ptr(), grid.data_ptr(), tol, None) == 0
        assert engine.gbnufft_trim_scratch(0) == 0
        free0 = _free_bytes()
        assert engine.cufinufftf_spread_noalloc(3, m, M, *[a.data_ptr() for a in pts_c],
                                                cd.data_ptr(), grid.data_ptr(), tol, None) == 0
        free1 = _free_bytes()
        assert free1 >= free0, (free0, free1)
        got = grid.cpu().numpy()
        ns, beta = oracle.gpu_kernel(tol, 2.0, 1, True)
        want = oracle._spread([p.astype(np.float64) for p in pts], c, list(nm_c), ns, beta).ravel()
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < 1e-5, (tol, err)
