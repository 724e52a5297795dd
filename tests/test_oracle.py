"""CPU tests of the oracle: pinned to the reference's own code (golden
fixtures generated by tests/golden/make_golden.py from the reference's
src/common) and to FP64 direct sums."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_planning.json")


@pytest.fixture(scope="module")
def gold():
    with open(GOLD) as f:
        return json.load(f)


def test_next235_against_reference(oracle, gold):
    for n, v in gold["next235_even"]:
        assert oracle.next235_even(n) == v, n


def test_next235_known_answers(oracle):
    # the true outputs next235(n, 2) for n = 0..20 (test/testutils.cpp:39-44)
    want = [2, 2, 2, 4, 4, 6, 6, 8, 8, 10, 10, 12, 12, 16, 16, 16, 16, 18, 18, 20, 20]
    assert [oracle.next235_even(n) for n in range(21)] == want
    assert oracle.next235_even(3 * 10 ** 9) >= 3 * 10 ** 9


def test_gauss_legendre_against_reference(oracle, gold):
    for n, (x, w) in gold["gaussquad"].items():
        xx, ww = oracle.gauss_legendre(int(n))
        np.testing.assert_allclose(xx, x, atol=1e-15)
        np.testing.assert_allclose(ww, w, rtol=1e-13, atol=5e-15)


def test_gauss_legendre_integrates(oracle):
    # test/testutils.cpp:73-85: 16 nodes integrate f' exactly to 1e-14
    x, w = oracle.gauss_legendre(16)
    f = lambda t: np.sin(4 * t + 1.0) + 0.3
    fp = lambda t: 4 * np.cos(4 * t + 1.0)
    assert abs(np.dot(w, fp(x)) - (f(1.0) - f(-1.0))) < 1e-14


def test_type3_grid_against_reference(oracle, gold):
    for s, X, S, ns, nf, h, gam in gold["nhg_type3"]:
        a, b, c = oracle.type3_grid(s, X, S, ns)
        assert a == nf
        assert b == pytest.approx(h, rel=1e-15)
        assert c == pytest.approx(gam, rel=1e-14)


def test_cpu_kernel_shape_against_reference(oracle, gold):
    for tol, dim, ty, s, ns, beta in gold["cpu_kernel"]:
        n2, b2 = oracle.cpu_kernel(tol, dim, ty, s, clip=False)
        assert n2 == ns
        assert b2 == pytest.approx(beta, rel=1e-14)


def test_pswf_against_reference(oracle, gold):
    z = np.array(gold["pswf"]["z"])
    for c, v in gold["pswf"]["values"].items():
        np.testing.assert_allclose(oracle.pswf0(float(c), z), v, atol=2e-15)


def test_gpu_kernel_rule(oracle):
    # widths/betas of the GPU rule (src/cuda/makeplan.cu:91-115) at the metric configs
    assert oracle.gpu_kernel(1e-5, 2.0, 1, True) == (6, pytest.approx(13.8, rel=1e-6))
    ns, beta = oracle.gpu_kernel(1e-12, 2.0, 1, False)
    assert ns == 13 and beta == pytest.approx(29.9)
    assert oracle.gpu_kernel(1e-6, 1.25, 1, True)[0] == 10
    assert oracle.gpu_kernel(1e-1, 2.0, 1, True)[0] == 2
    assert oracle.gpu_kernel(1e-16, 2.0, 1, False)[0] == 16  # clipped
    with pytest.raises(ValueError, match="8"):
        oracle.gpu_kernel(1e-5, 1.5, 1, True)
    with pytest.raises(ValueError, match="7"):
        oracle.gpu_kernel(1e-5, 0.9, 0, True)


def test_dirft_small_against_numpy(oracle):
    rng = np.random.default_rng(0)
    x, y = rng.uniform(-np.pi, np.pi, (2, 7))
    c = rng.standard_normal(7) + 1j * rng.standard_normal(7)
    nm = (4, 3)
    f = oracle.dirft1([x, y], c, -1, nm).reshape(3, 4)
    k1 = np.arange(4) - 2
    k2 = np.arange(3) - 1
    want = np.array([[np.sum(c * np.exp(-1j * (a * x + b * y))) for a in k1] for b in k2])
    np.testing.assert_allclose(f, want, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("ty", [1, 2, 3])
def test_es_restatement_against_dirft(oracle, dim, ty):
    rng = np.random.default_rng(dim * 10 + ty)
    M = 200
    nm = [16, 12, 10][:dim]
    xs = [rng.uniform(-np.pi, np.pi, M) for _ in range(dim)]
    c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    tol = 1e-9 if ty != 3 else 1e-6
    if ty == 1:
        got = oracle.nufft_es(1, xs, c, 1, tol, n_modes=nm, is_float=False)
        ref = oracle.dirft1(xs, c, 1, nm)
    elif ty == 2:
        fk = rng.standard_normal(tuple(reversed(nm))) + 1j * rng.standard_normal(tuple(reversed(nm)))
        got = oracle.nufft_es(2, xs, fk, -1, tol, n_modes=nm, is_float=False)
        ref = oracle.dirft2(xs, fk, -1, nm)
    else:
        ss = [rng.uniform(-30, 30, 60) for _ in range(dim)]
        got = oracle.nufft_es(3, xs, c, 1, tol, ss=ss, is_float=False)
        ref = oracle.dirft3(xs, c, 1, ss)
    assert oracle.rel_l2(got, ref) < 10 * tol


@pytest.mark.parametrize("ty", [1, 2])
@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-9), (np.complex64, 1e-4)])
def test_cpu_pswf_restatement_against_dirft(oracle, ty, dtype, tol):
    rng = np.random.default_rng(5)
    M, nm = 500, [20, 16, 12]
    xs = [rng.uniform(-np.pi, np.pi, M) for _ in range(3)]
    plan = oracle.CpuPlan(ty, nm, 1 if ty == 1 else -1, tol, dtype=dtype)
    plan.setpts(xs)
    if ty == 1:
        c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
        err = oracle.rel_l2(plan.execute(c), oracle.dirft1(xs, c, 1, nm))
    else:
        fk = rng.standard_normal((12, 16, 20)) + 1j * rng.standard_normal((12, 16, 20))
        err = oracle.rel_l2(plan.execute(fk), oracle.dirft2(xs, fk, -1, nm))
    assert err < (10 * tol if dtype == np.complex128 else 5 * tol)


def test_bin_sort_is_stable_and_bin_ordered(oracle):
    rng = np.random.default_rng(3)
    M = 5000
    xs = [rng.uniform(-np.pi, np.pi, M) for _ in range(3)]
    xs[0][:10] = np.pi  # exactly on the periodic seam
    xs[1][10:20] = -np.pi
    nf, bins = [40, 30, 20], [8, 7, 6]
    perm, loc = oracle.bin_sort(xs, nf, bins)
    assert sorted(perm.tolist()) == list(range(M))
    # loc lies in [0, bin]
    for d in range(3):
        assert loc[d].min() >= 0 and loc[d].max() <= bins[d]
    # key = bin * binvol + cell inside the bin (x fastest); stable inside a key
    nb = [(nf[d] + bins[d] - 1) // bins[d] for d in range(3)]
    cell = []
    for d in range(3):
        r = np.mod(xs[d] / (2 * np.pi) + 0.5, 1.0) * nf[d]
        cell.append(np.minimum(np.floor(r).astype(np.int64), nf[d] - 1))
    b = [cell[d] // bins[d] for d in range(3)]
    lc = [cell[d] - b[d] * bins[d] for d in range(3)]
    key = (b[0] + nb[0] * (b[1] + nb[1] * b[2])) * (bins[0] * bins[1] * bins[2]) + \
        lc[0] + bins[0] * (lc[1] + bins[1] * lc[2])
    ks = key[perm]
    # away from float ties the numpy key agrees with the exact fold
    assert np.mean(np.diff(ks) >= 0) > 0.999
    same = np.diff(ks) == 0
    assert np.all(np.diff(perm)[same] > 0)


def test_bin_sort_start_cell_keys_for_odd_widths(oracle):
    """odd kernel widths: inside a bin the host sort orders points by the cell
    where their support starts (the cell, or the next one when the fraction is
    at least one half; bin + 1 values per axis), so points that start at the
    same cell are adjacent; even widths keep whole-cell keys"""
    rng = np.random.default_rng(4)
    M = 6000
    xs = [rng.uniform(-np.pi, np.pi, M) for _ in range(3)]
    nf, bins = [48, 36, 24], [8, 6, 4]
    nb = [(nf[d] + bins[d] - 1) // bins[d] for d in range(3)]
    cell, frac = [], []
    for d in range(3):
        r = np.mod(xs[d] / (2 * np.pi) + 0.5, 1.0) * nf[d]
        c = np.minimum(np.floor(r).astype(np.int64), nf[d] - 1)
        cell.append(c)
        frac.append(r - c)
    b = [cell[d] // bins[d] for d in range(3)]
    binid = b[0] + nb[0] * (b[1] + nb[1] * b[2])
    for ns in (5, 6, 7):
        perm, loc = oracle.bin_sort(xs, nf, bins, loc_dtype=np.float64, ns=ns)
        assert sorted(perm.tolist()) == list(range(M))
        ex = ns % 2
        st = [cell[d] - b[d] * bins[d] + (ex * (frac[d] >= 0.5)) for d in range(3)]
        w = [bins[d] + ex for d in range(3)]
        key = binid * (w[0] * w[1] * w[2]) + st[0] + w[0] * (st[1] + w[1] * st[2])
        ks = key[perm]
        assert np.mean(np.diff(ks) >= 0) > 0.999, ns
        # the support start computed from the sorted bin-local coordinates
        # (ceil(l - ns/2) + ns/2, the spreader's rule) is the key's start cell
        # or one less, and never decreases along z inside a bin (the tile
        # clear's z bounds rely on it)
        s = np.ceil(loc - ns / 2) + ns // 2
        if ex:
            kz = st[2][perm]
            assert np.mean((s[2] <= kz) & (s[2] >= kz - 1)) > 0.999, ns
        same_bin = np.diff(binid[perm]) == 0
        assert np.mean(np.diff(np.floor(loc[2]))[same_bin] >= -1) == 1.0


def test_single_precision_fold_matches_fp64_fold(oracle):
    """The engine's float fold (error-free float arithmetic) places float
    coordinates where the FP64 fold does: same cell except within 1e-6 of a
    cell edge, grid positions equal to ~1e-12 of the grid, including the
    period seam, exact multiples of pi and large |x|."""
    rng = np.random.default_rng(5)
    base = np.concatenate([rng.uniform(-np.pi, np.pi, 200000), rng.uniform(-50, 50, 50000),
                           np.float32([0.0, np.pi, -np.pi, 3 * np.pi, -np.float32(np.pi),
                                       np.nextafter(np.float32(np.pi), np.float32(0))]),
                           # a coordinate 1e-8 cells below a cell edge on a 512 grid
                           np.uint32([3158904795]).view(np.float32)]).astype(np.float32)
    for nf in (16, 512, 2048, 100000, (1 << 20) - 2):
        # coordinates on and next to every cell edge (all edges for small grids)
        j = np.arange(0, nf + 1, max(1, nf // 4096))
        e = (2 * np.pi * (j / nf - 0.5)).astype(np.float32)
        x = np.concatenate([base, e, np.nextafter(e, np.float32(9)), np.nextafter(e, np.float32(-9))])
        c1, f1 = oracle.fold_positions(x, nf, True)
        c0, f0 = oracle.fold_positions(x, nf, False)
        assert ((c1 >= 0) & (c1 < nf)).all() and ((f1 >= 0) & (f1 <= 1)).all()
        # positions on the circle of length nf
        d = (c1 + f1) - (c0 + f0)
        d = np.where(d > nf / 2, d - nf, np.where(d < -nf / 2, d + nf, d))
        assert np.abs(d).max() < 1e-12 * nf + 1e-7, nf  # float frac rounding: < 6e-8
        same = c1 == c0
        edge = np.minimum(f0, 1 - f0) < 1e-6
        assert (same | edge).all(), nf


def test_bin_sort_reference_ordering(oracle):
    """bin_only: the reference's bin ordering -- bin index floor(folded cell /
    bin) with x fastest (include/cufinufft/spreadinterp.hpp:139-150) and
    points of a bin in input order, as the CPU library's stable counting sort
    (include/finufft/spread.hpp:459-584) -- computed here independently"""
    rng = np.random.default_rng(5)
    M = 6000
    xs = [rng.uniform(-np.pi, np.pi, M) for _ in range(3)]
    xs[0][:10] = np.pi
    xs[2][10:20] = -np.pi
    nf, bins = [40, 30, 20], [8, 7, 6]
    nb = [(nf[d] + bins[d] - 1) // bins[d] for d in range(3)]
    for ns in (6, 7):
        perm, _ = oracle.bin_sort(xs, nf, bins, loc_dtype=np.float64, ns=ns, bin_only=True)
        b = []
        for d in range(3):
            r = np.mod(xs[d] / (2 * np.pi) + 0.5, 1.0) * nf[d]
            b.append(np.minimum(np.floor(r).astype(np.int64), nf[d] - 1) // bins[d])
        binid = b[0] + nb[0] * (b[1] + nb[1] * b[2])
        expect = np.argsort(binid, kind="stable")
        # away from float ties at bin edges the numpy fold agrees with the exact one
        assert np.mean(perm == expect) > 0.999, ns
        ks = binid[perm]
        same = np.diff(ks) == 0
        assert np.all(np.diff(perm)[same] > 0), ns
