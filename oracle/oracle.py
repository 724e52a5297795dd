"""TEST INFRASTRUCTURE ONLY: the CPU oracle for the GB300 NUFFT engine.

Used by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py as the checker; the engine itself never imports this module.

It restates flatironinstitute/finufft's arithmetic on the CPU:
  * FP64 direct NUDFTs (test/utils/dirft{1,2,3}d.hpp) -- the ground truth;
  * the GPU library's algorithm with its ES kernel, in FP64
    (src/cuda/execute.cu:105-258 pipeline, include/cufinufft/spreadinterp.hpp
    kernel), with numpy's FFT -- a same-algorithm reference for tight parity;
  * the CPU library's algorithm with its PSWF kernel (src/common/kernel.cpp,
    include/finufft/makeplan.hpp:112-315, spreadinterp.hpp, execute.hpp),
    OpenMP spreading in C and scipy's FFT -- the "CPU FINUFFT" baseline;
  * the engine's FP64 fold and a stable host bin sort, which the device sort
    must reproduce bit for bit.
C parts live in oracle.c (built by oracle/Makefile into oracle/_build).
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
PI = math.pi

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P, I64 = ctypes.c_void_p, ctypes.c_int64
        i, d = ctypes.c_int, ctypes.c_double
        L.or_next235_even.argtypes = [I64]
        L.or_next235_even.restype = I64
        L.or_gauss_legendre.argtypes = [i, P, P]
        L.or_gpu_kernel.argtypes = [d, d, i, i, P]
        L.or_gpu_kernel.restype = i
        L.or_fine_grid.argtypes = [I64, d, i]
        L.or_fine_grid.restype = I64
        L.or_type3_grid.argtypes = [d, d, d, i, P]
        L.or_bin_sort.argtypes = [i, I64, P, P, P, P, P, P, P, i, i, i, i]
        L.or_fold_many.argtypes = [I64, P, i, i, P, P]
        L.or_dirft1.argtypes = [i, I64, P, P, i, P, I64, P, P]
        L.or_dirft2.argtypes = [i, I64, P, i, P, P, I64, P, P]
        L.or_dirft3.argtypes = [i, I64, P, P, i, P, I64, P, P]
        L.or_spread_es.argtypes = [i, I64, P, P, P, P, P, i, d, i, P, P]
        L.or_interp_es.argtypes = [i, I64, P, P, P, P, P, i, d, i, P, P]
        for suf in ("f", "d"):
            getattr(L, "or_cpu_sort_" + suf).argtypes = [i, I64, P, P, P]
            getattr(L, "or_cpu_spread_" + suf).argtypes = [i, I64, P, P, P, P, i, i, P, i, P]
            getattr(L, "or_cpu_interp_" + suf).argtypes = [i, I64, P, P, P, P, i, i, P, P]
        L.or_num_threads.restype = i
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _ptrs(arrs):
    """array of pointers to the given arrays (kept alive by the caller)"""
    arr = (ctypes.c_void_p * 3)(*[a.ctypes.data if a is not None else None for a in arrs]
                                + [None] * (3 - len(arrs)))
    return arr


def _cplx(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


# ------------------------------------------------------------- planning ----
def next235_even(n):
    return int(lib().or_next235_even(int(n)))


def gauss_legendre(n):
    x, w = np.zeros(n), np.zeros(n)
    lib().or_gauss_legendre(n, _ptr(x), _ptr(w))
    return x, w


def gpu_kernel(tol, sigma=2.0, kerevalmeth=1, is_float=True):
    """(ns, beta) of the GPU library's rule; raises on the reference's error cases."""
    b = np.zeros(1)
    ns = lib().or_gpu_kernel(float(tol), float(sigma), int(kerevalmeth), int(is_float), _ptr(b))
    if ns < 0:
        raise ValueError("finufft error %d" % -ns)
    return ns, float(b[0])


def fine_grid(ms, sigma, ns):
    return int(lib().or_fine_grid(int(ms), float(sigma), int(ns)))


def type3_grid(sigma, X, S, ns):
    out = np.zeros(3)
    lib().or_type3_grid(float(sigma), float(X), float(S), int(ns), _ptr(out))
    return int(out[0]), float(out[1]), float(out[2])


def width_center(lo, hi):
    """include/cufinufft/utils.hpp:119-130 (arraywidcen)"""
    w, c = (hi - lo) / 2, (hi + lo) / 2
    if abs(c) < 0.1 * w:
        w += abs(c)
        c = 0.0
    return w, c


def es_kernel(x, ns, beta):
    z = 2.0 * np.asarray(x, dtype=np.float64) / ns
    out = np.zeros_like(z)
    m = np.abs(z) < 1
    out[m] = np.exp(beta * (np.sqrt(1 - z[m] ** 2) - 1))
    return out


# -------------------------------------------------------- PSWF (CPU lib) ----
def pswf0(c, z):
    """Prolate spheroidal wave function psi_0^c on [-1,1], normalised psi(0)=1.

    Restates the published Legendre-expansion method (Bouwkamp; Xiao, Rokhlin
    & Yarvin 2001) that src/common/pswf.cpp implements: psi_0 is the eigenvector
    of the lowest eigenvalue of the prolate operator in the even normalised
    Legendre basis, a symmetric tridiagonal matrix."""
    from scipy.linalg import eigh_tridiagonal

    K = int(c) + 40
    n = 2 * np.arange(K, dtype=np.float64)
    bn = (2 * n * n + 2 * n - 1) / ((2 * n - 1) * (2 * n + 3))
    diag = n * (n + 1) + c * c * bn
    off = c * c * (n[:-1] + 1) * (n[:-1] + 2) / ((2 * n[:-1] + 3) * np.sqrt((2 * n[:-1] + 1) * (2 * n[:-1] + 5)))
    _, vec = eigh_tridiagonal(diag, off, select="i", select_range=(0, 0))
    v = vec[:, 0]
    coef = np.zeros(2 * K)
    coef[0::2] = v * np.sqrt(n + 0.5)
    z = np.asarray(z, dtype=np.float64)
    val = np.polynomial.legendre.legval(z, coef)
    val0 = np.polynomial.legendre.legval(0.0, coef)
    out = val / val0
    return np.where(np.abs(z) <= 1, out, 0.0)


def cpu_kernel(tol, dim, nufft_type, sigma=2.0, is_float=False, clip=True):
    """CPU library kernel width/shape (src/common/kernel.cpp:60-146, kerformula 8);
    clip=False returns the unclipped width of theoretical_kernel_ns."""
    tolfac = 0.18 * 1.4 ** (dim - 1) * (1.4 if nufft_type == 3 else 1.0)
    ns = int(math.ceil(math.log(tolfac / tol) / (PI * math.sqrt(1 - 1 / sigma)) + 1.0))
    if clip:
        ns = max(2, min(ns, 12 if is_float else 16))
        if is_float and sigma < 1.4:
            ns = min(ns, 8)
    beta = PI * ns * (1 - 1 / (2 * sigma)) - 0.05
    return ns, beta


def engine_kernel(tol, sigma=2.0, dim=3, nufft_type=1, is_float=True, kernel="pswf"):
    """The engine's kernel choice: (ns, beta, phi, horner table or None).

    kernel "es": the GPU library's rule and ES kernel (src/cuda/makeplan.cu:43-119);
    "pswf": the CPU library's PSWF (src/common/kernel.cpp:79-146, kerformula 8)
    with width max(CPU width law, GPU rule), clipped to 12 (float) / 16."""
    ns_g, beta_g = gpu_kernel(tol, sigma, 0 if sigma not in (2.0, 1.25) else 1, is_float)
    if kernel == "es":
        return ns_g, beta_g, (lambda x: es_kernel(x, ns_g, beta_g)), None
    eps = max(tol, np.finfo(np.float32 if is_float else np.float64).eps)
    ns_c = cpu_kernel(eps, dim, nufft_type, sigma, is_float, clip=False)[0]
    ns = max(2, min(max(ns_c, ns_g), 12 if is_float else 16))
    beta = PI * ns * (1 - 1 / (2 * sigma)) - 0.05
    fun = lambda x: pswf0(beta, 2.0 * np.asarray(x) / ns)
    return ns, beta, fun, np.ascontiguousarray(horner_table(fun, ns, min(ns + 6, 24)))


def horner_table(fun, ns, ncoef):
    """Monomial coefficients (highest degree first) of ns polynomial pieces of
    fun(x), piece j on x in [-ns/2+j, -ns/2+j+1], variable u = 2(x-start)-1,
    from Chebyshev interpolation at ncoef points. Returns array [ncoef, ns]."""
    k = np.arange(ncoef)
    u = np.cos(PI * (k + 0.5) / ncoef)
    tab = np.zeros((ncoef, ns))
    for j in range(ns):
        x = -ns / 2 + j + (u + 1) / 2
        cheb = np.polynomial.chebyshev.chebfit(u, fun(x), ncoef - 1)
        mono = np.polynomial.chebyshev.cheb2poly(cheb)
        tab[:, j] = mono[::-1]
    return tab


def kernel_ft(fun, ns, freqs, nodes_per_halfwidth):
    """phihat(k) = sum_n f_n 2cos(k z_n) by Gauss-Legendre (src/cuda/fft.cu:185-202)."""
    J2 = ns / 2.0
    q = int(2 + nodes_per_halfwidth * J2)
    x, w = np.polynomial.legendre.leggauss(2 * q)
    z = J2 * x[:q]
    f = J2 * w[:q] * fun(z)
    freqs = np.asarray(freqs, dtype=np.float64)
    return (2 * f[None, :] * np.cos(freqs[:, None] * z[None, :])).sum(axis=1)


# ---------------------------------------------------------- direct sums ----
def _coords(xs):
    return [np.ascontiguousarray(a, dtype=np.float64) for a in xs]


def dirft1(xs, c, isign, n_modes, kidx=None):
    """FP64 type 1: modes in CMCL order, n_modes[0] fastest; kidx = flat indices."""
    xs = _coords(xs)
    c = _cplx(c)
    nm = np.array(list(n_modes) + [1] * (3 - len(n_modes)), dtype=np.int64)
    nk = int(np.prod(nm)) if kidx is None else len(kidx)
    kidx_a = None if kidx is None else np.ascontiguousarray(kidx, dtype=np.int64)
    out = np.zeros(nk, dtype=np.complex128)
    lib().or_dirft1(len(xs), len(xs[0]), _ptrs(xs), _ptr(c), int(isign), _ptr(nm), nk,
                    _ptr(kidx_a), _ptr(out))
    return out


def dirft2(xs, f, isign, n_modes, jidx=None):
    xs = _coords(xs)
    f = _cplx(f).reshape(-1)
    nm = np.array(list(n_modes) + [1] * (3 - len(n_modes)), dtype=np.int64)
    M = len(xs[0])
    nj = M if jidx is None else len(jidx)
    jidx_a = None if jidx is None else np.ascontiguousarray(jidx, dtype=np.int64)
    out = np.zeros(nj, dtype=np.complex128)
    lib().or_dirft2(len(xs), M, _ptrs(xs), int(isign), _ptr(nm), _ptr(f), nj, _ptr(jidx_a),
                    _ptr(out))
    return out


def dirft3(xs, c, isign, ss, kidx=None):
    xs, ss = _coords(xs), _coords(ss)
    c = _cplx(c)
    nk = len(ss[0]) if kidx is None else len(kidx)
    kidx_a = None if kidx is None else np.ascontiguousarray(kidx, dtype=np.int64)
    out = np.zeros(nk, dtype=np.complex128)
    lib().or_dirft3(len(xs), len(xs[0]), _ptrs(xs), _ptr(c), int(isign), _ptrs(ss), nk,
                    _ptr(kidx_a), _ptr(out))
    return out


def rel_l2(a, b):
    """relative l2 error of a against the reference b (test/utils/norms.hpp:17-37)"""
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ------------------------------------------------------------ bin sort ----
def fold_positions(x, nf, f32):
    """grid positions cell + frac of float coordinates x under the engine's
    single-precision fold (f32) or its FP64 fold: (cell int32, frac float64)"""
    x = np.ascontiguousarray(x, dtype=np.float32)
    cell = np.zeros(max(len(x), 1), np.int32)
    frac = np.zeros(max(len(x), 1), np.float64)
    lib().or_fold_many(len(x), _ptr(x), int(nf), int(f32), _ptr(cell), _ptr(frac))
    return cell[:len(x)], frac[:len(x)]


def bin_sort(xs, nf, bins, shift=None, scale=None, loc_dtype=np.float32, ns=0, bin_only=False):
    """Host replica of the device bin sort: (perm, loc[dim, M]); ns = the plan's
    kernel width (odd widths sort by the start cell of the support, the cell
    or the next one when the fraction is at least one half, when the keys fit
    32 bits); bin_only: the reference's ordering, bin index with x fastest and
    input order within a bin (include/cufinufft/spreadinterp.hpp:139-150,
    include/finufft/spread.hpp:459-584)."""
    dim = len(xs)
    float_inputs = all(np.asarray(x).dtype == np.float32 for x in xs)
    xs = _coords(xs)
    M = len(xs[0])
    shift = np.zeros(3) if shift is None else np.asarray(list(shift) + [0] * (3 - dim), np.float64)
    scale = np.ones(3) if scale is None else np.asarray(list(scale) + [1] * (3 - dim), np.float64)
    nfa = np.array(list(nf) + [1] * (3 - dim), dtype=np.int32)
    ba = np.array(list(bins) + [1] * (3 - dim), dtype=np.int32)
    perm = np.zeros(max(M, 1), dtype=np.int32)
    loc = np.zeros((dim, max(M, 1)), dtype=loc_dtype)
    lib().or_bin_sort(dim, M, _ptrs(xs), _ptr(shift), _ptr(scale), _ptr(nfa), _ptr(ba),
                      _ptr(perm), _ptr(loc), int(loc_dtype == np.float32), int(float_inputs),
                      int(ns), int(bin_only))
    return perm[:M], loc[:, :M]


# ------------------------------------------------ ES-kernel NUFFT (FP64) ----
def _fft_sign(grid, isign, axes):
    """sum_g grid[g] exp(isign 2 pi i k g / n) over the given axes"""
    if isign > 0:
        n = int(np.prod([grid.shape[a] for a in axes]))
        return np.fft.ifftn(grid, axes=axes) * n
    return np.fft.fftn(grid, axes=axes)


def _phihat_series(fun, ns, nf):
    k = np.arange(nf // 2 + 1)
    ph = kernel_ft(fun, ns, 2 * PI * k / nf, 3.0)
    return ph * np.where(k % 2 == 1, -1.0, 1.0)


def _spread(xs, c, nf, ns, beta, shift=None, scale=None, coef=None):
    dim = len(xs)
    xs = _coords(xs)
    c = _cplx(c)
    sh = np.zeros(3) if shift is None else np.asarray(list(shift) + [0] * (3 - dim), np.float64)
    sc = np.ones(3) if scale is None else np.asarray(list(scale) + [1] * (3 - dim), np.float64)
    nfa = np.array(list(nf) + [1] * (3 - dim), dtype=np.int32)
    grid = np.zeros(int(np.prod(nfa)), dtype=np.complex128)
    nco = 0 if coef is None else coef.shape[0]
    lib().or_spread_es(dim, len(xs[0]), _ptrs(xs), _ptr(sh), _ptr(sc), _ptr(c), _ptr(nfa), ns,
                       beta, nco, _ptr(coef), _ptr(grid))
    return grid.reshape(tuple(reversed(list(nf))))


def _interp(xs, grid, nf, ns, beta, shift=None, scale=None, coef=None):
    dim = len(xs)
    xs = _coords(xs)
    g = _cplx(grid).reshape(-1)
    sh = np.zeros(3) if shift is None else np.asarray(list(shift) + [0] * (3 - dim), np.float64)
    sc = np.ones(3) if scale is None else np.asarray(list(scale) + [1] * (3 - dim), np.float64)
    nfa = np.array(list(nf) + [1] * (3 - dim), dtype=np.int32)
    out = np.zeros(len(xs[0]), dtype=np.complex128)
    nco = 0 if coef is None else coef.shape[0]
    lib().or_interp_es(dim, len(xs[0]), _ptrs(xs), _ptr(sh), _ptr(sc), _ptr(g), _ptr(nfa), ns,
                       beta, nco, _ptr(coef), _ptr(out))
    return out


def _mode_index(n, modeord):
    """array of modes k for positions 0..n-1"""
    i = np.arange(n)
    return i - n // 2 if modeord == 0 else np.where(i < n - n // 2, i, i - n)


def _deconv_factor(n_modes, nf, ph, modeord):
    """prod_d 1/phihat_d(|k_d|) as an array of shape reversed(n_modes)"""
    f = None
    for d in range(len(n_modes)):
        k = _mode_index(n_modes[d], modeord)
        v = 1.0 / ph[d][np.abs(k)]
        shape = [1] * len(n_modes)
        shape[len(n_modes) - 1 - d] = n_modes[d]
        v = v.reshape(shape)
        f = v if f is None else f * v
    return f


def _grid_take(grid, n_modes, nf, modeord):
    idx = []
    for d in reversed(range(len(n_modes))):
        k = _mode_index(n_modes[d], modeord)
        idx.append(np.where(k >= 0, k, nf[d] + k))
    return grid[np.ix_(*idx)]


def nufft_es(nufft_type, xs, data, isign, tol, n_modes=None, ss=None, sigma=None,
             is_float=True, modeord=0, kernel="es"):
    """The GPU library's algorithm, entirely in FP64, with its ES kernel
    (kernel="es") or with the engine's default PSWF kernel (kernel="pswf").

    Types 1/2: n_modes (x fastest); data is c[M] (type 1) or f with shape
    reversed(n_modes) (type 2). Type 3: ss = target coordinates."""
    dim = len(xs)
    if sigma is None:
        # the engine's rule: 1.25 for type 3 at tol >= 1e-9, but in single
        # precision only at tol >= 1e-4 (compared in single precision)
        ok = np.float32(tol) >= np.float32(1e-4) if is_float else tol >= 1e-9
        sigma = 1.25 if (nufft_type == 3 and tol >= 1e-9 and ok) else 2.0
    ns, beta, fun, coef = engine_kernel(tol, sigma, dim, nufft_type, is_float, kernel)
    if nufft_type == 3 and kernel == "pswf":
        # the inner type-2 plan chooses its own (type-2) width
        ns2, beta2, fun2, coef2 = engine_kernel(tol, sigma, dim, 2, is_float, kernel)
    else:
        ns2, beta2, fun2, coef2 = ns, beta, fun, coef
    if nufft_type in (1, 2):
        nf = [fine_grid(m, sigma, ns) for m in n_modes]
        ph = [_phihat_series(fun, ns, n) for n in nf]
        axes = tuple(range(dim))
        if nufft_type == 1:
            G = _fft_sign(_spread(xs, data, nf, ns, beta, coef=coef), isign, axes)
            return _grid_take(G, n_modes, nf, modeord) * _deconv_factor(n_modes, nf, ph, modeord)
        fk = np.asarray(data, dtype=np.complex128).reshape(tuple(reversed(list(n_modes))))
        grid = np.zeros(tuple(reversed(nf)), dtype=np.complex128)
        idx = []
        for d in reversed(range(dim)):
            k = _mode_index(n_modes[d], modeord)
            idx.append(np.where(k >= 0, k, nf[d] + k))
        grid[np.ix_(*idx)] = fk * _deconv_factor(n_modes, nf, ph, modeord)
        return _interp(xs, _fft_sign(grid, isign, axes), nf, ns, beta, coef=coef)
    # type 3
    xs, ss = _coords(xs), _coords(ss)
    X, C, S, D = [], [], [], []
    for d in range(dim):
        w, c0 = width_center(xs[d].min(), xs[d].max())
        X.append(w), C.append(c0)
        w, c0 = width_center(ss[d].min(), ss[d].max())
        S.append(w), D.append(c0)
    nf, h, gam = [], [], []
    for d in range(dim):
        a, b, g = type3_grid(sigma, X[d], S[d], ns)
        nf.append(a), h.append(b), gam.append(g)
    pre = np.exp(1j * isign * sum(D[d] * xs[d] for d in range(dim)))
    grid = _spread(xs, np.asarray(data) * pre, nf, ns, beta, shift=C, scale=[1 / g for g in gam],
                   coef=coef)
    # inner type 2 on the grid (mode m at position m + nf/2) at s' = h gam (s - D)
    sp = [h[d] * gam[d] * (ss[d] - D[d]) for d in range(dim)]
    nf2 = [fine_grid(n, sigma, ns2) for n in nf]
    ph2 = [_phihat_series(fun2, ns2, n) for n in nf2]
    g2 = np.zeros(tuple(reversed(nf2)), dtype=np.complex128)
    idx = []
    for d in reversed(range(dim)):
        k = _mode_index(nf[d], 0)
        idx.append(np.where(k >= 0, k, nf2[d] + k))
    g2[np.ix_(*idx)] = grid * _deconv_factor(nf, nf2, ph2, 0)
    vals = _interp(sp, _fft_sign(g2, isign, tuple(range(dim))), nf2, ns2, beta2, coef=coef2)
    phis = np.ones(len(ss[0]))
    for d in range(dim):
        phis = phis * kernel_ft(fun, ns, sp[d], 2.0)
    post = np.exp(1j * isign * sum(C[d] * (ss[d] - D[d]) for d in range(dim))) / phis
    return vals * post


# ------------------------------------------- CPU FINUFFT restatement (PSWF) ----
class CpuPlan:
    """The CPU library's pipeline with its PSWF kernel (sigma fixed, default 2):
    bin sort at setpts, then spread (OpenMP C) -> FFT (scipy, all threads) ->
    deconvolve, or the reverse for type 2. Precision follows dtype.
    Type 3 (n_modes = the dimension): see CpuPlan3."""

    def __new__(cls, nufft_type, *args, **kw):
        if nufft_type == 3 and cls is CpuPlan:
            return CpuPlan3(*args, **kw)
        return super().__new__(cls)

    def __init__(self, nufft_type, n_modes, isign, tol, dtype=np.complex64, sigma=2.0,
                 threads=None, maxsub=10000):
        assert nufft_type in (1, 2)
        self.type, self.n_modes, self.isign, self.tol = nufft_type, list(n_modes), isign, tol
        self.dim = len(n_modes)
        self.is_float = np.dtype(dtype) == np.complex64
        self.cdt = np.complex64 if self.is_float else np.complex128
        self.rdt = np.float32 if self.is_float else np.float64
        self.ns, self.beta = cpu_kernel(tol, self.dim, nufft_type, sigma, self.is_float)
        self.fun = lambda x: pswf0(self.beta, 2.0 * np.asarray(x) / self.ns)
        self.ncoef = self.ns + 4
        self.coef = np.ascontiguousarray(horner_table(self.fun, self.ns, self.ncoef))
        self.nf = [fine_grid(m, sigma, self.ns) for m in n_modes]
        ph = [_phihat_series(self.fun, self.ns, n) for n in self.nf]
        self.dec = _deconv_factor(self.n_modes, self.nf, ph, 0).astype(self.rdt)
        self.threads = threads or lib().or_num_threads()
        self.maxsub = maxsub

    def setpts(self, xs):
        self.xs = [np.ascontiguousarray(a, dtype=self.rdt) for a in xs]
        self.M = len(self.xs[0])
        self.perm = np.zeros(max(self.M, 1), dtype=np.int32)
        nfa = np.array(self.nf + [1] * (3 - self.dim), dtype=np.int32)
        self._nfa = nfa
        self._px = _ptrs(self.xs)
        suf = "f" if self.is_float else "d"
        getattr(lib(), "or_cpu_sort_" + suf)(self.dim, self.M, self._px, _ptr(nfa), _ptr(self.perm))

    def execute(self, data):
        import scipy.fft as sfft

        suf = "f" if self.is_float else "d"
        axes = tuple(range(self.dim))
        shape = tuple(reversed(self.nf))
        if self.type == 1:
            c = np.ascontiguousarray(data, dtype=self.cdt)
            grid = np.zeros(shape, dtype=self.cdt)
            getattr(lib(), "or_cpu_spread_" + suf)(
                self.dim, self.M, self._px, _ptr(self.perm), _ptr(c), _ptr(self._nfa), self.ns,
                self.ncoef, _ptr(self.coef), self.maxsub, _ptr(grid))
            if self.isign > 0:
                G = sfft.ifftn(grid, axes=axes, workers=self.threads, norm="forward", overwrite_x=True)
            else:
                G = sfft.fftn(grid, axes=axes, workers=self.threads, overwrite_x=True)
            return _grid_take(G, self.n_modes, self.nf, 0) * self.dec
        fk = np.asarray(data, dtype=self.cdt).reshape(tuple(reversed(self.n_modes)))
        grid = np.zeros(shape, dtype=self.cdt)
        idx = []
        for d in reversed(range(self.dim)):
            k = _mode_index(self.n_modes[d], 0)
            idx.append(np.where(k >= 0, k, self.nf[d] + k))
        grid[np.ix_(*idx)] = fk * self.dec
        if self.isign > 0:
            G = sfft.ifftn(grid, axes=axes, workers=self.threads, norm="forward", overwrite_x=True)
        else:
            G = sfft.fftn(grid, axes=axes, workers=self.threads, overwrite_x=True)
        G = np.ascontiguousarray(G, dtype=self.cdt)
        out = np.zeros(self.M, dtype=self.cdt)
        getattr(lib(), "or_cpu_interp_" + suf)(
            self.dim, self.M, self._px, _ptr(self.perm), _ptr(G), _ptr(self._nfa), self.ns,
            self.ncoef, _ptr(self.coef), _ptr(out))
        return out


class CpuPlan3:
    """The CPU library's type 3 (include/finufft/setpts.hpp:163-319 and
    execute.hpp type-3 branch) with its PSWF kernel: sources rescaled to
    x' = (x - C)/gamma, pre-phase exp(i isign D.x), spread onto the outer grid
    of nhg_type3 (type-3 kernel width), an inner type-2 CpuPlan at the same tol
    on that grid evaluated at s' = h gamma (s - D), and the post factor
    exp(i isign (s - D).C) / prod phihat(s'). sigma is fixed (default 2; the
    CPU library picks it by a cost model at setpts)."""

    def __init__(self, dim, isign, tol, dtype=np.complex64, sigma=2.0, threads=None,
                 maxsub=10000):
        self.dim, self.isign, self.tol, self.sigma = int(dim), isign, tol, sigma
        self.is_float = np.dtype(dtype) == np.complex64
        self.cdt = np.complex64 if self.is_float else np.complex128
        self.rdt = np.float32 if self.is_float else np.float64
        self.ns, self.beta = cpu_kernel(tol, self.dim, 3, sigma, self.is_float)
        self.fun = lambda x: pswf0(self.beta, 2.0 * np.asarray(x) / self.ns)
        self.ncoef = self.ns + 4
        self.coef = np.ascontiguousarray(horner_table(self.fun, self.ns, self.ncoef))
        self.threads = threads or lib().or_num_threads()
        self.maxsub = maxsub
        self.dtype = dtype

    def setpts(self, xs, ss):
        dim = self.dim
        xs = [np.asarray(a, dtype=np.float64) for a in xs]
        ss = [np.asarray(a, dtype=np.float64) for a in ss]
        self.M, self.N = len(xs[0]), len(ss[0])
        X, C, S, D = [], [], [], []
        for d in range(dim):
            w, c0 = width_center(xs[d].min(), xs[d].max()) if self.M else (0.0, 0.0)
            X.append(w), C.append(c0)
            w, c0 = width_center(ss[d].min(), ss[d].max()) if self.N else (0.0, 0.0)
            S.append(w), D.append(c0)
        self.nf, h, gam = [], [], []
        for d in range(dim):
            a, b, g = type3_grid(self.sigma, X[d], S[d], self.ns)
            self.nf.append(a), h.append(b), gam.append(g)
        self.xp = [np.ascontiguousarray((xs[d] - C[d]) / gam[d], dtype=self.rdt)
                   for d in range(dim)]
        self.pre = np.exp(1j * self.isign * sum(D[d] * xs[d] for d in range(dim))).astype(self.cdt)
        sp = [h[d] * gam[d] * (ss[d] - D[d]) for d in range(dim)]
        phis = np.ones(self.N)
        for d in range(dim):
            phis = phis * kernel_ft(self.fun, self.ns, sp[d], 2.0)
        self.post = (np.exp(1j * self.isign * sum(C[d] * (ss[d] - D[d]) for d in range(dim)))
                     / phis).astype(self.cdt)
        self.perm = np.zeros(max(self.M, 1), dtype=np.int32)
        self._nfa = np.array(self.nf + [1] * (3 - dim), dtype=np.int32)
        self._px = _ptrs(self.xp)
        suf = "f" if self.is_float else "d"
        getattr(lib(), "or_cpu_sort_" + suf)(dim, self.M, self._px, _ptr(self._nfa),
                                             _ptr(self.perm))
        self.inner = CpuPlan(2, self.nf, self.isign, self.tol, dtype=self.dtype,
                             sigma=self.sigma, threads=self.threads, maxsub=self.maxsub)
        self.inner.setpts([np.ascontiguousarray(a, dtype=self.rdt) for a in sp])

    def execute(self, c):
        suf = "f" if self.is_float else "d"
        cp = np.ascontiguousarray(np.asarray(c, dtype=self.cdt) * self.pre)
        grid = np.zeros(tuple(reversed(self.nf)), dtype=self.cdt)
        getattr(lib(), "or_cpu_spread_" + suf)(
            self.dim, self.M, self._px, _ptr(self.perm), _ptr(cp), _ptr(self._nfa), self.ns,
            self.ncoef, _ptr(self.coef), self.maxsub, _ptr(grid))
        return self.inner.execute(grid) * self.post
