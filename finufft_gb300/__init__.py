"""GB300-native NUFFT engine (types 1, 2, 3 in 1D/2D/3D).

The compute path is the in-tree CUDA library ``_build/libcufinufft.so``, a
drop-in for cufinufft's C ABI. This module mirrors the reference's Python
front end (python/cufinufft/cufinufft/_plan.py: ``Plan(nufft_type, n_modes,
n_trans, eps, isign, dtype, **opts)`` with ``setpts`` and ``execute``) on
torch CUDA tensors. Axis conventions are the reference's: arrays are
row-major, so the last axis of ``n_modes`` is the fastest one and the point
coordinates are handed to the C layer in reverse order.
"""
import ctypes
import numbers

from . import _lib

__all__ = ["Plan", "load_library", "smem_atomic_peak", "ERRORS"]

ERRORS = {
    2: "FINUFFT_ERR_MAXNALLOC", 3: "FINUFFT_ERR_SPREAD_BOX_SMALL", 6: "FINUFFT_ERR_SPREAD_DIR",
    7: "FINUFFT_ERR_UPSAMPFAC_TOO_SMALL", 8: "FINUFFT_ERR_HORNER_WRONG_BETA",
    9: "FINUFFT_ERR_NTRANS_NOTVALID", 10: "FINUFFT_ERR_TYPE_NOTVALID",
    11: "FINUFFT_ERR_ALLOC", 12: "FINUFFT_ERR_DIM_NOTVALID",
    14: "FINUFFT_ERR_NDATA_NOTVALID", 15: "FINUFFT_ERR_CUDA_FAILURE",
    16: "FINUFFT_ERR_PLAN_NOTVALID", 17: "FINUFFT_ERR_METHOD_NOTVALID",
    18: "FINUFFT_ERR_BINSIZE_NOTVALID", 19: "FINUFFT_ERR_INSUFFICIENT_SHMEM",
    20: "FINUFFT_ERR_NUM_NU_PTS_INVALID", 21: "FINUFFT_ERR_INVALID_ARGUMENT",
    25: "FINUFFT_ERR_UNKNOWN_EXCEPTION", 26: "FINUFFT_ERR_EPS_TOO_SMALL",
}


def load_library():
    return _lib.load()


def smem_atomic_peak(device=0, i32=False):
    """Measured conflict-free shared-memory atomicAdd rate (lane ops/s): f32,
    or native int32 (the fixed-point tile's operation) with i32=True."""
    r = ctypes.c_double()
    lib = _lib.load()
    fn = lib.gbnufft_smem_atomic_rate_i32 if i32 else lib.gbnufft_smem_atomic_rate
    _check("smem_atomic_rate", fn(device, ctypes.byref(r)))
    return r.value


class NufftError(RuntimeError):
    def __init__(self, what, code):
        super().__init__("%s failed: %s (%d)" % (what, ERRORS.get(code, "error"), code))
        self.code = code


def _check(what, ier):
    if ier != 0:
        raise NufftError(what, ier)


class Plan:
    """A planned NUFFT on the GPU (same call pattern as ``cufinufft.Plan``)."""

    def __init__(self, nufft_type, n_modes, n_trans=1, eps=1e-6, isign=None,
                 dtype="complex64", **kwargs):
        import torch

        lib = _lib.load()
        self._plan = None
        if isign is None:
            isign = -1 if nufft_type == 2 else +1
        if dtype in ("complex64", torch.complex64):
            self._pfx, self._real, self._cplx = "cufinufftf", torch.float32, torch.complex64
        elif dtype in ("complex128", torch.complex128):
            self._pfx, self._real, self._cplx = "cufinufft", torch.float64, torch.complex128
        else:
            raise TypeError("Expected complex64 or complex128.")
        if nufft_type == 3:
            if not isinstance(n_modes, numbers.Integral):
                raise ValueError("For a type 3 plan, n_modes_or_dim must be the dimension")
            dim, n_modes = int(n_modes), (1,) * int(n_modes)
        else:
            n_modes = (n_modes,) if isinstance(n_modes, numbers.Integral) else tuple(n_modes)
            dim = len(n_modes)
        if dim not in (1, 2, 3):
            raise ValueError("Only dimensions 1, 2, and 3 supported")
        self.type, self.dim, self.n_modes, self.n_trans = nufft_type, dim, n_modes, n_trans
        self.isign, self.eps = isign, float(eps)
        self.opts = _lib.default_opts()
        self.ext = _lib.default_ext_opts()
        names = [n for n, _ in self.opts._fields_]
        ext_names = [n for n, _ in self.ext._fields_ if n != "reserved"]
        for k, v in kwargs.items():
            if k in names:
                setattr(self.opts, k, v)
            elif k in ext_names:
                setattr(self.ext, k, v)
            else:
                raise TypeError("Invalid option '%s'" % k)
        modes = (ctypes.c_int64 * 3)(*(list(reversed(n_modes)) + [1] * (3 - dim)))
        plan = ctypes.c_void_p()
        ier = getattr(lib, self._pfx + "_makeplan_ext")(
            nufft_type, dim, modes, isign, n_trans, self.eps, ctypes.byref(plan),
            ctypes.byref(self.opts), ctypes.byref(self.ext))
        _check("makeplan", ier)
        self._plan = plan
        self._lib = lib
        self._refs = []
        self.nj = self.nk = 0

    def _vec(self, a, name):
        import torch

        if a is None:
            return None
        if not isinstance(a, torch.Tensor) or not a.is_cuda:
            raise TypeError("Argument `%s` must be a CUDA tensor" % name)
        if a.dtype != self._real:
            raise TypeError("Argument `%s` has dtype %s, expected %s" % (name, a.dtype, self._real))
        return a.contiguous().reshape(-1)

    def setpts(self, x, y=None, z=None, s=None, t=None, u=None):
        pts = [self._vec(v, n) for v, n in ((x, "x"), (y, "y"), (z, "z"))]
        if sum(p is not None for p in pts) != self.dim or pts[0] is None:
            raise TypeError("Plan dimension is %d: pass exactly that many coordinates" % self.dim)
        axes = list(reversed(pts[: self.dim])) + [None] * (3 - self.dim)
        M = axes[0].numel()
        if any(a is not None and a.numel() != M for a in axes):
            raise TypeError("coordinate arrays must have equal length")
        N, taxes = 0, [None] * 3
        if self.type == 3:
            tp = [self._vec(v, n) for v, n in ((s, "s"), (t, "t"), (u, "u"))]
            if sum(p is not None for p in tp) != self.dim:
                raise TypeError("type 3 needs %d target coordinates" % self.dim)
            taxes = list(reversed(tp[: self.dim])) + [None] * (3 - self.dim)
            N = taxes[0].numel()
        ptr = lambda a: a.data_ptr() if a is not None else None
        ier = getattr(self._lib, self._pfx + "_setpts")(
            self._plan, M, ptr(axes[0]), ptr(axes[1]), ptr(axes[2]), N, ptr(taxes[0]),
            ptr(taxes[1]), ptr(taxes[2]))
        _check("setpts", ier)
        self._refs = [a for a in axes + taxes if a is not None]
        self.nj, self.nk = M, N

    def _shapes(self, adjoint):
        modes = tuple(self.n_modes)
        src = (self.n_trans, self.nj)
        dst = (self.n_trans,) + (modes if self.type != 3 else (self.nk,))
        if self.type == 2:
            src, dst = dst, src
        return (dst, src) if adjoint else (src, dst)

    def _run(self, data, out, adjoint):
        import torch

        if not isinstance(data, torch.Tensor) or not data.is_cuda or data.dtype != self._cplx:
            raise TypeError("`data` must be a CUDA tensor of dtype %s" % self._cplx)
        in_shape, out_shape = self._shapes(adjoint)
        single = self.n_trans == 1 and data.dim() == len(in_shape) - 1
        data = data.contiguous().reshape(in_shape)
        if out is None:
            out = torch.empty(out_shape, dtype=self._cplx, device=data.device)
        elif out.numel() != int(torch.tensor(out_shape).prod()) or not out.is_contiguous():
            raise TypeError("`out` must be contiguous with %s elements" % (out_shape,))
        # C order of arguments: (c, fk); c holds the points side
        points_side_is_input = (self.type != 2) != adjoint
        c, fk = (data, out) if points_side_is_input else (out, data)
        name = "_execute_adjoint" if adjoint else "_execute"
        ier = getattr(self._lib, self._pfx + name)(self._plan, c.data_ptr(), fk.data_ptr())
        _check(name[1:], ier)
        res = out.reshape(out_shape)
        return res[0] if single else res

    def execute(self, data, out=None):
        return self._run(data, out, False)

    def execute_adjoint(self, data, out=None):
        return self._run(data, out, True)

    def info(self):
        i = _lib.PlanInfo()
        _check("plan_info", getattr(self._lib, self._pfx + "_plan_info")(self._plan, ctypes.byref(i)))
        return i

    def stage_times(self, enable=True):
        ms = (ctypes.c_float * 4)()
        _check("stage_times", getattr(self._lib, self._pfx + "_stage_times")(self._plan, int(enable), ms))
        return list(ms)

    def graph_capture(self, c, fk):
        _check("graph_capture", getattr(self._lib, self._pfx + "_graph_capture")(
            self._plan, c.data_ptr(), fk.data_ptr()))

    def graph_launch(self):
        _check("graph_launch", getattr(self._lib, self._pfx + "_graph_launch")(self._plan))

    def __del__(self):
        if getattr(self, "_plan", None) is not None:
            try:
                getattr(self._lib, self._pfx + "_destroy")(self._plan)
            except Exception:
                pass
            self._plan = None
