"""CPU checks of the C-ABI library: it loads, exports every entry point that
include/*.h declares, and its host-only paths (option defaults, argument
validation that precedes any device work) behave as the reference's."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = ["cufinufft.h", "finufft.h", "gbnufft_ext.h"]


def declared_symbols():
    """Names declared with GBNUFFT_EXPORT, found by preprocessing the headers."""
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    names = set()
    for h in HEADERS:
        src = '#define GBNUFFT_EXPORT __gbx__\n#include "%s"\n' % h
        out = subprocess.run(["gcc", "-E", "-P", "-x", "c", "-I", os.path.join(ROOT, "include"),
                              "-I", cuda_inc, "-"], input=src, capture_output=True, text=True,
                             check=True).stdout
        names |= set(re.findall(r"__gbx__[^;(]*?\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", out))
        names |= set(re.findall(r"__gbx__\s+extern\s+const\s+int\s+([A-Za-z_][A-Za-z0-9_]*)", out))
    return sorted(names)


def test_headers_declare_the_reference_surface():
    names = declared_symbols()
    cu = [n for n in names if n.startswith("cufinufft")]
    # 45 cufinufft* symbols of the reference (include/cufinufft.h) + 12 extensions
    base = [n for n in cu if not re.search(r"(adjoint|plan_info|stage_times|get_sort|graph_|_ext$|noalloc|_batch_)", n)]
    assert len(base) == 45
    host = [n for n in names if n.startswith("finufft")]
    assert len(host) == 12 + 36  # guru (6 x 2) + simple (18 x 2)
    assert "FINUFFT_FFT_DEFAULT" in names


def test_library_exports_every_declared_symbol(engine):
    missing = [n for n in declared_symbols() if not hasattr(engine, n)]
    assert missing == []


def test_cufinufft_default_opts(engine):
    from finufft_gb300 import _lib

    o = _lib.default_opts()
    # src/cuda/c_interface.cpp:151-173
    assert o.gpu_method == 0 and o.gpu_sort == 1 and o.gpu_kerevalmeth == 1
    assert o.upsampfac == 0.0 and o.gpu_maxsubprobsize == 1024 and o.gpu_maxbatchsize == 0
    assert o.gpu_binsizex == o.gpu_binsizey == o.gpu_binsizez == 0
    assert o.modeord == 0 and o.gpu_spreadinterponly == 0 and o.gpu_np == 0 and o.debug == 0
    assert ctypes.sizeof(o) == 88  # 8 + 13 ints, pad, stream pointer, 3 ints, pad


def test_finufft_default_opts(engine):
    from finufft_gb300 import _lib

    o = _lib.FinufftOpts()
    engine.finufft_default_opts(ctypes.byref(o))
    assert o.showwarn == 1 and o.spread_sort == 2 and o.spread_nthr_atomic == -1
    assert o.upsampfac == 0.0 and o.maxbatchsize == 0 and o.allow_eps_too_small == 0


def _mk(engine, pfx, ty, dim, modes, ntr=1, tol=1e-6):
    p = ctypes.c_void_p()
    m = (ctypes.c_int64 * 3)(*modes)
    fn = getattr(engine, pfx + "_makeplan")
    return fn(ty, dim, m, 1, ntr, tol, ctypes.byref(p), None)


@pytest.mark.parametrize("pfx", ["cufinufft", "cufinufftf"])
def test_device_api_host_side_errors(engine, pfx):
    # test/cuda/test_makeplan.c: checks that precede any device work
    assert _mk(engine, pfx, 1, 0, (10, 20, 15)) == 12  # FINUFFT_ERR_DIM_NOTVALID
    assert _mk(engine, pfx, 1, 4, (10, 20, 15)) == 12
    assert _mk(engine, pfx, 1, 1, (0, 20, 15)) == 14  # FINUFFT_ERR_NDATA_NOTVALID
    assert _mk(engine, pfx, 1, 1, (2 ** 31, 1, 1)) == 14
    assert _mk(engine, pfx, 1, 2, (10, 0, 1)) == 14
    assert _mk(engine, pfx, 1, 2, (2 ** 31 - 1, 2, 1)) == 14
    assert _mk(engine, pfx, 1, 3, (10, 15, 0)) == 14
    assert _mk(engine, pfx, 1, 3, (2 ** 30, 2, 2)) == 14
    assert getattr(engine, pfx + "_destroy")(None) == 16  # FINUFFT_ERR_PLAN_NOTVALID
    assert getattr(engine, pfx + "_setpts")(None, 10, None, None, None, 0, None, None, None) == 16
    assert getattr(engine, pfx + "_setpts")(None, 2 ** 31, None, None, None, 0, None, None, None) == 14
    assert getattr(engine, pfx + "_execute")(None, None, None) == 16


@pytest.mark.parametrize("pfx", ["finufft", "finufftf"])
def test_host_api_host_side_errors(engine, pfx):
    assert _mk(engine, pfx, 4, 1, (10, 1, 1)) == 10  # FINUFFT_ERR_TYPE_NOTVALID
    assert _mk(engine, pfx, 1, 0, (10, 1, 1)) == 12
    assert _mk(engine, pfx, 1, 1, (10, 1, 1), ntr=0) == 9  # FINUFFT_ERR_NTRANS_NOTVALID
    assert _mk(engine, pfx, 1, 1, (10, 1, 1), tol=1e-30) == 26  # FINUFFT_ERR_EPS_TOO_SMALL
    assert getattr(engine, pfx + "_destroy")(None) == 16


def test_pswf_kernel_values_against_reference(engine):
    """the engine's PSWF (the CPU library's kernel, which the default plans fit
    their Horner pieces to) equals the reference's own psi_0 (src/common/pswf.cpp,
    golden values generated from the reference tree) to rounding"""
    import json

    import numpy as np

    g = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_planning.json")))
    z = np.array(g["pswf"]["z"])
    for c, vals in g["pswf"]["values"].items():
        ns = 8
        x = np.ascontiguousarray(z * ns / 2)
        out = np.zeros_like(x)
        assert engine.gbnufft_kernel_eval(2, ns, float(c), len(x), x.ctypes.data,
                                          out.ctypes.data) == 0
        assert np.abs(out - np.array(vals)).max() < 2e-15, c


def test_kernel_choice_rules(engine, oracle):
    """width/shape rules: the ES form is the GPU library's (src/cuda/makeplan.cu:
    43-119), the PSWF form the CPU library's (src/common/kernel.cpp:79-146,
    golden values from the reference) widened to the GPU rule where that is
    wider, as the oracle's engine_kernel states it"""
    import json

    g = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_planning.json")))
    ns, beta = ctypes.c_int(), ctypes.c_double()
    for tol, dim, ty, sigma, ref_ns, ref_beta in g["cpu_kernel"]:
        for f32 in (0, 1):
            assert engine.gbnufft_kernel_choice(tol, sigma, dim, ty, f32, 2, 0, ctypes.byref(ns),
                                                ctypes.byref(beta)) == 0
            want = oracle.engine_kernel(tol, sigma, dim, ty, bool(f32), "pswf")
            assert (ns.value, beta.value) == (want[0], pytest.approx(want[1], rel=1e-14))
            gpu_ns = oracle.gpu_kernel(max(tol, 1.2e-7 if f32 else 2.3e-16), sigma, 0, bool(f32))[0]
            if ref_ns <= (12 if f32 else 16) and tol >= (1.2e-7 if f32 else 2.3e-16):
                assert ns.value == max(ref_ns, gpu_ns)
                if ns.value == ref_ns:
                    assert beta.value == pytest.approx(ref_beta, rel=1e-14)
        assert engine.gbnufft_kernel_choice(tol, sigma, dim, ty, 0, 1, 0, ctypes.byref(ns),
                                            ctypes.byref(beta)) == 0
        want = oracle.gpu_kernel(tol, sigma, 0, False)
        assert (ns.value, beta.value) == (want[0], pytest.approx(want[1], rel=1e-12))
    # kerformula: 7, 8, 9 are PSWF shape choices; 1-6 (the removed kernels) are errors
    for kf in (7, 8, 9):
        assert engine.gbnufft_kernel_choice(1e-6, 2.0, 2, 1, 0, 2, kf, ctypes.byref(ns),
                                            ctypes.byref(beta)) == 0
    assert engine.gbnufft_kernel_choice(1e-6, 2.0, 2, 1, 0, 2, 3, ctypes.byref(ns),
                                        ctypes.byref(beta)) == 24  # KERFORMULA_NOTVALID
