"""The reference's own Python binding (python/cufinufft, loaded unchanged from
the reference tree) finds this library through its system-path lookup and
binds its entry points: the drop-in check for ctypes callers. No GPU call is
made (only cufinufft_default_opts). Skipped where the reference tree is absent."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_dir():
    """the reference source tree: FINUFFT_REFERENCE_DIR, else the oracle
    Makefile's default"""
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"],
                       capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


REF_PY = os.path.join(_reference_dir(), "python", "cufinufft")
LIB_DIR = os.path.join(ROOT, "finufft_gb300", "_build")

PROBE = r"""
import ctypes, json
import cufinufft
from cufinufft import _cufinufft as b
o = b.NufftOpts()
b._default_opts(o)
fs = sorted(n for n in dir(b) if isinstance(getattr(b, n), ctypes._CFuncPtr))
print(json.dumps({"lib": b.lib._name, "sizeof": ctypes.sizeof(o), "maxsub": o.gpu_maxsubprobsize,
                  "method": o.gpu_method, "sort": o.gpu_sort, "kereval": o.gpu_kerevalmeth,
                  "upsampfac": o.upsampfac, "funcs": fs, "plan": cufinufft.Plan.__name__}))
"""


def test_reference_python_binding_loads_this_library():
    pytest.importorskip("packaging")
    if not os.path.isdir(REF_PY):
        pytest.skip("reference tree not present")
    if not os.path.exists(os.path.join(LIB_DIR, "libcufinufft.so")):
        pytest.skip("library not built")
    env = dict(os.environ, PYTHONPATH=REF_PY, LD_LIBRARY_PATH=LIB_DIR)
    r = subprocess.run([sys.executable, "-c", PROBE], env=env, capture_output=True, text=True,
                       cwd="/tmp", timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    import json

    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["lib"] == "libcufinufft.so"
    assert d["sizeof"] == 88
    # reference defaults (src/cuda/c_interface.cpp:151-173)
    assert (d["maxsub"], d["method"], d["sort"], d["kereval"], d["upsampfac"]) == (1024, 0, 1, 1, 0.0)
    assert {"_make_plan", "_make_planf", "_set_pts", "_set_ptsf", "_exec_plan", "_exec_planf",
            "_destroy_plan", "_destroy_planf"} <= set(d["funcs"])
