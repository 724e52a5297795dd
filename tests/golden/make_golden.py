"""Generate tests/golden/reference_planning.json from the REFERENCE's own code.

Runs only where the reference source tree is present: it builds
oracle/_ref/libfinufft_common.so from flatironinstitute/finufft's
src/common/{utils,kernel,pswf}.cpp (oracle/Makefile, target `ref`) and records
what those functions return. The committed JSON pins the oracle's restatement
(tests/test_oracle.py) on machines without the reference.

Usage: python tests/golden/make_golden.py
"""
import ctypes
import json
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
ORACLE = os.path.join(ROOT, "oracle")


def main():
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    L = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libfinufft_common.so"))
    L.ref_next235.argtypes = [ctypes.c_longlong, ctypes.c_longlong]
    L.ref_next235.restype = ctypes.c_longlong
    P = ctypes.c_void_p
    L.ref_gaussquad.argtypes = [ctypes.c_int, P, P]
    L.ref_nhg_type3.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, P]
    L.ref_cpu_kernel.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, P]
    L.ref_cpu_kernel.restype = ctypes.c_int
    L.ref_pswf.argtypes = [ctypes.c_double, ctypes.c_int, P, P]
    out = {"source": "flatironinstitute/finufft src/common (compiled from the reference tree)"}
    ns = list(range(0, 200)) + [1000, 12345, 65537, 10 ** 6 + 1, 2 ** 31 + 11, 3 * 10 ** 9]
    out["next235_even"] = [[n, int(L.ref_next235(n, 2))] for n in ns]
    gq = {}
    for n in (2, 5, 16, 27, 40, 64):
        x, w = np.zeros(n), np.zeros(n)
        L.ref_gaussquad(n, x.ctypes.data, w.ctypes.data)
        gq[str(n)] = [x.tolist(), w.tolist()]
    out["gaussquad"] = gq
    t3 = []
    for sigma in (1.25, 2.0):
        for X, S in ((1.0, 200.0), (2.0, 100.0), (4.0, 50.0), (0.0, 0.0), (0.0, 5.0), (3.0, 0.0),
                     (1e-3, 1e-3), (np.pi, 64.0)):
            for nsp in (4, 7, 10, 13):
                r = np.zeros(3)
                L.ref_nhg_type3(sigma, X, S, nsp, r.ctypes.data)
                t3.append([sigma, X, S, nsp, int(r[0]), r[1], r[2]])
    out["nhg_type3"] = t3
    ck = []
    for tol in (1e-2, 1e-4, 1e-5, 1e-6, 1e-9, 1e-12, 1e-14):
        for dim in (1, 2, 3):
            for ty in (1, 3):
                for sigma in (1.25, 2.0):
                    b = np.zeros(1)
                    n = L.ref_cpu_kernel(tol, dim, ty, sigma, b.ctypes.data)
                    ck.append([tol, dim, ty, sigma, n, b[0]])
    out["cpu_kernel"] = ck
    z = np.linspace(-1, 1, 41)
    ps = {}
    for c in (5.0, 14.09, 20.0, 30.0, 45.0):
        v = np.zeros_like(z)
        L.ref_pswf(c, len(z), z.ctypes.data, v.ctypes.data)
        ps[repr(c)] = v.tolist()
    out["pswf"] = {"z": z.tolist(), "values": ps}
    path = os.path.join(ROOT, "tests", "golden", "reference_planning.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", path)


if __name__ == "__main__":
    main()
