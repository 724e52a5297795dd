"""Build the GB300 NUFFT engine: one shared library, libcufinufft.so, in-tree.

The library exports the cufinufft_* device API, the finufft_* host API and the
gbnufft extensions (include/*.h). Device code is compiled for sm_103a only;
translation units are compiled in parallel and linked with cuFFT.

Usage: python -m finufft_gb300.build   (or finufft_gb300.build.build())
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcufinufft.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

CU_SOURCES = [
    "sort.cu",
    "elementwise.cu",
    "spreadinterp_1d.cu",
    "spreadinterp_2d.cu",
    "spreadinterp_3d.cu",
    "noalloc.cu",
    "batch.cu",
    "planner.cu",
]
CPP_SOURCES = ["planning.cpp", "plan.cpp", "c_api.cpp", "host_api.cpp"]


def _nvcc():
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the GB300 engine needs the CUDA toolkit")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(obj, src_files):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in src_files)


def build(verbose=False, force=False, extra_nvcc=()):
    """Compile every translation unit (in parallel) and link libcufinufft.so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    headers += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    common = ["-O3", "-std=c++20", "-I", INC, "-I", CSRC, "-DNDEBUG"]
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        cmd = [nvcc, *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills",
               "-Xcompiler", "-fvisibility=hidden", *extra_nvcc,
               "-c", s, "-o", o]
        jobs.append((o, [s] + headers, cmd))
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        cmd = ["g++", *common, "-fPIC", "-fvisibility=hidden", "-ffp-contract=off",
               "-I", os.path.join(CUDA_HOME, "include"), "-c", s, "-o", o]
        jobs.append((o, [s] + headers, cmd))
    todo = [j for j in jobs if force or _stale(j[0], j[1])]
    logs = []
    if todo:
        with ThreadPoolExecutor(max_workers=max(2, min(len(todo), os.cpu_count() or 4))) as ex:
            for log in ex.map(lambda j: _run(j[2]), todo):
                logs.append(log)
    objs = [j[0] for j in jobs]
    if force or todo or not os.path.exists(LIB):
        # SONAME libcufinufft.so: ctypes.util.find_library (the reference Python
        # binding's system-path lookup) reports a library by its SONAME
        link = [nvcc, *ARCH, "-shared", "-Xlinker", "-soname=libcufinufft.so", "-o", LIB, *objs,
                "-lcufft", "-lcudart"]
        logs.append(_run(link))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
