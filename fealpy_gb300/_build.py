"""Build recipe for the in-tree CUDA library ``fealpy_gb300/_lib/libfealpy_gb300.so``.

The kernels are plain CUDA C++ with an ``extern "C"`` surface
(``include/fealpy_gb300.h``); they are compiled for sm_103a only, one
translation unit per process in parallel, and linked into one shared library
that :mod:`fealpy_gb300._lib` loads with ctypes.  No torch headers are used, so
the build takes a few seconds and does not depend on the PyTorch version.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(OUT_DIR, "build")
LIB_NAME = "libfealpy_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fealpy_gb300")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    """Compile every ``csrc/*.cu`` for sm_103a and link the shared library.

    Returns the library path.  Object files are reused when newer than their
    source and the shared headers.
    """
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "fealpy_gb300.h"))
    flags = ARCH_FLAGS + COMMON_FLAGS + list(extra_flags or [])
    srcs = sources()
    objs = []
    jobs = []
    for src in srcs:
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr, flush=True)
        return res

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not _newer(LIB_PATH, objs):
        run([nvcc] + ARCH_FLAGS + ["-shared", "-o", LIB_PATH] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
