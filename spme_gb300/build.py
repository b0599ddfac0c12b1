"""Build libspme_gb300.so in-tree with nvcc for sm_103a (one -gencode).

Each .cu under csrc/ compiles to an object in parallel; the objects link into
spme_gb300/libspme_gb300.so (cuFFT linked, CUDA runtime static).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libspme_gb300.so")
DRIVER = os.path.join(HERE, "pme")
DRIVER_SRC = os.path.join(HERE, "driver", "pme.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps += [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    extra = extra or []
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if _stale(obj, src) or extra:
            jobs.append([nv, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in sources()]
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcufft"])
        os.replace(tmp, LIB)
    build_driver(verbose)
    return LIB


def build_driver(verbose: bool = False) -> str:
    """The `pme` command-line driver (host C++ over the C ABI, rpath to the library)."""
    if (os.path.exists(DRIVER) and os.path.getmtime(DRIVER) > os.path.getmtime(DRIVER_SRC)
            and os.path.getmtime(DRIVER) > os.path.getmtime(LIB)):
        return DRIVER
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), DRIVER_SRC,
           "-L" + HERE, "-lspme_gb300", "-Wl,-rpath,$ORIGIN", "-lm", "-o", DRIVER]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
