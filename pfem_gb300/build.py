"""Build libpfemgpu.so in-tree with nvcc for sm_103a (GB300).

Each .cu under csrc/ is compiled to an object in parallel, then linked into
pfem_gb300/libpfemgpu.so with the CUDA runtime linked statically, so the library has no
dependency on torch or on a runtime installed next to it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpfemgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-fvisibility=hidden", "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(HERE, "..", "include", "pfem_gpu.h"))
    return max(os.path.getmtime(h) for h in hs if os.path.exists(h))


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in sources()) and _headers_mtime() <= t


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra)
    if verbose:
        extra += ["-Xptxas", "-v"]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), sources()))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-Xcompiler", "-fPIC", *objs, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


REMESH_SRC = os.path.join(HERE, "host", "pfem_remesh.cpp")
REMESH_LIB = os.path.join(HERE, "libpfemremesh.so")


def build_remesh(force=False):
    """The C++ host remesh, libpfemremesh.so (g++, no CUDA)."""
    hdr = os.path.join(HERE, "..", "include", "pfem_remesh.h")
    if (not force and os.path.exists(REMESH_LIB) and
            os.path.getmtime(REMESH_LIB) >= max(os.path.getmtime(REMESH_SRC), os.path.getmtime(hdr))):
        return REMESH_LIB
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = REMESH_LIB + f".tmp{os.getpid()}"
    # no contraction into FMAs: the same roundings on x86 and Arm as the Python host remesh
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-shared", "-fPIC", "-fvisibility=hidden",
           REMESH_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on {REMESH_SRC}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, REMESH_LIB)
    return REMESH_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
