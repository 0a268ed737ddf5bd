"""Build the in-tree shared libraries for sm_103a.

Usage: python merging-ilu0_gb300/bilu_build.py [--force]

libbilu.so: every translation unit under csrc/ (CUDA kernels + C ABI) is
compiled in parallel with nvcc for sm_103a only, then linked.
libbilu_ref.so: the drop-in C++ interface of the original code (shim/: batch
containers, Matrix Market I/O and the solver entry points), host C++ on top of
libbilu.so.  Objects go to merging-ilu0_gb300/_build/ (git-ignored).  Rebuilds
only what changed.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbilu.so")
SHIM = os.path.join(HERE, "shim")
SHIM_LIB = os.path.join(HERE, "libbilu_ref.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime():
    m = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src, force):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if not force and os.path.exists(obj):
        if os.path.getmtime(obj) >= max(os.path.getmtime(path), _headers_mtime()):
            return obj, None
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O3,-ffp-contract=off",
           "-I", INCLUDE, "-I", CSRC, "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    build_shim(force)
    if verbose:
        print("built", LIB, "and", SHIM_LIB)
    return LIB


def _cuda_dirs():
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    libs = [d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib")) if os.path.isdir(d)]
    return os.path.join(cuda, "include"), libs


def build_shim(force=False):
    """libbilu_ref.so: g++ over shim/*.cpp, linked to libbilu.so (rpath $ORIGIN) and the CUDA runtime."""
    srcs = sorted(os.path.join(SHIM, f) for f in os.listdir(SHIM) if f.endswith(".cpp"))
    hdrs = [os.path.join(SHIM, "include", f) for f in os.listdir(os.path.join(SHIM, "include"))]
    deps = srcs + hdrs + [os.path.join(INCLUDE, "bilu.h"), LIB]
    if not force and os.path.exists(SHIM_LIB) and os.path.getmtime(SHIM_LIB) >= max(map(os.path.getmtime, deps)):
        return SHIM_LIB
    inc, libdirs = _cuda_dirs()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
           "-I", os.path.join(SHIM, "include"), "-I", INCLUDE, "-I", inc, *srcs, "-o", SHIM_LIB,
           "-L", HERE, "-lbilu", *[f"-L{d}" for d in libdirs], "-lcudart", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"shim build failed:\n$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return SHIM_LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
