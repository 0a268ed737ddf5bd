"""Recipe for oracle/_ref: the reference's own kernels, compiled from its sources.

  python oracle/build_ref.py

Test infrastructure only.  Two outputs, both in the git-ignored oracle/_ref/:

1. Where the reference sources are present (this build container), each
   reference translation unit on the solver path is compiled for sm_103a into
   a cubin, straight from the files of the reference checkout (the directory
   named by MERGING_ILU0_REFERENCE, default /root/reference).  A generated
   wrapper unit includes the reference's header.h first and raises its
   compile-time capacity limits (MAX_NUM_ROWS 54 -> 512, MAX_NUM_NZ 2560 kept),
   then includes the reference .cu unchanged; header.h's `#pragma once` keeps
   the raised limits.  Device code only: the reference's host code is compiled
   for x86 and would not run on the Arm GPU host, so it is not built.
2. On every machine: oracle/ref_launch.cpp (this project's own driver-API
   launcher) into oracle/_ref/libreflaunch.so, which loads the cubins and
   launches the reference kernels on inputs that the tests prepare.

The cubins travel to the GPU host with the repository snapshot; nothing
there reads /root/reference.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout: MERGING_ILU0_REFERENCE names its root (default /root/reference)
REF_ROOT = os.environ.get("MERGING_ILU0_REFERENCE", "/root/reference")
REF = os.path.join(REF_ROOT, "Batched-ILU0-merged", "ILU0_ISAI_bicgstab")

# (cubin name, reference translation unit)
UNITS = [
    ("merged", "PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu"),
    ("ilu_split", "PrecondBiCGSTAB_ilu_gpu.cu"),
    ("ilu_isai", "PrecondBiCGSTAB_ilu_isai_gpu.cu"),
    ("ilu0", "ILU_0_gpu.cu"),
    ("parilu", "parILU_0_gpu.cu"),
    ("isai", "isai_gpu.cu"),
    ("general_isai", "PrecondBiCGSTAB_general_isai_gpu.cu"),
]
MAX_NUM_ROWS = 512
MAX_NUM_NZ = 2560


def nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_cubins(force=False):
    if not os.path.isdir(REF):
        return False
    os.makedirs(OUT, exist_ok=True)
    for name, unit in UNITS:
        cubin = os.path.join(OUT, name + ".cubin")
        src = os.path.join(REF, unit)
        if not force and os.path.exists(cubin) and os.path.getmtime(cubin) >= os.path.getmtime(src):
            continue
        wrapper = os.path.join(OUT, f"wrap_{name}.cu")
        with open(wrapper, "w") as f:
            f.write(f'#include "{REF}/header.h"\n'
                    f"#undef MAX_NUM_ROWS\n#define MAX_NUM_ROWS {MAX_NUM_ROWS}\n"
                    f"#undef MAX_NUM_NZ\n#define MAX_NUM_NZ {MAX_NUM_NZ}\n"
                    f'#include "{src}"\n')
        cmd = [nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-I", REF, wrapper,
               "-o", cubin]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference cubin build failed:\n$ {' '.join(cmd)}\n{r.stderr}")
    return True


def build_launcher(force=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_launch.cpp")
    lib = os.path.join(OUT, "libreflaunch.so")
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= os.path.getmtime(src):
        return lib
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    libdirs = [os.path.join(cuda, "lib64"), os.path.join(cuda, "lib64", "stubs"),
               os.path.join(cuda, "targets", "sbsa-linux", "lib", "stubs")]
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-o", lib, "-I", os.path.join(cuda, "include")]
    for d in libdirs:
        if os.path.isdir(d):
            cmd += ["-L", d]
    cmd += ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference launcher build failed:\n$ {' '.join(cmd)}\n{r.stderr}")
    return lib


def build(force=False):
    build_cubins(force)
    have = all(os.path.exists(os.path.join(OUT, n + ".cubin")) for n, _ in UNITS)
    if have:
        build_launcher(force)
    return have


if __name__ == "__main__":
    print("reference kernels available:", build(force="--force" in sys.argv))
