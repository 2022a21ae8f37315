"""Build the native library libfe_gb300.so in-tree (pyoomph_gb300/lib/).

One translation unit, compiled by nvcc for sm_103a only:
    nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3 -shared ...
The element kernels themselves are generated at run time and compiled by
nvrtc (also for sm_103a) through this library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libfe_gb300.so")
ROOT = os.path.dirname(HERE)
GENCODE = "arch=compute_103a,code=sm_103a"


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _libdirs(home: str):
    out = []
    for d in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        p = os.path.join(home, d)
        if os.path.isdir(p):
            out.append(p)
    return out


def sources():
    return [os.path.join(CSRC, "fe_gb300.cu")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "fe_gb300.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    home = cuda_home()
    os.makedirs(LIBDIR, exist_ok=True)
    libdirs = _libdirs(home)
    cmd = [os.path.join(home, "bin", "nvcc"), "-gencode", GENCODE, "-lineinfo", "-O3", "-std=c++17",
           "-shared", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    cmd += sources()
    cmd += ["-o", LIB + ".tmp"]
    for d in libdirs:
        cmd += ["-L", d, f"-Xlinker=-rpath={d}"]
    cmd += ["-lnvrtc"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
