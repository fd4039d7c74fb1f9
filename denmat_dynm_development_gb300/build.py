"""In-tree build of the native libraries.

* ``libdmdgpu.so`` -- CUDA kernels + C ABI (include/dmd_gpu.h), compiled for sm_103a only.
* ``libdmdhost.so`` -- host-side C++ (ldbd_data reader, param.in, set-up, run driver).

Both are built with plain nvcc/g++ command lines next to the sources; the .so files are
git-ignored and rebuilt on each machine (the GPU host is aarch64, this container x86_64).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
GPU_LIB = os.path.join(PKG, "libdmdgpu.so")
HOST_LIB = os.path.join(PKG, "libdmdhost.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

GPU_SRCS = [os.path.join(CSRC, "dmd_api.cu"), os.path.join(CSRC, "dmd_layout.cpp"), os.path.join(CSRC, "dmd_noalloc.cu")]
GPU_DEPS = GPU_SRCS + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
    [os.path.join(INC, "dmd_gpu.h")]
HOST_SRCS = [os.path.join(CSRC, f) for f in ("dmd_host.cpp",) if os.path.exists(os.path.join(CSRC, f))]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        sys.stderr.write(p.stdout + p.stderr)
        raise RuntimeError("build failed: " + " ".join(cmd))
    return p


def build_gpu(force=False, verbose=False):
    if not force and not _stale(GPU_LIB, GPU_DEPS):
        return GPU_LIB
    objs = []
    cmds = []
    for src in GPU_SRCS:
        obj = os.path.join(CSRC, os.path.basename(src) + ".o")
        objs.append(obj)
        cmds.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                    "-I", INC, "-c", src, "-o", obj] + (["-Xptxas", "-v"] if verbose else []))
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for p in ex.map(_run, cmds):
            if verbose:
                sys.stderr.write(p.stderr)
    tmp = GPU_LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


def build_host(force=False):
    if not HOST_SRCS:
        return None
    deps = HOST_SRCS + [os.path.join(INC, "dmd_host.h"), os.path.join(INC, "dmd_gpu.h"), GPU_LIB]
    if not force and not _stale(HOST_LIB, deps):
        return HOST_LIB
    tmp = HOST_LIB + ".tmp"
    build_gpu()
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", INC, "-o", tmp] + HOST_SRCS +
         ["-L", PKG, "-l:libdmdgpu.so", "-Wl,-rpath,$ORIGIN", "-lm", "-lpthread"])
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


def build_all(force=False, verbose=False):
    g = build_gpu(force, verbose)
    return g, build_host(force)


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv, verbose="-v" in sys.argv))
