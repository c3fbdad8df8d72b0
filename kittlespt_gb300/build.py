"""Builds libkpt.so (the CUDA path tracer behind include/kpt.h) in-tree.

Seven translation units, compiled in parallel with nvcc for sm_103a only:
kpt_path.cu (path and ray kernels, fast maths like the reference's GPU
build), kpt_adjoint.cu (path-replay adjoint, fast maths), kpt_post.cu (post
chain, IEEE), kpt_api.cu (C ABI), kpt_scene.cpp (host
acceleration-structure build), kpt_build.cu (the same BLAS build on the
GPU, IEEE without contraction) and kpt_fsr.cu (the FSR upscale path, IEEE
without contraction).  Host code is compiled without
floating-point contraction so x86-64 and aarch64 builds agree.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "libkpt.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          f"-I{CSRC}", f"-I{INCLUDE}"]

UNITS = {
    "kpt_path.cu": ["-use_fast_math"],
    "kpt_adjoint.cu": ["-use_fast_math"],
    "kpt_post.cu": [],
    "kpt_api.cu": [],
    "kpt_scene.cpp": [],
    "kpt_build.cu": ["-fmad=false"],
    "kpt_fsr.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return False


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _sources_newer(OUT):
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(name):
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name + ".o")
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], "-c", src, "-o", obj]
        if name.endswith(".cpp"):
            cmd = [cc, "-x", "cu", *cmd[1:]]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {name}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = OUT + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
