"""Build libamca3d.so (and the amca3d CLI) in-tree with nvcc for sm_103a.

Device code is compiled with -fmad=false: the envelope arithmetic must stay
unfused to match the reference bit for bit (its x86-64 build has no FMA).
Host code is compiled with -ffp-contract=off for the same reason on hosts
whose compilers would otherwise contract a*b+c (aarch64).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libamca3d.so")
CLI = os.path.join(HERE, "amca3d")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc() -> str:
    p = os.path.join(CUDA_HOME, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp") and f != "cli.cpp")
    return cu, cpp


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "-fmad=false", "-Xptxas", "-v", *common, "-c", src, "-o", obj]
    else:
        cmd = [nvcc(), *common, "-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if src.endswith(".cu"):
        with open(obj + ".ptxas.txt", "w") as f:
            f.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = _sources()
    srcs = [os.path.join(CSRC, f) for f in cu + cpp]
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src):
        cmd = [nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
               "-x", "c++", cli_src, "-o", CLI, "-L", HERE, "-lamca3d", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        for f in sorted(os.listdir(BUILD)):
            if f.endswith(".ptxas.txt"):
                print(open(os.path.join(BUILD, f)).read())
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
