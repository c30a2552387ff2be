"""Builds the engine's shared library, libngrav_gpu.so, and the deck front
end, nbody_gb300, in-tree.

Every CUDA translation unit under ``csrc/`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
``opengl-physics_gb300/libngrav_gpu.so`` next to this file.  The C++ sources
under ``host/`` (deck parser, output writer, scenarios, CLI) are compiled with
the host g++ and linked into ``opengl-physics_gb300/nbody_gb300`` against that
library (rpath ``$ORIGIN``).  Objects go to ``_build/`` at the repository
root.  No cmake; nvcc and the host gcc only.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
HOST = os.path.join(PKG, "host")
LIB = os.path.join(PKG, "libngrav_gpu.so")
EXE = os.path.join(PKG, "nbody_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ftz=true / -prec-sqrt=false: FP32 denormals are flushed and sqrtf is the
# hardware approximation; no force term or opening test comes near the FP32
# denormal range, and FP64 code is unaffected by either flag.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-prec-sqrt=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


HOST_FLAGS = ["-O2", "-std=c++17", "-Wall", "-I", INCLUDE, "-I", HOST]


def gxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("g++ not found")


def _newer(target: str, deps) -> bool:
    """True when target exists and is at least as new as every dep."""
    return os.path.isfile(target) and os.path.getmtime(target) >= max(os.path.getmtime(d) for d in deps)


def _compile_host(src: str) -> str:
    obj = os.path.join(BUILD, "host_" + os.path.basename(src) + ".o")
    deps = [src] + glob.glob(os.path.join(HOST, "*.hpp")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    if _newer(obj, deps):
        return obj
    r = subprocess.run([gxx()] + HOST_FLAGS + ["-c", src, "-o", obj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_host(jobs: int | None = None) -> str:
    """Compile host/*.cpp and link nbody_gb300 against libngrav_gpu.so."""
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile_host, srcs))
    if not _newer(EXE, objs + [LIB]):
        tmp = EXE + ".tmp"
        cmd = [gxx(), "-o", tmp] + objs + ["-L", PKG, "-lngrav_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed for nbody_gb300:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, EXE)
    return EXE


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(d) for d in _deps()])
    if os.path.isfile(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose_ptxas else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose_ptxas: bool = False, jobs: int | None = None, host: bool = True) -> str:
    """Compile and link libngrav_gpu.so (and, with host=True, nbody_gb300);
    returns the library's path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not (os.path.isfile(LIB) and os.path.getmtime(LIB) >= newest):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if host:
        build_host(jobs)
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
