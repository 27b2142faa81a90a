"""Builds libphysicore_gb300.so in-tree with nvcc for sm_103a.

The translation units compile in parallel into physicore_gb300/_build/ and link
into physicore_gb300/libphysicore_gb300.so (static CUDA runtime, no torch types).
The C++20 host mirror of the reference's solver plugin surface (csrc/host/*.cpp)
links against it as libphysicore_gb300_host.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libphysicore_gb300.so")
HOST_LIB = os.path.join(PKG, "libphysicore_gb300_host.so")
HOST = os.path.join(CSRC, "host")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def headers() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + headers() + [__file__]):
        return obj
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
           "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), *extra, "-c", src, "-o", obj + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, extra: list[str] | None = None, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra or []), srcs))
    if _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], check=True)
        os.replace(tmp, LIB)
    build_host()
    return LIB


def cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand:
            return cand
    raise RuntimeError("no C++ compiler found")


def build_host() -> str:
    """The host mirror: solver interface, registry and the gb300_solver plugin."""
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    deps = srcs + sorted(glob.glob(os.path.join(HOST, "*.h"))) + headers() + [LIB, __file__]
    if _stale(HOST_LIB, deps):
        tmp = HOST_LIB + f".tmp{os.getpid()}"
        subprocess.run([cxx(), "-std=c++20", "-O2", "-fPIC", "-shared", "-Wall", "-Wextra", *srcs,
                        "-I", os.path.join(ROOT, "include"), "-L", PKG, "-lphysicore_gb300",
                        "-Wl,-rpath,$ORIGIN", "-o", tmp], check=True)
        os.replace(tmp, HOST_LIB)
    return HOST_LIB


if __name__ == "__main__":
    print(build())
