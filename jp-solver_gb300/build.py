"""Build the engine in-tree: libjpsolver.so (CUDA kernels + C ABI) and the drop-in `uniform` / `amr`
programs.  Plain nvcc/g++ calls, one translation unit per process, no cmake.

    python jp-solver_gb300/build.py          # build what is out of date
    python jp-solver_gb300/build.py --clean  # rebuild everything
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libjpsolver.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE, "-I", CSRC,
                  "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CXX = os.environ.get("CXX", "g++")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    # keep ptxas spill warnings visible
    for line in (r.stdout + r.stderr).splitlines():
        if "spill" in line and "0 bytes spill" not in line:
            print("  ptxas:", line, file=sys.stderr)


def build_lib(verbose: bool = True) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdrs = _headers()
    jobs = []
    objs = []
    for f in srcs:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    if jobs:
        if verbose:
            print("nvcc: %d translation unit(s)" % len(jobs), file=sys.stderr)
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_cli(verbose: bool = True) -> list[str]:
    os.makedirs(BINDIR, exist_ok=True)
    out = []
    if not os.path.isdir(HOST):
        return out
    for f in sorted(os.listdir(HOST)):
        if not f.endswith(".cpp"):
            continue
        src = os.path.join(HOST, f)
        exe = os.path.join(BINDIR, f[:-4])
        out.append(exe)
        deps = [src, LIB] + [os.path.join(HOST, h) for h in os.listdir(HOST) if h.endswith(".h")]
        deps += [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")]
        if _stale(exe, deps):
            _run([CXX, "-O2", "-std=c++17", "-I", INCLUDE, "-I", HOST, src, "-o", exe, "-L", LIBDIR, "-ljpsolver",
                  "-Wl,-rpath,$ORIGIN/../lib"])
    return out


def build(verbose: bool = True) -> None:
    build_lib(verbose)
    build_cli(verbose)


def clean() -> None:
    for d in (BUILD, LIBDIR, BINDIR):
        if os.path.isdir(d):
            shutil.rmtree(d)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    build()
    print(LIB)
