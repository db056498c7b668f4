"""ORACLE - test infrastructure only.  Build recipe for the checkers:

  oracle/liboracle.so        CPU restatement of the reference (g++ -fopenmp, no FP contraction)
  oracle/librefrun.so        loader that runs the reference's own kernels from the cubins below
  oracle/_ref/*.cubin        the reference's CUDA files compiled where they lie in the reference
                             checkout (only when that checkout is present; the cubins then travel
                             with the repository copy, the sources never do)

    python oracle/build.py [--reference DIR]

The reference checkout is taken from --reference, else from the JP_REFERENCE environment variable,
else from the location this recipe was written for (DEFAULT_REFERENCE); without a checkout the
cubins are left as they are.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
CUDA = "/usr/local/cuda"
NVCC = os.path.join(CUDA, "bin", "nvcc") if os.path.exists(os.path.join(CUDA, "bin", "nvcc")) else "nvcc"
CXX = os.environ.get("CXX", "g++")
DEFAULT_REFERENCE = "/root/reference"


def reference_dir(argv: list[str] | None = None) -> str:
    """--reference DIR, else $JP_REFERENCE, else DEFAULT_REFERENCE."""
    argv = sys.argv if argv is None else argv
    if "--reference" in argv:
        return argv[argv.index("--reference") + 1]
    return os.environ.get("JP_REFERENCE") or DEFAULT_REFERENCE


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle() -> str:
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in sorted(os.listdir(HERE)) if f.endswith("_oracle.cpp")]
    if _stale(out, srcs):
        _run([CXX, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
              "-o", out] + srcs)
    return out


def build_refrun() -> str | None:
    src = os.path.join(HERE, "refrun.cpp")
    out = os.path.join(HERE, "librefrun.so")
    if not os.path.exists(os.path.join(CUDA, "include", "cuda_runtime.h")):
        return None
    if _stale(out, [src]):
        _run([CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(CUDA, "include"), src, "-o", out,
              "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")])
    return out


def build_reference_cubins(reference: str | None = None) -> list[str]:
    """Compile the reference's .cu files, in place in its checkout, to device-only cubins (MB=8, the
    reference's default; AMR with its Makefile's -maxrregcount=128)."""
    src_dir = os.path.join(reference or reference_dir([]), "src")
    if not os.path.isdir(src_dir):
        return []
    os.makedirs(REF_OUT, exist_ok=True)
    arch = ["-gencode", "arch=compute_103a,code=sm_103a"]
    jobs = [
        (os.path.join(REF_OUT, "ref_uniform_mb8.cubin"), os.path.join(HERE, "ref_uniform_kernels.cu"),
         os.path.join(src_dir, "tgv3d_uniform.cu"), ["-DMB=8"]),
        (os.path.join(REF_OUT, "ref_amr_mb8.cubin"), os.path.join(HERE, "ref_amr_kernels.cu"),
         os.path.join(src_dir, "tgv3d_amr.cu"),
         ["-DMB=8", "-maxrregcount=128", "-include", os.path.join(HERE, "thrust_identity_shim.h")]),
    ]
    outs = []
    for out, tu, ref_src, extra in jobs:
        if _stale(out, [tu, ref_src]):
            _run([NVCC, "-cubin", "-O3"] + arch + extra + ["-I", src_dir, "-diag-suppress", "177", tu, "-o", out])
        outs.append(out)
    return outs


def build(reference: str | None = None) -> None:
    build_oracle()
    build_refrun()
    build_reference_cubins(reference)


if __name__ == "__main__":
    build(reference_dir())
