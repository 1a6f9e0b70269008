"""Build libfrgpu.so from csrc/ with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel into _build/, then linked into
libfrgpu.so next to the package.  No CMake, no torch extension machinery.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(PKG_ROOT, "libfrgpu.so")
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code contracts no multiply-adds either (-ffp-contract=off), so that host
# arithmetic (setup math, metric scales) gives the same bits on x86 and Arm
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfrgpu.so")


def _extra_flags(src: str) -> list[str]:
    """FP64 translation units (and the filter) contract no multiply-adds on
    their own: their only fused operations are the explicit fma() calls,
    which the oracle performs in the same order, so the FP64 path reproduces
    the oracle bit for bit.  The FP32 units keep the default contraction."""
    name = os.path.basename(src)
    if name.endswith("_f64.cu") or name in ("filter.cu", "limiter.cu", "erk.cu", "tri.cu", "central2d.cu"):
        return ["-fmad=false"]
    return []


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(INCLUDE, "frgpu.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    procs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *_extra_flags(src), "-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd[1:1] = ["-x", "cu"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"{os.path.basename(src)}:\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("libfrgpu build failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
