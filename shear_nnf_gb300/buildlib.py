"""Build recipe of the CUDA library libshearbox.so (sm_103a, in-tree).

Compiles the translation units of csrc/ in parallel with nvcc and links one
shared library with the C-ABI of include/shearbox.h.  No cmake, no torch
extension: the library is plain CUDA C++ behind an ``extern "C"`` interface.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libshearbox.so")
# (source, extra flags): sb_kernels.cu is compiled twice (its FP64 and
# FP32-mixed instantiations in parallel), sb_yline.cu six times (1, 2 or 3
# warps per line solve, each precision)
UNITS = [("sb_kernels.cu", ["-DSB_FLOAT_TU=0"]), ("sb_kernels.cu", ["-DSB_FLOAT_TU=1"]),
         # the y-line kernels once per (warps per line solve, precision)
         *[("sb_yline.cu", [f"-DSB_FLOAT_TU={f}", f"-DSB_KSEG={k}"]) for k in (1, 2, 3)
           for f in (0, 1)],
         ("sb_box.cu", []), ("sb_implicit.cu", []),
         ("sb_ops.cu", []), ("sb_noalloc.cu", []), ("sb_api.cu", []), ("sb_krylov.cu", []),
         # host set-up (coefficients, factorisations, the seeded field) without
         # fused multiply-adds: the same bits on x86 and Arm hosts
         ("sb_host.cpp", ["-Xcompiler", "-ffp-contract=off"]),
         ("sb_io.cpp", []),
         # the finite-difference perturbations as written, without fused multiply-adds
         ("sb_newton.cpp", ["-Xcompiler", "-ffp-contract=off"])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC"]
# extra compile flags for tuning builds, e.g. SB_NVCC_EXTRA="-DSB_KSEG=4"
EXTRA = os.environ.get("SB_NVCC_EXTRA", "").split()


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "shearbox.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    procs = []
    objs = []
    for src, defs in UNITS:
        tag = "".join(d.split("=")[-1] for d in defs if d.startswith("-D"))
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + (f"_{tag}" if tag else "") + ".o")
        objs.append(obj)
        cmd = [nvcc(), *ARCH, *FLAGS, *EXTRA, *defs, "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc(), *FLAGS, *defs, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{out.decode(errors='replace')}")
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
