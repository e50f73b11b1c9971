"""Build recipe for the native parts of hsmc_gb300.

Compiles the CUDA sources in ``csrc/`` for sm_103a into
``hsmc_gb300/libhsmc_gpu.so`` (the C-ABI library declared in
``include/hsmc_gpu.h``), the drop-in host program ``hsmc_gb300/bin/hsmc`` and
the analysis tool ``hsmc_gb300/bin/hsmc_stat``.
Translation units are compiled in parallel; nothing is installed outside the
package directory.
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
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhsmc_gpu.so")
BIN_DIR = os.path.join(PKG, "bin")
EXE = os.path.join(BIN_DIR, "hsmc")

CU_SOURCES = ["api.cu", "sweep.cu", "move_pass.cu", "observables.cu", "batch.cu", "lwidom.cu", "cluster.cu", "cavity.cu", "sweep_small.cu", "batch_persist.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(ROOT, "include", "hsmc_gpu.h")]


C_SOURCES = ["cavity_coeffs.c"]  # host C (C99 complex arithmetic), compiled by gcc


def _compile_c(src: str) -> str:
    obj = os.path.join(OBJ, os.path.basename(src).replace(".c", "_c.o"))
    if _newer(obj, [src] + _headers()):
        return obj
    subprocess.run(["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-fPIC", "-Wall", "-c", src, "-o", obj],
                   check=True)
    return obj


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src).replace(".cu", ".o"))
    if _newer(obj, [src] + _headers()) and not verbose_ptxas:
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose_ptxas else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"nvcc failed on {src}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build_library(verbose_ptxas: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    objs += [_compile_c(os.path.join(CSRC, s)) for s in C_SOURCES]
    if not _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


def build_host() -> str | None:
    """The drop-in C program (reference CLI, keywords and output files)."""
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".c")) if os.path.isdir(HOST) else []
    if not srcs:
        return None
    os.makedirs(BIN_DIR, exist_ok=True)
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + [LIB]
    if _newer(EXE, deps):
        return EXE
    cuda_lib = "/usr/local/cuda/lib64"
    cmd = ["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-Wall", "-I" + os.path.join(ROOT, "include"),
           "-o", EXE] + srcs + ["-L" + PKG, "-lhsmc_gpu", "-Wl,-rpath," + PKG, "-L" + cuda_lib,
                                "-Wl,-rpath," + cuda_lib, "-lcudart", "-lz", "-lm"]
    subprocess.run(cmd, check=True)
    return EXE


STAT_SRC = os.path.join(PKG, "analysis", "hsmc_stat.c")
STAT_EXE = os.path.join(BIN_DIR, "hsmc_stat")


def build_stat() -> str:
    """The analysis tool (blocking, jackknife, contact fits) in plain C."""
    os.makedirs(BIN_DIR, exist_ok=True)
    if not _newer(STAT_EXE, [STAT_SRC]):
        subprocess.run(["gcc", "-O2", "-std=gnu99", "-Wall", "-o", STAT_EXE, STAT_SRC, "-lm"], check=True)
    return STAT_EXE


def build(verbose_ptxas: bool = False) -> None:
    build_library(verbose_ptxas)
    build_host()
    build_stat()


if __name__ == "__main__":
    build(verbose_ptxas="-v" in sys.argv)
    print(LIB)
