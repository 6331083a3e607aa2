"""Build recipes for the native parts: the CUDA library (sm_103a only) and the C oracle.

All outputs stay in-tree and are git-ignored:
  dynamic-occupancy-grid-map_gb300/lib/libdogm_gb300.so   CUDA kernels + C ABI
  oracle/_build/libdogm_oracle.so                         C restatement (test/bench checker)
Objects are rebuilt only when a source or header is newer than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG_DIR, "_build")
LIB_DIR = os.path.join(PKG_DIR, "lib")
LIB = os.path.join(LIB_DIR, "libdogm_gb300.so")
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libdogm_oracle.so")

CUDA_SOURCES = ["k_particles.cu", "k_sort.cu", "k_cells.cu", "k_resample.cu", "runtime.cu", "serving.cu", "k_meas.cu", "k_extract.cu", "evaluate.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdogm_gb300.so")


def _headers(directory: str, exts=(".h", ".cuh")) -> list[str]:
    out = []
    for root, _, files in os.walk(directory):
        out += [os.path.join(root, f) for f in files if f.endswith(exts)]
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_cuda(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile every .cu for sm_103a in parallel and link libdogm_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers(CSRC) + _headers(INCLUDE)
    flags = NVCC_FLAGS + (extra_flags or [])
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers + [__file__]):
            jobs.append([nvcc] + ARCH + flags + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for _ in ex.map(_run, jobs):
                pass
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle(verbose: bool = False) -> str:
    """Compile the C restatement (FP32 and FP64 instantiations, OpenMP) into one .so."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE_DIR, f) for f in ("dogm_oracle.c",)]
    deps = srcs + _headers(ORACLE_DIR, (".h",)) + [__file__]
    if _stale(ORACLE_LIB, deps):
        cc = shutil.which("gcc") or "cc"
        tmp = ORACLE_LIB + ".tmp"
        _run([cc, "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
              "-o", tmp] + srcs + ["-lm"])
        os.replace(tmp, ORACLE_LIB)
    if verbose:
        print("built", ORACLE_LIB)
    return ORACLE_LIB


REF_HARNESS_SRC = os.path.join(ORACLE_DIR, "ref", "ref_harness.cu")
REF_HARNESS_LIB = os.path.join(ORACLE_BUILD, "libdogm_ref.so")


def build_ref_harness(verbose: bool = False) -> str:
    """Compile the reference-build harness (test infrastructure: loads the reference's kernel
    cubins from oracle/_ref and runs them in the reference's host sequence)."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    if _stale(REF_HARNESS_LIB, [REF_HARNESS_SRC, __file__]):
        tmp = REF_HARNESS_LIB + ".tmp"
        _run([_nvcc()] + ARCH + ["-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", REF_HARNESS_SRC, "-lcuda",
                                 "-o", tmp])
        os.replace(tmp, REF_HARNESS_LIB)
    if verbose:
        print("built", REF_HARNESS_LIB)
    return REF_HARNESS_LIB


def build_all(verbose: bool = False) -> None:
    build_cuda(verbose)
    build_oracle(verbose)
    build_ref_harness(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
