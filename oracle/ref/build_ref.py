"""Reference build recipe (test infrastructure; the checker, not the product).

Compiles the reference's own CUDA kernels -- every file of dogm/src/kernel/ of
TheCodez/dynamic-occupancy-grid-map, read where the reference sources lie -- into sm_103a
cubins under oracle/_ref/, one per source file.  Nothing of the reference is copied: the
outputs are compiled device code only, git-ignored, and they travel with the repository to
the GPU machine, where oracle/ref/ref_harness.cu loads them with the CUDA driver API and runs them
in the reference's host sequence (dogm/src/dogm.cu, restated there).

The reference needs GLM, which is not installed; oracle/ref/glm/ is a minimal project-written
stand-in (vec4, mat4x4, transpose, matrix-vector product).  dogm_types.h uses assert without
including <cassert>, so it is force-included.  The reference's CMake build cannot be used here
(it requires OpenGL and downloads googletest, dogm/CMakeLists.txt:9,31).

The demo's accuracy evaluator (dogm/demo/utils/dbscan.cpp, metrics.cpp,
precision_evaluator.cpp) is plain host C++; it is compiled where it lies together with
oracle/ref/eval_harness.cu into oracle/_ref/libref_eval.so, a host library for the CPU tests of
this machine (it does not run on the Arm GPU machine, where the tests that need it skip).

    python oracle/ref/build_ref.py            # where the reference sources are present
    DOGM_REFERENCE_DIR=<checkout> python oracle/ref/build_ref.py
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
# where the reference's sources lie: DOGM_REFERENCE_DIR (the repository's root), by default the
# read-only checkout this recipe was written against
REFERENCE = os.path.join(os.environ.get("DOGM_REFERENCE_DIR", "/root/reference"), "dogm")
KERNEL_FILES = ["ego_motion_compensation", "init", "init_new_particles", "mass_update", "particle_to_grid", "predict",
                "resampling", "statistical_moments", "update_persistent_particles"]
FLAGS = ["-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--expt-extended-lambda",
         "-include", "cassert", "-I" + HERE, "-I" + os.path.join(REFERENCE, "include")]


def available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "src", "kernel"))


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _one(name: str) -> str:
    src = os.path.join(REFERENCE, "src", "kernel", name + ".cu")
    dst = os.path.join(OUT, name + ".cubin")
    deps = [src, __file__] + [os.path.join(HERE, "glm", f) for f in os.listdir(os.path.join(HERE, "glm"))]
    for d in ("dogm", os.path.join("dogm", "kernel")):
        inc = os.path.join(REFERENCE, "include", d)
        deps += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    if os.path.exists(dst) and all(os.path.getmtime(d) <= os.path.getmtime(dst) for d in deps):
        return dst
    tmp = dst + ".tmp"
    r = subprocess.run([_nvcc()] + FLAGS + [src, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference kernel %s did not compile:\n%s%s" % (name, r.stdout, r.stderr))
    os.replace(tmp, dst)
    return dst


MEAS_SRC = os.path.join("demo", "simulator", "mapping", "kernel", "measurement_grid.cu")


def build_meas() -> str:
    """Builds oracle/_ref/measurement_grid.cubin: the demo's measurement-grid kernels (inverse
    sensor model into a polar surface, its fusion, framebuffer -> MeasurementCell), plain CUDA
    compiled from dogm/demo/simulator/mapping/kernel/measurement_grid.cu with the demo's own
    flags (no fast math, multiply-add contraction as nvcc defaults)."""
    src = os.path.join(REFERENCE, MEAS_SRC)
    dst = os.path.join(OUT, "measurement_grid.cubin")
    inc = os.path.join(REFERENCE, "demo", "simulator", "include")
    deps = [src, __file__, os.path.join(inc, "mapping", "kernel", "measurement_grid.h")]
    if os.path.exists(dst) and all(os.path.getmtime(d) <= os.path.getmtime(dst) for d in deps):
        return dst
    tmp = dst + ".tmp"
    r = subprocess.run([_nvcc()] + FLAGS + ["-I" + inc, src, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference measurement-grid kernels did not compile:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, dst)
    return dst


EVAL_SOURCES = ["dbscan.cpp", "metrics.cpp", "precision_evaluator.cpp"]
EVAL_LIB = os.path.join(OUT, "libref_eval.so")


def build_eval() -> str:
    """Builds oracle/_ref/libref_eval.so: the reference's evaluator plus eval_harness.cu."""
    utils = os.path.join(REFERENCE, "demo", "utils")
    srcs = [os.path.join(utils, f) for f in EVAL_SOURCES] + [os.path.join(HERE, "eval_harness.cu")]
    deps = srcs + [__file__] + [os.path.join(HERE, "glm", f) for f in os.listdir(os.path.join(HERE, "glm"))]
    if os.path.exists(EVAL_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(EVAL_LIB) for d in deps):
        return EVAL_LIB
    tmp = EVAL_LIB + ".tmp"
    cmd = [_nvcc(), "-x", "cu", "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-include", "cassert", "-I" + HERE, "-I" + os.path.join(REFERENCE, "include"),
           "-I" + os.path.join(utils, "include"), "-I" + os.path.join(REFERENCE, "demo", "simulator", "include")]
    r = subprocess.run(cmd + srcs + ["-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference evaluator did not compile:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, EVAL_LIB)
    return EVAL_LIB


def build(verbose: bool = False) -> list[str]:
    """Builds oracle/_ref/*.cubin from the reference sources (no-op without them)."""
    if not available():
        if verbose:
            print("reference sources absent: using the prebuilt", OUT)
        return []
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(KERNEL_FILES)) as ex:
        ev = ex.submit(build_eval)
        ms = ex.submit(build_meas)
        outs = list(ex.map(_one, KERNEL_FILES)) + [ev.result(), ms.result()]
    if verbose:
        print("built %d reference cubins in %s" % (len(outs), OUT))
    return outs


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
