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

    python oracle/ref/build_ref.py            # where the reference sources are present
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
REFERENCE = "/root/reference/dogm"
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


def build(verbose: bool = False) -> list[str]:
    """Builds oracle/_ref/*.cubin from the reference sources (no-op without them)."""
    if not available():
        if verbose:
            print("reference sources absent: using the prebuilt", OUT)
        return []
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(KERNEL_FILES)) as ex:
        outs = list(ex.map(_one, KERNEL_FILES))
    if verbose:
        print("built %d reference cubins in %s" % (len(outs), OUT))
    return outs


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
