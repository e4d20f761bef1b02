"""Build recipe for the reference's own CUDA kernels -- TEST INFRASTRUCTURE ONLY.

The reference GPU path (src/pd_solver.cu) compiles with nvcc without Eigen,
because its Eigen-dependent members sit behind #ifndef __CUDACC__.  Where the
reference sources are present (not on the GPU machine), this recipe compiles
that file, as it lies in the reference tree, into a device image for sm_103a:

    oracle/_ref/pd_solver_ref.cubin

The reference tree is the directory named by the environment variable
CLOTH_CUDA_REFERENCE, or the first command-line argument:

    CLOTH_CUDA_REFERENCE=/path/to/cloth-cuda python oracle/ref_build.py
    python oracle/ref_build.py /path/to/cloth-cuda

(default when neither is given: /root/reference).

Only its kernels are used; its host code (PDSolver) is never compiled or run.
The image is git-ignored and travels to the GPU machine with the rest of the
tree.  ref_harness.c (compiled on the GPU machine) loads it with the CUDA driver API
and launches the reference kernels in the order PDSolver::step launches them
(src/pd_solver.cu:496-621), to produce golden vectors for the oracle's
literal restatement.  The image is never read or disassembled; it is only
loaded and run.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF_ROOT = "/root/reference"


def ref_root() -> str:
    """The reference tree: CLOTH_CUDA_REFERENCE, else the default."""
    return os.environ.get("CLOTH_CUDA_REFERENCE") or DEFAULT_REF_ROOT


OUT_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT_DIR, "pd_solver_ref.cubin")
HARNESS_SRC = os.path.join(HERE, "ref_harness.c")
HARNESS_LIB = os.path.join(HERE, "libref_harness.so")


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuda.h")):
            return cand
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc))) if nvcc else None


def build_cubin(root: str | None = None) -> bool:
    root = root or ref_root()
    src = os.path.join(root, "src", "pd_solver.cu")
    if not os.path.exists(src):
        return os.path.exists(CUBIN)
    if os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= os.path.getmtime(src):
        return True
    os.makedirs(OUT_DIR, exist_ok=True)
    ch = _cuda_home()
    nvcc = os.path.join(ch, "bin", "nvcc") if ch else "nvcc"
    subprocess.check_call([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                           "-I" + os.path.join(root, "include"), "-I" + os.path.join(root, "src"),
                           src, "-o", CUBIN])
    return True


def build_harness() -> bool:
    """The driver-API harness (plain C); links libcuda (the stub here)."""
    ch = _cuda_home()
    if not ch:
        return False
    if os.path.exists(HARNESS_LIB) and os.path.getmtime(HARNESS_LIB) >= os.path.getmtime(HARNESS_SRC):
        return True
    libdirs = [os.path.join(ch, "lib64", "stubs"), os.path.join(ch, "lib64"), os.path.join(ch, "targets", "sbsa-linux", "lib", "stubs")]
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-I" + os.path.join(ch, "include"), HARNESS_SRC,
           "-o", HARNESS_LIB + ".tmp"] + ["-L" + d for d in libdirs if os.path.isdir(d)] + ["-lcuda"]
    subprocess.check_call(cmd, cwd=HERE)
    os.replace(HARNESS_LIB + ".tmp", HARNESS_LIB)
    return True


def build_if_available() -> None:
    try:
        build_cubin()
    except (OSError, subprocess.CalledProcessError):
        pass
    try:
        build_harness()
    except (OSError, subprocess.CalledProcessError):
        pass


if __name__ == "__main__":
    import sys
    print("cubin", build_cubin(sys.argv[1] if len(sys.argv) > 1 else None), "harness", build_harness())
