"""Build recipe of the PD cloth library: libpdg.so (sm_103a) and the
sim_cloth command-line driver, compiled in-tree with nvcc/g++ in parallel.

    python cloth-cuda_gb300/build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpdg.so")
BIN = os.path.join(HERE, "bin")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, cwd=HERE, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    ch = cuda_home()
    nvcc = os.path.join(ch, "bin", "nvcc")
    inc = ["-I" + os.path.join(ch, "include"), "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
    os.makedirs(OBJ, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + [os.path.abspath(__file__)]
    cxx_flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
    # host code of the .cu files is compiled without FMA contraction too, so
    # host-side arithmetic (Chebyshev weights) rounds the same on x86 and Arm
    nv_flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-O3",
                "--expt-relaxed-constexpr"]
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp")) + glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            if src.endswith(".cu"):
                cmd = [nvcc] + nv_flags + inc + ["-c", src, "-o", obj]
            else:
                cmd = ["g++"] + cxx_flags + inc + ["-c", src, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nvcc, ARCH, "-shared", "-cudart", "static", "-o", tmp] + objs +
             ["-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    # command-line driver (links the library)
    tool_src = os.path.join(CSRC, "tools", "sim_cloth.cpp")
    if os.path.exists(tool_src):
        os.makedirs(BIN, exist_ok=True)
        exe = os.path.join(BIN, "sim_cloth")
        if force or _stale(exe, [tool_src, LIB] + headers):
            _run(["g++"] + cxx_flags + ["-I" + os.path.join(ROOT, "include"), tool_src, "-o", exe,
                  "-L" + HERE, "-lpdg", "-Wl,-rpath," + HERE])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
