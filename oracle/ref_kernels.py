"""Run the reference's own CUDA kernels on one frame -- TEST INFRASTRUCTURE ONLY.

Wraps oracle/libref_harness.so (ref_harness.c), which loads the reference's
src/pd_solver.cu compiled into oracle/_ref/pd_solver_ref.cubin by
ref_build.py.  Used by tests/golden/make_ref_golden.py to record golden
vectors on a GPU machine, and by a GPU test that times the reference's kernels
beside the fused sweep.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import ref_build

_lib = None


def available() -> bool:
    return os.path.exists(ref_build.CUBIN) and (os.path.exists(ref_build.HARNESS_LIB) or ref_build.build_harness())


def _load():
    global _lib
    if _lib is None:
        ref_build.build_harness()
        _lib = C.CDLL(ref_build.HARNESS_LIB)
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


def _args(scene):
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    return dict(mass=f32(scene.mass), tris=i32(scene.tris), G=f32(scene.G), area=f32(scene.area),
                k=f32(scene.k_stretch), diag=f32(scene.diag), quads=i32(scene.hinge), bw=f32(scene.w),
                bn=f32(scene.nrest), bk=f32(scene.hk), pins=i32(scene.pins), tgt=f32(scene.pin_targets))


def ref_time(scene, x, v, iters, nframes, gravity=None):
    """Mean device time (ms) of the reference's frame (PDSolver::step's
    launches, `iters` iterations) and of its iteration loop, over `nframes`
    frames from the state (x, v) after one untimed frame (CUDA events)."""
    L = _load()
    x = np.ascontiguousarray(x, np.float32).reshape(-1).copy()
    v = np.ascontiguousarray(v, np.float32).reshape(-1).copy()
    g = scene.ext[1] if gravity is None else gravity
    err = C.create_string_buffer(512)
    a = _args(scene)
    fm, lm = C.c_float(), C.c_float()
    rc = L.ref_time(ref_build.CUBIN.encode(), scene.N, scene.T, len(scene.hinge), len(scene.pins), _p(x), _p(v),
                    _p(a["mass"]), _p(a["tris"]), _p(a["G"]), _p(a["area"]), _p(a["k"]), _p(a["diag"]),
                    _p(a["quads"]), _p(a["bw"]), _p(a["bn"]), _p(a["bk"]), _p(a["pins"]), _p(a["tgt"]), int(iters),
                    C.c_float(scene.h), C.c_float(g), C.c_float(scene.damping), int(nframes), C.byref(fm),
                    C.byref(lm), err, 512)
    if rc != 0:
        raise RuntimeError("reference kernels failed: " + err.value.decode())
    return fm.value, lm.value


def ref_step(scene, x, v, iters, gravity=None):
    """One reference PDSolver::step on the arrays of an oracle.Scene.
    Gravity acts on y only, as in predict_kernel (src/pd_solver.cu:18-30)."""
    L = _load()
    x = np.ascontiguousarray(x, np.float32).reshape(-1).copy()
    v = np.ascontiguousarray(v, np.float32).reshape(-1).copy()
    g = scene.ext[1] if gravity is None else gravity
    err = C.create_string_buffer(512)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    i32 = lambda a: np.ascontiguousarray(a, np.int32)
    arrs = dict(mass=f32(scene.mass), tris=i32(scene.tris), G=f32(scene.G), area=f32(scene.area),
                k=f32(scene.k_stretch), diag=f32(scene.diag), quads=i32(scene.hinge), bw=f32(scene.w),
                bn=f32(scene.nrest), bk=f32(scene.hk), pins=i32(scene.pins), tgt=f32(scene.pin_targets))
    rc = L.ref_step(ref_build.CUBIN.encode(), scene.N, scene.T, len(scene.hinge), len(scene.pins), _p(x), _p(v),
                    _p(arrs["mass"]), _p(arrs["tris"]), _p(arrs["G"]), _p(arrs["area"]), _p(arrs["k"]),
                    _p(arrs["diag"]), _p(arrs["quads"]), _p(arrs["bw"]), _p(arrs["bn"]), _p(arrs["bk"]),
                    _p(arrs["pins"]), _p(arrs["tgt"]), int(iters), C.c_float(scene.h), C.c_float(g),
                    C.c_float(scene.damping), err, 512)
    if rc != 0:
        raise RuntimeError("reference kernels failed: " + err.value.decode())
    return x.reshape(-1, 3), v.reshape(-1, 3)
