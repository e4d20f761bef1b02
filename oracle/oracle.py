"""Python access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check in __graft_entry__.py and the CPU-baseline leg of
bench.py import this module.  The product (cloth-cuda_gb300/) never does.

`build()` compiles oracle.c (plain C, gcc) into oracle/liboracle.so; the
wrappers below call it through ctypes on numpy arrays.  Which reference
function each routine restates is documented in oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SOURCES = [os.path.join(HERE, f) for f in ("oracle.c", "oracle_solve.inc", "oracle.h")]

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc if it is missing or stale."""
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fno-fast-math",
               "-ffp-contract=off", os.path.join(HERE, "oracle.c"), "-o", tmp, "-lm"]
        subprocess.check_call(cmd, cwd=HERE)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Problem(C.Structure):
    _fields_ = [
        ("N", C.c_int), ("T", C.c_int), ("E", C.c_int),
        ("tris", C.c_void_p), ("Dm_inv", C.c_void_p), ("area", C.c_void_p),
        ("k_stretch", C.c_void_p), ("hinge", C.c_void_p), ("hinge_w", C.c_void_p),
        ("hinge_n", C.c_void_p), ("hinge_k", C.c_void_p), ("mass", C.c_void_p),
        ("P", C.c_int), ("pin_idx", C.c_void_p), ("pin_target", C.c_void_p),
        ("h", C.c_double), ("damping", C.c_double), ("ext", C.c_double * 3),
    ]


class _JacobiOpts(C.Structure):
    _fields_ = [("iters", C.c_int), ("tol", C.c_double), ("use_cheb", C.c_int),
                ("rho", C.c_double), ("delay", C.c_int), ("gamma", C.c_double),
                ("init", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------- setup

def generate_grid(nrows, ncols, size, mtype):
    """Reference generator (x-z plane, `size` = cell edge)."""
    L = lib()
    N = C.c_int(); T = C.c_int()
    if L.orc_grid_counts(nrows, ncols, mtype, C.byref(N), C.byref(T)) != 0:
        raise ValueError("bad grid")
    pos = np.zeros((N.value, 3), np.float32)
    tris = np.zeros((T.value, 3), np.int32)
    L.orc_generate_grid(nrows, ncols, C.c_float(size), mtype, _p(pos), _p(tris))
    return pos, tris


def rest_state(pos, tris, density=0.1, with_dfdx=False):
    pos = _f32(pos); tris = _i32(tris)
    N, T = len(pos), len(tris)
    G = np.zeros((T, 4), np.float32); area = np.zeros(T, np.float32)
    mass = np.zeros(N, np.float32)
    dfdx = np.zeros((T, 6, 9), np.float32) if with_dfdx else None
    lib().orc_rest_state(N, T, _p(pos), _p(tris), C.c_float(density), _p(G), _p(area),
                         _p(mass), _p(dfdx))
    return (G, area, mass, dfdx) if with_dfdx else (G, area, mass)


def topology(N, tris):
    tris = _i32(tris)
    edges = np.zeros((3 * len(tris) + 1, 4), np.int32)
    nE = lib().orc_topology(N, len(tris), _p(tris), _p(edges))
    return edges[:nE]


def build_bend(pos, tris, edges, kb):
    pos = _f32(pos); tris = _i32(tris); edges = _i32(edges)
    n = len(edges)
    hinge = np.zeros((n + 1, 4), np.int32); w = np.zeros((n + 1, 4), np.float32)
    nr = np.zeros(n + 1, np.float32); hk = np.zeros(n + 1, np.float32)
    E = lib().orc_build_bend(len(pos), _p(pos), _p(tris), n, _p(edges), C.c_float(kb),
                             _p(hinge), _p(w), _p(nr), _p(hk))
    return hinge[:E], w[:E], nr[:E], hk[:E]


def jacobi_diag(N, tris, G, area, k_stretch, hinge, w, hk, mass, h):
    diag = np.zeros(N, np.float32)
    tris = _i32(tris); G = _f32(G); area = _f32(area); k_stretch = _f32(k_stretch)
    hinge = _i32(hinge); w = _f32(w); hk = _f32(hk); mass = _f32(mass)
    lib().orc_jacobi_diag(N, len(tris), _p(tris), _p(G), _p(area), _p(k_stretch), len(hinge),
                          _p(hinge), _p(w), _p(hk), _p(mass), C.c_float(h), _p(diag))
    return diag


class Scene:
    """A cloth with its full setup computed by the oracle.

    pos/tris are the rest mesh in the caller's vertex order; pins default to
    the rest positions of `pins`."""

    def __init__(self, pos, tris, *, density=0.1, k_stretch=1e3, k_bend=1e-2, pins=(),
                 h=1.0 / 60, gravity=-9.81, wind=(0.0, 0.0, 0.0), damping=0.0,
                 pin_targets=None):
        self.pos = _f32(pos).reshape(-1, 3)
        self.tris = _i32(tris).reshape(-1, 3)
        self.N, self.T = len(self.pos), len(self.tris)
        self.G, self.area, self.mass = rest_state(self.pos, self.tris, density)
        self.k_stretch = np.broadcast_to(np.float32(k_stretch), (self.T,)).astype(np.float32) \
            if np.ndim(k_stretch) == 0 else _f32(k_stretch)
        self.edges = topology(self.N, self.tris)
        if k_bend is not None and (np.ndim(k_bend) > 0 or k_bend > 0):
            self.hinge, self.w, self.nrest, self.hk = build_bend(self.pos, self.tris, self.edges,
                                                                 float(np.ravel(k_bend)[0]))
        else:
            self.hinge = np.zeros((0, 4), np.int32); self.w = np.zeros((0, 4), np.float32)
            self.nrest = np.zeros(0, np.float32); self.hk = np.zeros(0, np.float32)
        self.pins = _i32(np.asarray(pins, dtype=np.int32).reshape(-1))
        self.pin_targets = _f32(self.pos[self.pins] if pin_targets is None else pin_targets).reshape(-1, 3)
        self.h, self.damping = float(h), float(damping)
        self.ext = (float(wind[0]), float(gravity) + float(wind[1]), float(wind[2]))
        self.diag = jacobi_diag(self.N, self.tris, self.G, self.area, self.k_stretch, self.hinge,
                                self.w, self.hk, self.mass, np.float32(self.h))

    def problem(self):
        pr = _Problem()
        pr.N, pr.T, pr.E = self.N, self.T, len(self.hinge)
        pr.tris, pr.Dm_inv, pr.area = _p(self.tris), _p(self.G), _p(self.area)
        pr.k_stretch = _p(self.k_stretch)
        pr.hinge, pr.hinge_w, pr.hinge_n, pr.hinge_k = _p(self.hinge), _p(self.w), _p(self.nrest), _p(self.hk)
        pr.mass = _p(self.mass)
        pr.P, pr.pin_idx, pr.pin_target = len(self.pins), _p(self.pins), _p(self.pin_targets)
        pr.h, pr.damping = self.h, self.damping
        pr.ext[0], pr.ext[1], pr.ext[2] = self.ext
        return pr

    # ------------------------------------------------------------ solves
    def step_literal(self, x, v, iters):
        x = _f32(x).copy(); v = _f32(v).copy()
        pr = self.problem()
        lib().orc_step_literal_f32(C.byref(pr), _p(self.diag), iters, _p(x), _p(v))
        return x, v

    def step_jacobi(self, x, v, iters, *, tol=0.0, rho=0.99, delay=1, gamma=1.0, cheb=True,
                    init=0, x0=None, dtype=np.float64):
        dt = np.dtype(dtype)
        x = np.ascontiguousarray(x, dt).copy(); v = np.ascontiguousarray(v, dt).copy()
        x0a = None if x0 is None else np.ascontiguousarray(x0, dt)
        o = _JacobiOpts(iters, tol, 1 if cheb else 0, rho, delay, gamma, init)
        res = np.zeros(iters + 1); ry = C.c_double(); used = C.c_int()
        pr = self.problem()
        if dt == np.float64:
            diag = self.diag.astype(np.float64)
            lib().orc_step_jacobi_f64(C.byref(pr), _p(diag), C.byref(o), _p(x), _p(v), _p(x0a),
                                      _p(res), C.byref(ry), C.byref(used))
        else:
            lib().orc_step_jacobi_f32(C.byref(pr), _p(self.diag), C.byref(o), _p(x), _p(v), _p(x0a),
                                      _p(res), C.byref(ry), C.byref(used))
        return x, v, dict(res=res[: used.value + 1], res_y=ry.value, used=used.value)

    def residual(self, y, x):
        y = np.ascontiguousarray(y, np.float64); x = np.ascontiguousarray(x, np.float64)
        r = np.zeros_like(x)
        pr = self.problem()
        f = lib().orc_residual_f64
        f.restype = C.c_double
        n = f(C.byref(pr), _p(y), _p(x), _p(r))
        return n, r

    def predict(self, x, v):
        x = np.asarray(x, np.float64).reshape(-1, 3)
        v = np.asarray(v, np.float64).reshape(-1, 3)
        return (x + self.h * v + self.h * self.h * np.asarray(self.ext)).reshape(-1)

    def step_direct(self, x, v, iters=50, *, pin_elim=1, with_bend=False, dtype=np.float64):
        dt = np.dtype(dtype)
        x = np.ascontiguousarray(x, dt).copy(); v = np.ascontiguousarray(v, dt).copy()
        pr = self.problem()
        fn = lib().orc_step_direct_f64 if dt == np.float64 else lib().orc_step_direct_f32
        st = fn(C.byref(pr), iters, pin_elim, 1 if with_bend else 0, _p(x), _p(v))
        if st != 0:
            raise RuntimeError("LDL^T factorisation failed")
        return x, v

    @staticmethod
    def last_factor_nnz():
        """Strictly lower entries of the last LDL^T factor step_direct built."""
        f = lib().orc_last_factor_nnz
        f.restype = C.c_longlong
        return int(f())

    def global_matrix(self, with_bend=False):
        pr = self.problem()
        nnz = C.c_int()
        lib().orc_global_matrix_f64(C.byref(pr), 1, 1 if with_bend else 0, C.byref(nnz), None, None, None)
        ri = np.zeros(nnz.value, np.int32); ci = np.zeros(nnz.value, np.int32); val = np.zeros(nnz.value)
        lib().orc_global_matrix_f64(C.byref(pr), 1, 1 if with_bend else 0, C.byref(nnz), _p(ri), _p(ci), _p(val))
        return ri, ci, val


def hanging_cloth(n, side, *, seed=0, jitter=1e-4, mtype=1):
    """Square cloth in the x-y plane: row 0 on top (y = 0), rows going down
    along -y, alternating diagonals (type 1), z jitter N(0, jitter) from seed.
    Returns (pos, tris, corner pins)."""
    pos, tris = generate_grid(n, n, side / (n - 1), mtype)
    # the reference lays the grid in x-z; map z -> -y so row 0 is the top row
    out = np.zeros_like(pos)
    out[:, 0] = pos[:, 0]
    out[:, 1] = -pos[:, 2]
    rng = np.random.default_rng(seed)
    out[:, 2] = (rng.standard_normal(len(pos)) * jitter).astype(np.float32)
    return out.astype(np.float32), tris, np.array([0, n - 1], np.int32)
