"""Python binding of the PD cloth library (ctypes over the C ABI in include/pdg.h).

The classes mirror the reference's C++ interface for the per-frame solve:
Mesh ~ ClothMesh (include/cloth_mesh.h), Constraints ~ SimConstraints +
Constraints (include/sim_constraints.h, include/constraints.h), Config ~
PDSolverConfig and Solver ~ PDSolver (include/pd_solver.h).  Every call goes
to libpdg.so; there is no Python or CPU fallback -- loading fails loudly when
the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpdg.so")

OK, ERR_ARG, ERR_CUDA, ERR_ALLOC, ERR_STATE, ERR_TIMEOUT, ERR_NUMERIC, ERR_IO = 0, -1, -2, -3, -4, -5, -6, -7
MODE_CONSISTENT, MODE_REFERENCE_LITERAL = 0, 1
INIT_INERTIAL, INIT_PREVIOUS, INIT_WARMSTART, INIT_WARMSTART_KEEP = 0, 1, 2, 3
KERNEL_AUTO, KERNEL_GRAPH, KERNEL_PERSISTENT, KERNEL_RESIDENT, KERNEL_AUTOTUNE, KERNEL_STREAM = 0, 1, 2, 3, 4, 5
NODE_FEATURES = 14   # node features of the learned warm start


class PDGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("pdg error %d: %s" % (code, msg))
        self.code = code


class Config(C.Structure):
    """pdg_config: PDSolverConfig (include/pd_solver.h:4-15) plus extensions."""
    _fields_ = [
        ("max_iterations", C.c_int), ("tolerance", C.c_float), ("use_chebyshev", C.c_int),
        ("rho", C.c_float), ("gravity", C.c_float), ("dt", C.c_float),
        ("stretch_stiffness", C.c_float), ("bend_stiffness", C.c_float), ("damping", C.c_float),
        ("wind", C.c_float * 3), ("cheb_delay", C.c_int), ("gamma", C.c_float), ("mode", C.c_int),
        ("init", C.c_int), ("kernel", C.c_int), ("patch_verts", C.c_int), ("block_threads", C.c_int),
        ("compute_final_residual", C.c_int), ("smem_carveout", C.c_int),
    ]

    @classmethod
    def default(cls, **kw):
        c = cls()
        _check(lib().pdg_config_default(C.byref(c)))
        for k, v in kw.items():
            if k == "wind":
                for i in range(3):
                    c.wind[i] = float(v[i])
            elif not hasattr(c, k):
                raise AttributeError(k)
            else:
                setattr(c, k, v)
        return c


class FrameStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("warm_start_used", C.c_int),
                ("status", C.c_int), ("res_inertial", C.c_double), ("res_initial", C.c_double),
                ("res_final", C.c_double), ("rel_residual", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneEntry(C.Structure):
    _fields_ = [("kernel", C.c_int), ("patch_verts", C.c_int), ("block_threads", C.c_int),
                ("frame_ms", C.c_float), ("chosen", C.c_int), ("cached", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def autotune_clear_cache():
    lib().pdg_autotune_clear_cache()


class LayoutInfo(C.Structure):
    _fields_ = [("vertices", C.c_int), ("patches", C.c_int), ("max_owned", C.c_int), ("max_local", C.c_int),
                ("halo_total", C.c_longlong), ("boundary_total", C.c_longlong), ("cells", C.c_longlong),
                ("phase_a_cells", C.c_longlong), ("lone_hinges", C.c_longlong), ("smem_resident", C.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def layout_check(cfg, meshes, cons, patch_verts):
    """pdg_layout_check: build the patch layout of these cloths on the host
    and check the properties the kernels rely on.  Returns the layout summary
    as a dict; raises PDGError with the first violation.  No GPU needed."""
    single = isinstance(meshes, Mesh)
    meshes = [meshes] if single else list(meshes)
    cons = [cons] if single else list(cons)
    cfgs = [cfg] * len(meshes) if isinstance(cfg, Config) else list(cfg)
    n = len(meshes)
    info = LayoutInfo()
    _check(lib().pdg_layout_check(n, (Config * n)(*cfgs), (C.c_void_p * n)(*[m.h.value for m in meshes]),
                                  (C.c_void_p * n)(*[c.h.value for c in cons]), patch_verts, C.byref(info)))
    return info.as_dict()


def layout_check_planted(cfg, meshes, cons, patch_verts, mistake):
    """pdg_layout_check_planted: the layout check after planting mistake
    1..6 (see include/pdg.h); raises PDGError with the checker's finding."""
    single = isinstance(meshes, Mesh)
    meshes = [meshes] if single else list(meshes)
    cons = [cons] if single else list(cons)
    cfgs = [cfg] * len(meshes) if isinstance(cfg, Config) else list(cfg)
    n = len(meshes)
    info = LayoutInfo()
    _check(lib().pdg_layout_check_planted(n, (Config * n)(*cfgs), (C.c_void_p * n)(*[m.h.value for m in meshes]),
                                          (C.c_void_p * n)(*[c.h.value for c in cons]), patch_verts, mistake,
                                          C.byref(info)))
    return info.as_dict()


_lib = None


def lib():
    """Load libpdg.so (built by cloth-cuda_gb300/build.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libpdg.so is not built: run cloth-cuda_gb300/build.py (or __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        L.pdg_last_error_string.restype = C.c_char_p
        L.pdg_version.restype = C.c_char_p
        # the per-frame host-buffer call takes plain addresses (int or None):
        # converting them costs far less than building ctypes pointers
        L.pdg_solver_step_host.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 5
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise PDGError(rc, lib().pdg_last_error_string().decode())
    return rc


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


_F32 = np.dtype(np.float32)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Mesh:
    """Rest mesh + rest state (ClothMesh)."""

    def __init__(self, handle):
        self.h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        N = C.c_int(); T = C.c_int()
        _check(lib().pdg_mesh_counts(self.h, C.byref(N), C.byref(T)))
        self.N, self.T = N.value, T.value

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.pdg_mesh_destroy(self.h)
            self.h = None

    @classmethod
    def create(cls, pos, tris, density=0.1):
        pos = _f32(pos).reshape(-1, 3); tris = _i32(tris).reshape(-1, 3)
        h = C.c_void_p()
        _check(lib().pdg_mesh_create(_p(pos), len(pos), _p(tris), len(tris), C.c_float(density), C.byref(h)))
        return cls(h)

    @classmethod
    def generate(cls, nrows, ncols, size, mtype, density=0.1):
        h = C.c_void_p()
        _check(lib().pdg_mesh_generate(nrows, ncols, C.c_float(size), mtype, C.c_float(density), C.byref(h)))
        return cls(h)

    @classmethod
    def hanging(cls, n, side, mtype=1, jitter=1e-4, seed=0, density=0.1, ncols=None):
        h = C.c_void_p()
        _check(lib().pdg_mesh_generate_hanging(n, ncols or n, C.c_float(side), mtype, C.c_float(jitter),
                                               C.c_ulonglong(seed), C.c_float(density), C.byref(h)))
        return cls(h)

    @classmethod
    def load_obj(cls, path, density=0.1):
        h = C.c_void_p()
        _check(lib().pdg_mesh_load_obj(path.encode(), C.c_float(density), C.byref(h)))
        return cls(h)

    def arrays(self):
        N, T = self.N, self.T
        out = dict(rest=np.zeros((N, 3), np.float32), tris=np.zeros((T, 3), np.int32),
                   Dm_inv=np.zeros((T, 4), np.float32), area=np.zeros(T, np.float32),
                   mass=np.zeros(N, np.float32), dFdx=np.zeros((T, 6, 9), np.float32))
        _check(lib().pdg_mesh_get(self.h, _p(out["rest"]), _p(out["tris"]), _p(out["Dm_inv"]), _p(out["area"]),
                                  _p(out["mass"]), _p(out["dFdx"])))
        return out

    def topology(self):
        nE = C.c_int(); nI = C.c_int()
        _check(lib().pdg_topology_counts(self.h, C.byref(nE), C.byref(nI)))
        out = dict(edges=np.zeros((nE.value, 4), np.int32), rest_len=np.zeros(nE.value, np.float32),
                   vt_ptr=np.zeros(self.N + 1, np.int32), vt=np.zeros(3 * self.T, np.int32),
                   tri_tri=np.zeros((self.T, 3), np.int32), num_inner=nI.value)
        _check(lib().pdg_topology_get(self.h, _p(out["edges"]), _p(out["rest_len"]), _p(out["vt_ptr"]),
                                      _p(out["vt"]), _p(out["tri_tri"])))
        return out


class Constraints:
    """SimConstraints (stretch k, bend hinges, Jacobi diagonal) + pins."""

    def __init__(self, mesh: Mesh):
        self.mesh = mesh
        self.h = C.c_void_p()
        _check(lib().pdg_constraints_create(mesh.h, C.byref(self.h)))

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.pdg_constraints_destroy(self.h)
            self.h = None

    def build_stretch(self, k):
        _check(lib().pdg_constraints_build_stretch(self.h, C.c_float(k)))
        return self

    def set_stretch_k(self, k):
        k = _f32(k)
        assert k.size == self.mesh.T
        _check(lib().pdg_constraints_set_stretch_k(self.h, _p(k)))
        return self

    def build_bend(self, k):
        _check(lib().pdg_constraints_build_bend(self.h, C.c_float(k)))
        return self

    def set_pins(self, idx, targets=None):
        idx = _i32(idx).reshape(-1)
        t = None if targets is None else _f32(targets).reshape(-1, 3)
        _check(lib().pdg_constraints_set_pins(self.h, _p(idx) if idx.size else None, idx.size,
                                              _p(t) if t is not None else None))
        return self

    def pin_top_row(self, ncols):
        _check(lib().pdg_constraints_pin_top_row(self.h, ncols))
        return self

    def pin_corners(self, ncols):
        _check(lib().pdg_constraints_pin_corners(self.h, ncols))
        return self

    def arrays(self):
        nb = C.c_int(); npn = C.c_int()
        _check(lib().pdg_constraints_counts(self.h, C.byref(nb), C.byref(npn)))
        E, P, T = nb.value, npn.value, self.mesh.T
        out = dict(k_stretch=np.zeros(T, np.float32), quads=np.zeros((E, 4), np.int32), w=np.zeros((E, 4), np.float32),
                   n_rest=np.zeros(E, np.float32), bend_k=np.zeros(E, np.float32), pins=np.zeros(P, np.int32),
                   targets=np.zeros((P, 3), np.float32))
        _check(lib().pdg_constraints_get(self.h, _p(out["k_stretch"]), _p(out["quads"]), _p(out["w"]),
                                         _p(out["n_rest"]), _p(out["bend_k"]), _p(out["pins"]), _p(out["targets"])))
        return out

    def jacobi_diag(self, dt):
        d = np.zeros(self.mesh.N, np.float32)
        _check(lib().pdg_constraints_jacobi_diag(self.h, C.c_float(dt), _p(d)))
        return d


class Solver:
    """PDSolver over one cloth, or many cloths of uneven size (batch)."""

    def __init__(self, cfg, meshes, cons, stream=None):
        single = isinstance(meshes, Mesh)
        meshes = [meshes] if single else list(meshes)
        cons = [cons] if single else list(cons)
        cfgs = [cfg] * len(meshes) if isinstance(cfg, Config) else list(cfg)
        self.meshes, self.cons = meshes, cons   # keep the handles alive
        self.n = len(meshes)
        arr = (Config * self.n)(*cfgs)
        mh = (C.c_void_p * self.n)(*[m.h.value for m in meshes])
        ch = (C.c_void_p * self.n)(*[c.h.value for c in cons])
        self.h = C.c_void_p()
        st = C.c_void_p(stream) if stream is not None else None
        _check(lib().pdg_solver_create_batch(self.n, arr, mh, ch, st, C.byref(self.h)))
        self.N = [m.N for m in meshes]
        self.offsets = np.concatenate([[0], np.cumsum(self.N)]).astype(np.int64)

    def close(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.pdg_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def step(self, nframes=1, stats=True):
        st = (FrameStats * self.n)() if stats else None
        _check(lib().pdg_solver_step(self.h, nframes, st))
        return [s.as_dict() for s in st] if stats else None

    def set_state(self, x=None, v=None, cloth=0):
        xa = None if x is None else _f32(x).reshape(-1, 3)
        va = None if v is None else _f32(v).reshape(-1, 3)
        _check(lib().pdg_solver_set_state(self.h, cloth, _p(xa) if xa is not None else None,
                                          _p(va) if va is not None else None, 0))

    def get_state(self, cloth=0):
        n = self.N[cloth]
        x = np.zeros((n, 3), np.float32); v = np.zeros((n, 3), np.float32)
        _check(lib().pdg_solver_get_state(self.h, cloth, _p(x), _p(v), 0))
        return x, v

    def set_state_all(self, x=None, v=None, on_device=False):
        if on_device:
            _check(lib().pdg_solver_set_state_all(self.h, C.c_void_p(x) if x else None, C.c_void_p(v) if v else None, 1))
            return
        xa = None if x is None else _f32(x).reshape(-1, 3)
        va = None if v is None else _f32(v).reshape(-1, 3)
        _check(lib().pdg_solver_set_state_all(self.h, _p(xa) if xa is not None else None,
                                              _p(va) if va is not None else None, 0))

    def get_state_all(self, x=None, v=None, on_device=False):
        """Positions and velocities of every cloth in caller order.  With
        on_device, x and v are device pointers; otherwise they may be
        C-contiguous float32 (N, 3) host arrays to write into (e.g. pinned
        buffers reused every frame), else new arrays are returned."""
        if on_device:
            _check(lib().pdg_solver_get_state_all(self.h, C.c_void_p(x) if x else None, C.c_void_p(v) if v else None, 1))
            return None
        n = int(self.offsets[-1])
        xa = x if x is not None else np.empty((n, 3), np.float32)
        va = v if v is not None else np.empty((n, 3), np.float32)
        for arr in (xa, va):
            if arr.dtype != np.float32 or not arr.flags.c_contiguous or arr.size != 3 * n:
                raise ValueError("output arrays must be C-contiguous float32 with N*3 elements")
        _check(lib().pdg_solver_get_state_all(self.h, _p(xa), _p(va), 0))
        return xa, va

    def step_host(self, x_in=None, v_in=None, x_out=None, v_out=None, nframes=1, stats=False):
        """Upload / step / download in one call with one synchronisation
        (pdg_solver_step_host).  Inputs and outputs are C-contiguous float32
        (N, 3) host arrays of the whole batch in caller order (pinned ones
        copy fastest); any may be None.  Input and output may be the same
        arrays."""
        n = int(self.offsets[-1])
        addr = {}
        for arr in (x_in, v_in, x_out, v_out):
            if arr is not None and id(arr) not in addr:
                if arr.dtype != _F32 or not arr.flags.c_contiguous or arr.size != 3 * n:
                    raise ValueError("state arrays must be C-contiguous float32 with N*3 elements")
                addr[id(arr)] = arr.ctypes.data
        a = lambda arr: addr[id(arr)] if arr is not None else None
        st = (FrameStats * self.n)() if stats else None
        _check(lib().pdg_solver_step_host(self.h, nframes, a(x_in), a(v_in), a(x_out), a(v_out),
                                          C.cast(st, C.c_void_p) if stats else None))
        return [s.as_dict() for s in st] if stats else None

    def set_tolerance(self, tol, cloth=-1):
        """Relative-residual target of one cloth (-1: all); 0 runs the cap."""
        _check(lib().pdg_solver_set_tolerance(self.h, cloth, C.c_float(tol)))

    def set_pin_targets(self, targets, cloth=0):
        t = _f32(targets).reshape(-1, 3)
        _check(lib().pdg_solver_set_pin_targets(self.h, cloth, _p(t)))

    def prediction(self, cloth=0):
        y = np.zeros((self.N[cloth], 3), np.float32)
        _check(lib().pdg_solver_get_prediction(self.h, cloth, _p(y)))
        return y

    def time_frames(self, nframes):
        """(average frame ms, average fused-sweep ms) over `nframes` frames."""
        f = C.c_float(); sw = C.c_float()
        _check(lib().pdg_solver_time_frames(self.h, nframes, C.byref(f), C.byref(sw)))
        return f.value, sw.value

    @property
    def launches(self):
        n = C.c_longlong()
        _check(lib().pdg_solver_launch_count(self.h, C.byref(n)))
        return n.value

    @property
    def stream(self):
        s = C.c_void_p()
        _check(lib().pdg_solver_stream(self.h, C.byref(s)))
        return s.value or 0

    def launch_info(self):
        k = C.c_int(); pv = C.c_int(); nt = C.c_int(); npch = C.c_int()
        _check(lib().pdg_solver_launch_info(self.h, C.byref(k), C.byref(pv), C.byref(nt), C.byref(npch)))
        return dict(kernel=k.value, patch_verts=pv.value, block_threads=nt.value, npatches=npch.value)

    def tune_results(self):
        """Candidate table of the autotuner (empty unless created with KERNEL_AUTOTUNE)."""
        n = C.c_int()
        _check(lib().pdg_solver_tune_results(self.h, None, 0, C.byref(n)))
        out = (TuneEntry * max(1, n.value))()
        _check(lib().pdg_solver_tune_results(self.h, out, n.value, C.byref(n)))
        return [out[i].as_dict() for i in range(n.value)]

    def set_wait_budget(self, cycles):
        """clock64 cycles each grid-barrier / neighbour wait may spin before
        the one-launch-per-frame kernels give up with ERR_TIMEOUT."""
        _check(lib().pdg_solver_set_wait_budget(self.h, C.c_longlong(int(cycles))))

    def set_frame_tag(self, tag):
        """Test hook: the tag number the next resident frame's neighbour
        exchange starts from (near 2**32 it takes the clear-and-restart path)."""
        _check(lib().pdg_solver_set_frame_tag(self.h, C.c_ulonglong(int(tag))))


class WarmStart:
    """Learned warm start (mesh message-passing network on the GPU)."""

    def __init__(self, seed=0):
        self.h = C.c_void_p()
        _check(lib().pdg_warmstart_create(C.c_ulonglong(seed), C.byref(self.h)))
        n = C.c_int()
        _check(lib().pdg_warmstart_param_count(self.h, C.byref(n)))
        self.count = n.value
        self.solver = None

    def close(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.pdg_warmstart_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def get_params(self):
        p = np.zeros(self.count, np.float32)
        _check(lib().pdg_warmstart_get_params(self.h, _p(p)))
        return p

    def set_params(self, p):
        p = _f32(p)
        assert p.size == self.count
        _check(lib().pdg_warmstart_set_params(self.h, _p(p)))

    def eval(self, x, ptr, adj, ef, target, freew, ew=None):
        x = _f32(x).reshape(-1, NODE_FEATURES); ptr = _i32(ptr); adj = _i32(adj); ef = _f32(ef).reshape(-1, 4)
        target = _f32(target).reshape(-1, 3); freew = _f32(freew)
        ewa = None if ew is None else _f32(ew).reshape(-1)
        N = len(x)
        out = np.zeros((N, 3), np.float32); grads = np.zeros(self.count, np.float32); loss = C.c_float()
        _check(lib().pdg_warmstart_eval(self.h, N, _p(x), _p(ptr), _p(adj) if adj.size else None,
                                        _p(ef) if ef.size else None, _p(target), _p(freew),
                                        _p(ewa) if ewa is not None and ewa.size else None, _p(out),
                                        C.byref(loss), _p(grads)))
        return out, loss.value, grads

    def adam_step(self, lr):
        _check(lib().pdg_warmstart_adam_step(self.h, C.c_float(lr)))

    def attach(self, solver):
        _check(lib().pdg_warmstart_attach(self.h, solver.h))
        self.solver = solver   # keep alive

    def set_smoothness(self, lam):
        """Weight of the neighbour-difference term of the loss (0: plain MSE)."""
        _check(lib().pdg_warmstart_set_smoothness(self.h, C.c_float(lam)))
        return self

    def set_energy_norm(self, enable=True):
        """Weigh the neighbour-difference term by the PD system's stiffness
        (the error's energy norm) when training on an attached solver."""
        _check(lib().pdg_warmstart_set_energy_norm(self.h, 1 if enable else 0))
        return self

    def set_judge_sweeps(self, k):
        """Sweeps each start runs before the judge compares them (0: start residuals)."""
        _check(lib().pdg_warmstart_set_judge_sweeps(self.h, int(k)))
        return self

    def time_inference(self, reps=5):
        """Mean device ms of one prediction on the attached solver's state."""
        ms = C.c_float()
        _check(lib().pdg_warmstart_time_inference(self.h, int(reps), C.byref(ms)))
        return ms.value

    @property
    def judge_sweeps(self):
        k = C.c_int()
        _check(lib().pdg_warmstart_get_judge_sweeps(self.h, C.byref(k)))
        return k.value

    def train_pair(self, traj, deep, lr):
        """One training step on traj's trajectory with deep's solve as target."""
        loss = C.c_float()
        _check(lib().pdg_warmstart_train_pair(self.h, traj.h, deep.h, C.c_float(lr), C.byref(loss)))
        return loss.value

    def train_frame(self, solver, lr):
        loss = C.c_float()
        _check(lib().pdg_warmstart_train_frame(self.h, solver.h, C.c_float(lr), C.byref(loss)))
        return loss.value


def exported_symbols():
    """Names declared in include/pdg.h (parsed from the header)."""
    import re
    hdr = open(os.path.join(os.path.dirname(HERE), "include", "pdg.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(pdg_[a-z0-9_]+)\s*\(", hdr)))
