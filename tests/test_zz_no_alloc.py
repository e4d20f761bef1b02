"""The allocation-free frame entry point (pdg_step_noalloc) against the
solver entry point (pdg_solver_step), through the C ABI.

pdg_step_noalloc serves callers that cannot call cudaMalloc -- hosts that own
all device memory through their own pool and load this library as a plugin,
and real-time loops that cannot afford cudaMalloc's device-wide
synchronisation.  It takes the cloth in the reference's device layout and
keeps its scratch in a static device array.  This file is collected last so
that a run stopping at the first failure has run every other test first; it
also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_POS = 1e-5    # same bar as the other one-frame position comparisons
REL_VEL = 1e-3


def rel(a, b):
    a = np.asarray(a, np.float64).reshape(-1); b = np.asarray(b, np.float64).reshape(-1)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None and t.numel() else None


@pytest.mark.parametrize("tol", [0.0, 1e-4])
def test_noalloc_matches_solver_two_calls(pdg, tol):
    torch = pytest.importorskip("torch")
    n = 33
    m = pdg.Mesh.hanging(n, 1.0, mtype=1, jitter=1e-4, seed=4)
    c = pdg.Constraints(m).build_stretch(1e3).build_bend(1e-2).pin_corners(n)
    cfg = pdg.Config.default(max_iterations=12, rho=0.99, dt=1 / 60, gravity=-9.81, tolerance=tol,
                             kernel=pdg.KERNEL_GRAPH, wind=(0.3, 0.0, -0.2), damping=0.01)
    if tol > 0:   # a soft cloth so that the tolerance is reached within the cap
        m = pdg.Mesh.hanging(9, 0.5, mtype=1, jitter=1e-4, seed=4)
        c = pdg.Constraints(m).build_stretch(20.0).build_bend(1e-3).pin_corners(9)
        cfg.max_iterations, cfg.rho = 400, 0.9
    a = m.arrays(); ca = c.arrays()
    diag = c.jacobi_diag(cfg.dt)
    solver = pdg.Solver(cfg, m, c)

    dev = "cuda"
    f32 = lambda x: torch.as_tensor(np.ascontiguousarray(x, np.float32), device=dev)
    i32 = lambda x: torch.as_tensor(np.ascontiguousarray(x, np.int32), device=dev)
    pos = f32(a["rest"].reshape(-1)); vel = torch.zeros_like(pos)
    t = dict(mass=f32(a["mass"]), diag=f32(diag), tris=i32(a["tris"]), G=f32(a["Dm_inv"]), area=f32(a["area"]),
             ks=f32(ca["k_stretch"]), quads=i32(ca["quads"]), w=f32(ca["w"]), nr=f32(ca["n_rest"]),
             kb=f32(ca["bend_k"]), pins=i32(ca["pins"]), tgt=f32(ca["targets"]))
    torch.cuda.synchronize()
    E, P = len(ca["bend_k"]), len(ca["pins"])
    for call in range(2):
        st = pdg.FrameStats()
        rc = pdg.lib().pdg_step_noalloc(
            C.byref(cfg), m.N, _ptr(pos), _ptr(vel), _ptr(t["mass"]), _ptr(t["diag"]), m.T, _ptr(t["tris"]),
            _ptr(t["G"]), _ptr(t["area"]), _ptr(t["ks"]), E, _ptr(t["quads"]), _ptr(t["w"]), _ptr(t["nr"]),
            _ptr(t["kb"]), P, _ptr(t["pins"]), _ptr(t["tgt"]), None, C.byref(st))
        assert rc == 0, pdg.lib().pdg_last_error_string()
        ref = solver.step(1)[0]
        x_ref, v_ref = solver.get_state()
        torch.cuda.synchronize()
        x = pos.cpu().numpy().reshape(-1, 3); v = vel.cpu().numpy().reshape(-1, 3)
        assert rel(x, x_ref) < REL_POS, call
        assert rel(v, v_ref) < REL_VEL, call
        assert st.status == 0
        if tol > 0:
            # float atomics round differently from the solver's ordered gather,
            # so the sweep at which the residual crosses the tolerance may
            # differ by one
            assert abs(st.iterations - ref["iterations"]) <= 1
            assert st.converged == 1 and ref["converged"] == 1
            assert st.rel_residual <= tol
        else:
            assert st.iterations == ref["iterations"]
            assert abs(st.res_final - ref["res_final"]) <= 1e-3 * ref["res_final"]


def test_noalloc_rejects_oversize(pdg):
    cfg = pdg.Config.default()
    L = pdg.lib()
    rc = L.pdg_step_noalloc(C.byref(cfg), 131072 + 1, *([None] * 4), 0, *([None] * 4), 0, *([None] * 4), 0,
                            None, None, None, None)
    assert rc == pdg.ERR_ARG
    assert b"131072" in L.pdg_last_error_string()
    cfg.max_iterations = 5000
    rc = L.pdg_step_noalloc(C.byref(cfg), 10, *([None] * 4), 0, *([None] * 4), 0, *([None] * 4), 0,
                            None, None, None, None)
    assert rc == pdg.ERR_ARG and b"4096" in L.pdg_last_error_string()


def _cloth_arrays(pdg, torch, n=17, seed=4):
    m = pdg.Mesh.hanging(n, 1.0, mtype=1, jitter=1e-4, seed=seed)
    c = pdg.Constraints(m).build_stretch(1e3).build_bend(1e-2).pin_corners(n)
    a = m.arrays(); ca = c.arrays()
    dev = "cuda"
    f32 = lambda x: torch.as_tensor(np.ascontiguousarray(x, np.float32), device=dev)
    i32 = lambda x: torch.as_tensor(np.ascontiguousarray(x, np.int32), device=dev)
    t = dict(mass=f32(a["mass"]), tris=i32(a["tris"]), G=f32(a["Dm_inv"]), area=f32(a["area"]),
             ks=f32(ca["k_stretch"]), quads=i32(ca["quads"]), w=f32(ca["w"]), nr=f32(ca["n_rest"]),
             kb=f32(ca["bend_k"]), pins=i32(ca["pins"]), tgt=f32(ca["targets"]))
    return m, c, a, ca, t, f32


def _call(pdg, cfg, m, t, diag, pos, vel, E, P, stream=None):
    st = pdg.FrameStats()
    rc = pdg.lib().pdg_step_noalloc(
        C.byref(cfg), m.N, _ptr(pos), _ptr(vel), _ptr(t["mass"]), _ptr(diag), m.T, _ptr(t["tris"]),
        _ptr(t["G"]), _ptr(t["area"]), _ptr(t["ks"]), E, _ptr(t["quads"]), _ptr(t["w"]), _ptr(t["nr"]),
        _ptr(t["kb"]), P, _ptr(t["pins"]), _ptr(t["tgt"]), C.c_void_p(stream) if stream else None, C.byref(st))
    return rc, st


@pytest.mark.parametrize("cap,final", [(0, 1), (1, 1), (1, 0), (7, 1), (7, 0)])
def test_noalloc_sweep_caps_and_final_residual_match_solver(pdg, cap, final):
    # sweep caps of 0 and 1 and the final residual with and without its
    # extra sweep (no tolerance), against pdg_solver_step
    torch = pytest.importorskip("torch")
    m, c, a, ca, t, f32 = _cloth_arrays(pdg, torch)
    cfg = pdg.Config.default(max_iterations=cap, rho=0.99, dt=1 / 60, gravity=-9.81, tolerance=0.0,
                             compute_final_residual=final, kernel=pdg.KERNEL_GRAPH)
    diag = f32(c.jacobi_diag(cfg.dt))
    solver = pdg.Solver(cfg, m, c)
    pos = f32(a["rest"].reshape(-1)); vel = torch.zeros_like(pos)
    rc, st = _call(pdg, cfg, m, t, diag, pos, vel, len(ca["bend_k"]), len(ca["pins"]))
    assert rc == 0, pdg.lib().pdg_last_error_string()
    ref = solver.step(1)[0]
    x_ref, v_ref = solver.get_state()
    torch.cuda.synchronize()
    assert rel(pos.cpu().numpy(), x_ref) < REL_POS
    assert rel(vel.cpu().numpy(), v_ref) < REL_VEL or np.abs(v_ref).max() < 1e-6
    assert st.status == 0 and st.iterations == ref["iterations"] == cap
    if final:
        assert st.res_final >= 0 and abs(st.res_final - ref["res_final"]) <= 1e-3 * ref["res_final"]
    else:
        assert st.res_final == -1.0 and ref["res_final"] == -1.0


def test_noalloc_non_finite_frame_keeps_x_zeroes_v_and_reports_it(pdg):
    torch = pytest.importorskip("torch")
    m, c, a, ca, t, f32 = _cloth_arrays(pdg, torch)
    cfg = pdg.Config.default(max_iterations=6, rho=0.99, dt=1 / 60, gravity=-9.81, compute_final_residual=1)
    diag = f32(c.jacobi_diag(cfg.dt))
    x0 = a["rest"].reshape(-1).copy()
    free = next(i for i in range(m.N) if i not in set(ca["pins"].tolist()))
    x0[3 * free + 1] = np.nan
    pos = f32(x0); vel = f32(np.full(3 * m.N, 0.25, np.float32))
    rc, st = _call(pdg, cfg, m, t, diag, pos, vel, len(ca["bend_k"]), len(ca["pins"]))
    assert rc == 0   # the call returns OK; the failure is in the frame's record
    assert st.status == pdg.ERR_NUMERIC
    torch.cuda.synchronize()
    x = pos.cpu().numpy().reshape(-1, 3); v = vel.cpu().numpy()
    expect = x0.reshape(-1, 3).copy()
    expect[ca["pins"]] = ca["targets"]   # pins re-applied
    assert np.array_equal(x, expect, equal_nan=True)
    assert np.all(v == 0.0)


def test_noalloc_on_a_stream_of_its_own_two_calls(pdg):
    torch = pytest.importorskip("torch")
    m, c, a, ca, t, f32 = _cloth_arrays(pdg, torch, n=25, seed=9)
    cfg = pdg.Config.default(max_iterations=10, rho=0.99, dt=1 / 60, gravity=-9.81, kernel=pdg.KERNEL_GRAPH)
    diag = f32(c.jacobi_diag(cfg.dt))
    solver = pdg.Solver(cfg, m, c)
    side = torch.cuda.Stream()
    pos = f32(a["rest"].reshape(-1)); vel = torch.zeros_like(pos)
    torch.cuda.synchronize()
    for call in range(2):
        rc, st = _call(pdg, cfg, m, t, diag, pos, vel, len(ca["bend_k"]), len(ca["pins"]), stream=side.cuda_stream)
        assert rc == 0, pdg.lib().pdg_last_error_string()
        solver.step(1, stats=False)
        x_ref, v_ref = solver.get_state()
        side.synchronize()
        assert rel(pos.cpu().numpy(), x_ref) < REL_POS, call
        assert rel(vel.cpu().numpy(), v_ref) < REL_VEL, call
