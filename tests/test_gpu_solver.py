"""CUDA solver against the oracle, through the C ABI (GPU).

Tolerances: float32 arithmetic on both sides with different summation
order; one frame of 10 sweeps agrees to 1e-5 relative in positions, and
every multi-frame comparison against the float64 oracle to 1e-4 relative (the
accuracy bar for positions).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_ONE_FRAME = 1e-5
REL_F64 = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64).reshape(-1); b = np.asarray(b, np.float64).reshape(-1)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def scene(pdg, oracle, n=33, side=1.0, mtype=1, ks=1e3, kb=1e-2, pins="corners", seed=0, **cfgkw):
    m = pdg.Mesh.hanging(n, side, mtype=mtype, jitter=1e-4, seed=seed)
    c = pdg.Constraints(m).build_stretch(ks)
    if kb > 0:
        c.build_bend(kb)
    if pins == "corners":
        c.pin_corners(n)
    elif pins == "top":
        c.pin_top_row(n)
    kw = dict(max_iterations=10, rho=0.99, dt=1 / 60, gravity=-9.81)
    kw.update(cfgkw)
    cfg = pdg.Config.default(**kw)
    a = m.arrays(); ca = c.arrays()
    sc = oracle.Scene(a["rest"], a["tris"], k_stretch=ca["k_stretch"], k_bend=kb if kb > 0 else 0.0,
                      pins=ca["pins"], h=cfg.dt, gravity=cfg.gravity, wind=tuple(cfg.wind), damping=cfg.damping)
    return m, c, cfg, sc, a


def test_one_frame_matches_oracle(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle)
    s = pdg.Solver(cfg, m, c)
    st = s.step(1)[0]
    x, v = s.get_state()
    x0 = a["rest"]; v0 = np.zeros_like(x0)
    xo, vo, info = sc.step_jacobi(x0.reshape(-1), v0.reshape(-1), 10, rho=0.99, dtype=np.float32)
    xd, vd, info64 = sc.step_jacobi(x0.reshape(-1), v0.reshape(-1), 10, rho=0.99, dtype=np.float64)
    assert rel(x, xo) < REL_ONE_FRAME
    assert rel(x, xd) < REL_ONE_FRAME
    assert rel(v, vd) < 1e-3
    assert st["iterations"] == 10 and st["status"] == 0
    assert abs(st["res_inertial"] - info64["res_y"]) / info64["res_y"] < 1e-3
    assert abs(st["res_final"] - info64["res"][-1]) / info64["res"][-1] < 1e-2


def test_many_frames_match_f64(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=17, max_iterations=32)
    s = pdg.Solver(cfg, m, c)
    x = a["rest"].astype(np.float64).reshape(-1); v = np.zeros_like(x)
    for f in range(20):
        s.step(1, stats=False)
        x, v, _ = sc.step_jacobi(x, v, 32, rho=0.99)
    xg, vg = s.get_state()
    assert rel(xg, x) < REL_F64
    assert rel(vg, v) < 1e-2


def test_reference_literal_matches_oracle(pdg, oracle):
    # The reference's literal sweep (x = rhs/diag with the transposed
    # rotation) amplifies a 1e-7 perturbation to ~1e-2 within 10 sweeps and
    # collapses the cloth into degenerate triangles whose threshold branches
    # flip with the last bit, so parity is checked one sweep at a time from
    # well-conditioned states: the rest shape and random 1 % deformations.
    m, c, cfg, sc, a = scene(pdg, oracle, n=17, mode=pdg.MODE_REFERENCE_LITERAL, max_iterations=1)
    s = pdg.Solver(cfg, m, c)
    rng = np.random.default_rng(7)
    cell = 1.0 / 16
    for f in range(6):
        x = a["rest"] + (0 if f == 0 else 0.01 * cell) * rng.standard_normal(a["rest"].shape).astype(np.float32)
        v = (0.05 * rng.standard_normal(x.shape)).astype(np.float32) if f else np.zeros_like(x)
        # the reference re-applies the pins after every step, so its state
        # always holds them at their targets
        x[sc.pins] = sc.pin_targets
        v[sc.pins] = 0.0
        s.set_state(x, v)
        s.step(1, stats=False)
        xg, vg = s.get_state()
        xo, vo = sc.step_literal(x.reshape(-1), v.reshape(-1), 1)
        assert rel(xg, xo) < REL_ONE_FRAME
        assert rel(vg, vo) < 1e-3


def test_reference_literal_sensitivity_bound(pdg, oracle):
    # over 10 literal sweeps the GPU stays within the oracle's own spread
    # under 1e-7 input perturbations
    m, c, cfg, sc, a = scene(pdg, oracle, n=17, mode=pdg.MODE_REFERENCE_LITERAL, max_iterations=10)
    s = pdg.Solver(cfg, m, c)
    s.step(1, stats=False)
    xg, _ = s.get_state()
    x0 = a["rest"].reshape(-1)
    xo, _ = sc.step_literal(x0, np.zeros_like(x0), 10)
    rng = np.random.default_rng(0)
    spread = max(rel(sc.step_literal(x0 * (1 + 1e-7 * rng.standard_normal(x0.shape)).astype(np.float32),
                                     np.zeros_like(x0), 10)[0], xo) for _ in range(4))
    assert rel(xg, xo) < max(10 * spread, 1e-5)


KERNELS = {"persistent": 2, "resident": 3, "stream": 5}


@pytest.mark.parametrize("mtype", [1, 3])
@pytest.mark.parametrize("kernel", ["persistent", "resident", "resident256", "stream"])
@pytest.mark.parametrize("mode", [0, 1])
def test_launch_structures_agree_bitwise(pdg, oracle, kernel, mode, mtype):
    # one launch per sweep (CUDA graph), one cooperative launch per frame, the
    # resident kernel and the streaming kernel run the same per-vertex
    # arithmetic in the same order (type 3: valence-8 vertices)
    m, c, cfg, sc, a = scene(pdg, oracle, n=33, mtype=mtype, max_iterations=16, mode=mode, kernel=pdg.KERNEL_GRAPH)
    s1 = pdg.Solver(cfg, m, c)
    cfg.kernel = KERNELS[kernel.replace("256", "")]
    if kernel == "resident256":   # two blocks per SM
        cfg.block_threads = 256
    s2 = pdg.Solver(cfg, m, c)
    if kernel == "resident256":
        assert s2.launch_info()["block_threads"] == 256
    assert s1.launch_info()["kernel"] == pdg.KERNEL_GRAPH
    assert s2.launch_info()["kernel"] == cfg.kernel
    for _ in range(3):
        st1 = s1.step(1)[0]
        st2 = s2.step(1)[0]
    x1, v1 = s1.get_state(); x2, v2 = s2.get_state()
    assert np.array_equal(x1, x2) and np.array_equal(v1, v2)
    assert st1["iterations"] == st2["iterations"]
    if mode == 0:
        assert abs(st1["res_final"] - st2["res_final"]) <= 1e-5 * st1["res_final"]


def test_resident_tolerance_and_batch(pdg, oracle):
    # per-cloth convergence inside one resident launch equals the graph path
    scenes = [scene(pdg, oracle, n=n, seed=n, side=0.5, ks=20.0, kb=1e-3, rho=0.9, max_iterations=400,
                    tolerance=1e-4) for n in (9, 10, 11)]
    outs = []
    for kern in (pdg.KERNEL_GRAPH, pdg.KERNEL_RESIDENT):
        cfgs = []
        for sc_ in scenes:
            sc_[2].kernel = kern
            cfgs.append(sc_[2])
        b = pdg.Solver(cfgs, [sc_[0] for sc_ in scenes], [sc_[1] for sc_ in scenes])
        assert b.launch_info()["kernel"] == kern
        st = b.step(2)
        outs.append((b.get_state_all(), [s_["iterations"] for s_ in st], st))
    assert np.array_equal(outs[0][0][0], outs[1][0][0])
    assert outs[0][1] == outs[1][1]
    assert all(s_["converged"] for s_ in outs[1][2])


def test_patch_size_does_not_change_bits(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=33)
    out = []
    for pv, nt in [(64, 128), (256, 256), (1024, 512)]:
        cfg.patch_verts, cfg.block_threads = pv, nt
        s = pdg.Solver(cfg, m, c)
        s.step(2, stats=False)
        out.append(s.get_state())
    for x, v in out[1:]:
        assert np.array_equal(x, out[0][0]) and np.array_equal(v, out[0][1])


def test_batch_equals_single(pdg, oracle):
    scenes = [scene(pdg, oracle, n=n, seed=n, ks=k, kb=kb) for n, k, kb in [(9, 1e2, 1e-3), (17, 1e3, 1e-2), (12, 5e3, 0.0)]]
    singles = []
    for m, c, cfg, sc, a in scenes:
        s = pdg.Solver(cfg, m, c)
        s.step(2, stats=False)
        singles.append(s.get_state())
    b = pdg.Solver([sc_[2] for sc_ in scenes], [sc_[0] for sc_ in scenes], [sc_[1] for sc_ in scenes])
    b.step(2, stats=False)
    for i, (x, v) in enumerate(singles):
        xb, vb = b.get_state(i)
        assert np.array_equal(x, xb) and np.array_equal(v, vb)
    xa, va = b.get_state_all()
    assert np.array_equal(xa[b.offsets[1]:b.offsets[2]], singles[1][0])


def test_tolerance_mode_stops_like_oracle(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=9, side=0.5, ks=20.0, kb=1e-3, max_iterations=400, tolerance=1e-4,
                             rho=0.9)
    s = pdg.Solver(cfg, m, c)
    st = s.step(1)[0]
    x0 = a["rest"].astype(np.float64).reshape(-1)
    xo, vo, info = sc.step_jacobi(x0, np.zeros_like(x0), 400, tol=1e-4, rho=0.9)
    assert st["converged"] == 1 and st["rel_residual"] <= 1e-4
    assert abs(st["iterations"] - info["used"]) <= 2
    x, v = s.get_state()
    assert rel(x, xo) < 1e-5


def test_deterministic(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=33)
    r = []
    for _ in range(2):
        s = pdg.Solver(cfg, m, c)
        s.step(3, stats=False)
        r.append(s.get_state())
    assert np.array_equal(r[0][0], r[1][0]) and np.array_equal(r[0][1], r[1][1])


def test_state_roundtrip_and_free_fall(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=9, ks=0.0, kb=0.0, pins="none", max_iterations=5)
    s = pdg.Solver(cfg, m, c)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(m.N, 3)).astype(np.float32); v = rng.normal(size=(m.N, 3)).astype(np.float32)
    s.set_state(x, v)
    x2, v2 = s.get_state()
    assert np.array_equal(x, x2) and np.array_equal(v, v2)
    s.step(1, stats=False)
    x3, v3 = s.get_state()
    h = np.float32(cfg.dt)
    expect = x + h * v + h * h * np.array([0, cfg.gravity, 0], np.float32)
    assert np.allclose(x3, expect, rtol=0, atol=1e-6)


@pytest.mark.parametrize("kernel", [1, 3])
def test_step_host_equals_set_step_get(pdg, oracle, kernel):
    # pdg_solver_step_host is set_state_all + step + get_state_all in one call
    ms, cs, cfgs = [], [], []
    for i, n in enumerate((9, 17)):
        m, c, cfg, sc, a = scene(pdg, oracle, n=n, seed=i, kernel=kernel)
        ms.append(m); cs.append(c); cfgs.append(cfg)
    s1 = pdg.Solver(cfgs, ms, cs)
    s2 = pdg.Solver(cfgs, ms, cs)
    n = int(s1.offsets[-1])
    rng = np.random.default_rng(3)
    rest = np.concatenate([np.asarray(m.arrays()["rest"]).reshape(-1, 3) for m in ms])
    x = (rest + rng.normal(0, 1e-3, (n, 3))).astype(np.float32)
    v = rng.normal(0, 1e-2, (n, 3)).astype(np.float32)
    for f in range(3):
        s1.set_state_all(x, v); s1.step(1, stats=False); xa, va = s1.get_state_all()
        xb, vb = np.empty_like(x), np.empty_like(v)
        st = s2.step_host(x, v, xb, vb, stats=True)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)
        assert [t["iterations"] for t in st] == [10, 10]
        x, v = xb, vb
    # in place, and with the state kept on the device (no inputs)
    xc, vc = x.copy(), v.copy()
    s1.set_state_all(x, v); s1.step(2, stats=False); xa, va = s1.get_state_all()
    s2.step_host(xc, vc, xc, vc)
    s2.step_host(None, None, xc, None)
    assert np.array_equal(xa, xc)
    # page-locked buffers are read and written in place by the copy kernels
    torch = pytest.importorskip("torch")
    px = torch.empty((n, 3), dtype=torch.float32).pin_memory().numpy()
    pv = torch.empty((n, 3), dtype=torch.float32).pin_memory().numpy()
    px[:] = x; pv[:] = v
    s1.set_state_all(x, v); s1.step(1, stats=False); xa, va = s1.get_state_all()
    s2.step_host(px, pv, px, pv)
    assert np.array_equal(xa, px) and np.array_equal(va, pv)
    qx = torch.empty((n, 3), dtype=torch.float32).pin_memory().numpy()
    s1.step(1, stats=False); xa, _ = s1.get_state_all()
    s2.step_host(None, None, qx, None)   # pinned output, no input
    assert np.array_equal(xa, qx)


@pytest.mark.parametrize("kernel", [1, 3])
def test_step_host_several_frames_mixed_buffers(pdg, oracle, kernel):
    # Inputs are taken by the first frame of a call and outputs written by the
    # last (the resident kernel does both inside its frame launch); pageable
    # and page-locked buffers mix freely; an absent input keeps the state.
    torch = pytest.importorskip("torch")
    ms, cs, cfgs = [], [], []
    for i, n in enumerate((9, 17)):
        m, c, cfg, sc, a = scene(pdg, oracle, n=n, seed=i + 5, kernel=kernel)
        ms.append(m); cs.append(c); cfgs.append(cfg)
    s1 = pdg.Solver(cfgs, ms, cs)
    s2 = pdg.Solver(cfgs, ms, cs)
    n = int(s1.offsets[-1])
    rng = np.random.default_rng(11)
    rest = np.concatenate([np.asarray(m.arrays()["rest"]).reshape(-1, 3) for m in ms])
    x = (rest + rng.normal(0, 1e-3, (n, 3))).astype(np.float32)
    v = rng.normal(0, 1e-2, (n, 3)).astype(np.float32)
    pinned = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    # three frames in one call: pinned x in, pageable v in, pageable x out, pinned v out
    s1.set_state_all(x, v); s1.step(3, stats=False); xa, va = s1.get_state_all()
    px, qv = pinned(x), pinned(np.zeros_like(v))
    xo = np.full_like(x, np.nan)
    st = s2.step_host(px, v.copy(), xo, qv, nframes=3, stats=True)
    assert np.array_equal(xa, xo) and np.array_equal(va, qv)
    assert all(t["status"] == 0 for t in st)
    assert np.array_equal(px, x)   # an input that is not also an output stays as it was
    # x alone in (v stays the solver's own), both out into one pageable pair
    x2 = (xa + rng.normal(0, 1e-3, (n, 3))).astype(np.float32)
    s1.set_state_all(x2, None); s1.step(1, stats=False); xb, vb = s1.get_state_all()
    xo2, vo2 = np.empty_like(x), np.empty_like(v)
    s2.step_host(x2, None, xo2, vo2)
    assert np.array_equal(xb, xo2) and np.array_equal(vb, vo2)
    # v alone in from pinned memory, two frames, x alone out in place of the input buffer
    v3 = pinned(rng.normal(0, 1e-2, (n, 3)).astype(np.float32))
    s1.set_state_all(None, v3); s1.step(2, stats=False); xc, vc = s1.get_state_all()
    s2.step_host(None, v3, None, None, nframes=2)
    xo3 = pinned(np.zeros_like(x))
    s2.step_host(None, None, xo3, v3, nframes=0)   # no frame: the copies alone
    assert np.array_equal(xc, xo3) and np.array_equal(vc, v3)
    # page-locked arrays that start 4 bytes past a 16-byte boundary (an
    # interior pointer of a page-locked allocation), in place
    buf = pinned(np.zeros(3 * n + 1, np.float32))
    ux = buf[1:].reshape(n, 3)
    ux[:] = xc
    s1.step(1, stats=False); xd, vd = s1.get_state_all()
    s2.step_host(ux, None, ux, None)
    assert np.array_equal(xd, ux) and buf[0] == 0


def test_step_host_large_state_moves_by_dma(pdg):
    # from 4 MB per array the host buffers go through DMA into the staging
    # buffers instead of being read in place: a 641x641 cloth (410,881
    # vertices, 4.9 MB per array) on the streaming kernel, page-locked and
    # pageable buffers, equal bitwise to set_state_all + step + get_state_all
    torch = pytest.importorskip("torch")
    import scenes
    m, c = scenes.hanging(641, 3.0, ks=1e3, kb=1e-2, seed=2)
    cfg = pdg.Config.default(max_iterations=4, tolerance=0.0, rho=0.99, dt=scenes.H, gravity=scenes.G,
                             kernel=pdg.KERNEL_STREAM)
    s1 = pdg.Solver(cfg, m, c)
    s2 = pdg.Solver(cfg, m, c)
    n = m.N
    assert 12 * n >= 4 << 20
    rng = np.random.default_rng(5)
    x = (np.asarray(m.arrays()["rest"]).reshape(-1, 3) + rng.normal(0, 1e-3, (n, 3))).astype(np.float32)
    v = rng.normal(0, 1e-2, (n, 3)).astype(np.float32)
    pinned = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    s1.set_state_all(x, v); s1.step(2, stats=False); xa, va = s1.get_state_all()
    px, pv = pinned(x), pinned(v)
    s2.step_host(px, pv, px, pv, nframes=2)
    assert np.array_equal(xa, px) and np.array_equal(va, pv)
    s1.step(1, stats=False); xb, vb = s1.get_state_all()
    xo, vo = np.full_like(x, np.nan), np.full_like(v, np.nan)
    s2.step_host(px.copy(), pv.copy(), xo, vo)
    assert np.array_equal(xb, xo) and np.array_equal(vb, vo)


def test_apply_pins_device(pdg):
    torch = pytest.importorskip("torch")
    pos = torch.arange(30, dtype=torch.float32, device="cuda")
    vel = torch.ones(30, dtype=torch.float32, device="cuda")
    idx = torch.tensor([1, 7], dtype=torch.int32, device="cuda")
    tgt = torch.tensor([-1, -2, -3, -4, -5, -6], dtype=torch.float32, device="cuda")
    import ctypes
    rc = pdg.lib().pdg_apply_pins(ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(vel.data_ptr()),
                                  ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(tgt.data_ptr()), 2, None)
    assert rc == 0
    torch.cuda.synchronize()
    p = pos.view(10, 3).cpu().numpy(); v = vel.view(10, 3).cpu().numpy()
    assert np.array_equal(p[1], [-1, -2, -3]) and np.array_equal(p[7], [-4, -5, -6])
    assert np.all(v[[1, 7]] == 0) and np.all(v[[0, 2, 3]] == 1)


def test_nan_input_is_reported(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=9)
    s = pdg.Solver(cfg, m, c)
    x = a["rest"].copy(); x[4, 1] = np.nan
    s.set_state(x, np.zeros_like(x))
    st = s.step(1)[0]
    assert st["status"] == pdg.ERR_NUMERIC
    x2, v2 = s.get_state()
    assert np.all(v2[np.isfinite(x2).all(1)] == 0)


def test_pin_targets_move(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=9)
    s = pdg.Solver(cfg, m, c)
    t = c.arrays()["targets"] + np.array([0.0, 0.1, 0.0], np.float32)
    s.set_pin_targets(t)
    s.step(1, stats=False)
    x, v = s.get_state()
    assert np.allclose(x[[0, 8]], t) and np.all(v[[0, 8]] == 0)


@pytest.mark.parametrize("nr,mtype", [(2, 0), (3, 3), (5, 2)])
def test_small_and_other_meshes(pdg, oracle, nr, mtype):
    m, c, cfg, sc, a = scene(pdg, oracle, n=nr, mtype=mtype, max_iterations=6)
    s = pdg.Solver(cfg, m, c)
    s.step(1, stats=False)
    x, v = s.get_state()
    xo, vo, _ = sc.step_jacobi(a["rest"].reshape(-1), np.zeros(3 * m.N), 6, rho=0.99)
    assert rel(x, xo) < REL_ONE_FRAME


def test_zero_iterations(pdg, oracle):
    m, c, cfg, sc, a = scene(pdg, oracle, n=9, max_iterations=0)
    s = pdg.Solver(cfg, m, c)
    st = s.step(1)[0]
    x, v = s.get_state()
    y = sc.predict(a["rest"], np.zeros_like(a["rest"])).reshape(-1, 3)
    y[[0, 8]] = a["rest"][[0, 8]]
    assert np.allclose(x, y, atol=1e-7) and st["iterations"] == 0


@pytest.mark.parametrize("kernel", ["persistent", "resident", "stream"])
def test_bounded_waits_run_out_cleanly(pdg, oracle, kernel):
    # failure detection without a GPU fault: a wait budget of one cycle makes
    # every grid-barrier / neighbour wait run out; the kernel records the
    # error, all blocks leave, the host reads PDG_ERR_TIMEOUT, and the next
    # frame with a normal budget runs on the same context
    m, c, cfg, sc, a = scene(pdg, oracle, n=33, max_iterations=8)
    cfg.kernel = KERNELS[kernel]
    s = pdg.Solver(cfg, m, c)
    s.set_wait_budget(1)
    with pytest.raises(pdg.PDGError) as e:
        s.step(1)
    assert e.value.code == pdg.ERR_TIMEOUT
    s.set_wait_budget(2_000_000_000)
    s.set_state(a["rest"], np.zeros_like(a["rest"]))
    st = s.step(1)[0]
    x, v = s.get_state()
    cfg.kernel = pdg.KERNEL_GRAPH
    ref = pdg.Solver(cfg, m, c)
    ref.step(1, stats=False)
    assert np.array_equal(x, ref.get_state()[0]) and st["status"] == 0


def test_resident_exchange_tags_restart_before_they_wrap(pdg, oracle):
    # the resident kernel's neighbour exchange tags each published offset with
    # a 32-bit number from a device word that grows by the frame's sweep
    # count every frame; starting 40 below 2^32, the third frame's tags would
    # pass it, so that frame clears its patches' exchange words and restarts
    # the numbers.  Every frame must still give the per-sweep graph solver's
    # bits: a restart from a low number after the words hold high tags must
    # not read stale words.
    m, c, cfg, sc, a = scene(pdg, oracle, n=33, max_iterations=16, kernel=pdg.KERNEL_GRAPH)
    ref = pdg.Solver(cfg, m, c)
    cfg.kernel = pdg.KERNEL_RESIDENT
    s = pdg.Solver(cfg, m, c)
    assert s.launch_info()["kernel"] == pdg.KERNEL_RESIDENT
    s.set_frame_tag(2**32 - 40)
    for f in range(4):
        ref.step(1, stats=False)
        st = s.step(1)[0]
        assert st["status"] == 0
        assert np.array_equal(s.get_state()[0], ref.get_state()[0]), f


def test_autotuner_picks_a_plan_and_keeps_the_bits(pdg, oracle):
    # every candidate plan computes the same iterates, so the tuned solver
    # must equal the per-sweep graph solver bit for bit; the second creation
    # of the same problem shape comes from the cache
    pdg.autotune_clear_cache()
    m, c, cfg, sc, a = scene(pdg, oracle, n=65, max_iterations=12, kernel=pdg.KERNEL_AUTOTUNE)
    s = pdg.Solver(cfg, m, c)
    table = s.tune_results()
    timed = [t for t in table if t["frame_ms"] >= 0]
    assert len(timed) >= 2 and sum(t["chosen"] for t in table) == 1
    best = min(timed, key=lambda t: t["frame_ms"])
    info = s.launch_info()
    assert best["chosen"] == 1 and (info["kernel"], info["patch_verts"], info["block_threads"]) == \
        (best["kernel"], best["patch_verts"], best["block_threads"])
    assert not any(t["cached"] for t in table)
    s.step(2, stats=False)
    cfg.kernel = pdg.KERNEL_GRAPH
    g = pdg.Solver(cfg, m, c)
    g.step(2, stats=False)
    assert all(np.array_equal(u, w) for u, w in zip(s.get_state(), g.get_state()))
    cfg.kernel = pdg.KERNEL_AUTOTUNE
    s2 = pdg.Solver(cfg, m, c)
    assert all(t["cached"] for t in s2.tune_results())
    assert s2.launch_info() == info


def test_stream_kernel_walks_many_patches_per_block(pdg, oracle):
    # 513x513 cloth in 64-vertex patches: several thousand patches over at
    # most a few blocks per SM, so every block double-buffers several patches
    m, c, cfg, sc, a = scene(pdg, oracle, n=513, side=2.0, max_iterations=8, kernel=pdg.KERNEL_GRAPH,
                             patch_verts=64, block_threads=128)
    g = pdg.Solver(cfg, m, c)
    cfg.kernel = pdg.KERNEL_STREAM
    s = pdg.Solver(cfg, m, c)
    info = s.launch_info()
    assert info["kernel"] == pdg.KERNEL_STREAM and info["npatches"] > 3 * 152
    stg = g.step(2); sts = s.step(2)
    assert all(np.array_equal(u, w) for u, w in zip(g.get_state(), s.get_state()))
    assert abs(stg[0]["res_final"] - sts[0]["res_final"]) <= 1e-5 * stg[0]["res_final"]


def test_stream_sweeps_overlapping_their_predecessor_match_graph(pdg, oracle):
    # Each streaming sweep after the first is a programmatic dependent launch
    # of the previous one: its blocks start while that sweep's last blocks
    # still run and stage what the previous sweep does not write.  Many
    # frames of 24 sweeps, through the frame's CUDA graph and through the
    # eagerly launched timing path, must keep the bits of the per-patch graph
    # kernel.
    m, c, cfg, sc, a = scene(pdg, oracle, n=257, side=2.0, max_iterations=24, kernel=pdg.KERNEL_GRAPH,
                             patch_verts=128, block_threads=128)
    g = pdg.Solver(cfg, m, c)
    cfg.kernel = pdg.KERNEL_STREAM
    s = pdg.Solver(cfg, m, c)
    assert s.launch_info()["kernel"] == pdg.KERNEL_STREAM
    for _ in range(3):
        stg = g.step(2)
        sts = s.step(2)
        assert all(np.array_equal(u, w) for u, w in zip(g.get_state(), s.get_state()))
        # the per-sweep sums are double atomics, so only their order may differ
        assert abs(stg[0]["res_final"] - sts[0]["res_final"]) <= 1e-9 * stg[0]["res_final"]
    g.time_frames(3)
    s.time_frames(3)
    assert all(np.array_equal(u, w) for u, w in zip(g.get_state(), s.get_state()))


def test_auto_plan_streams_what_the_resident_kernel_cannot_hold(pdg, oracle):
    # 513x513 cloth: more 448-vertex patches than SMs, so AUTO falls back to
    # the streaming kernel at its default 256-vertex / 256-thread plan
    m, c, cfg, sc, a = scene(pdg, oracle, n=513, side=2.0, max_iterations=8, kernel=pdg.KERNEL_AUTO)
    s = pdg.Solver(cfg, m, c)
    info = s.launch_info()
    assert info["kernel"] == pdg.KERNEL_STREAM
    assert (info["patch_verts"], info["block_threads"]) == (256, 256)
    cfg.kernel = pdg.KERNEL_GRAPH
    g = pdg.Solver(cfg, m, c)
    s.step(1, stats=False); g.step(1, stats=False)
    assert all(np.array_equal(u, w) for u, w in zip(g.get_state(), s.get_state()))


def test_stream_kernel_tolerance_batch(pdg, oracle):
    scenes = [scene(pdg, oracle, n=n, seed=n, side=0.5, ks=20.0, kb=1e-3, rho=0.9, max_iterations=400,
                    tolerance=1e-4) for n in (9, 10, 11, 40)]
    outs = []
    for kern in (pdg.KERNEL_GRAPH, pdg.KERNEL_STREAM):
        for sc_ in scenes:
            sc_[2].kernel = kern
        b = pdg.Solver([sc_[2] for sc_ in scenes], [sc_[0] for sc_ in scenes], [sc_[1] for sc_ in scenes])
        assert b.launch_info()["kernel"] == kern
        st = b.step(2)
        outs.append((b.get_state_all(), [s_["iterations"] for s_ in st]))
    assert np.array_equal(outs[0][0][0], outs[1][0][0]) and np.array_equal(outs[0][0][1], outs[1][0][1])
    assert outs[0][1] == outs[1][1]


def test_converged_solve_matches_direct_local_global(pdg, oracle):
    # parity protocol: the fused consistent iteration run to convergence
    # reaches the fixed point of the oracle's direct local/global solve
    # (sparse LDL^T global step every iteration, consistent pin
    # elimination, float64) within 1e-5 relative in positions
    m, c, cfg, sc, a = scene(pdg, oracle, n=17, side=1.0, ks=20.0, kb=1e-3, rho=0.9, max_iterations=6000)
    s = pdg.Solver(cfg, m, c)
    st = s.step(1)[0]
    x, v = s.get_state()
    x0 = a["rest"].astype(np.float64).reshape(-1)
    xd, vd = sc.step_direct(x0, np.zeros_like(x0), iters=1500, pin_elim=1, with_bend=True)
    assert st["iterations"] == 6000
    assert rel(x, xd) < 1e-5


def irregular_mesh(n=24, drop=0.12, seed=3):
    """Grid with a random diagonal per cell and a random 12 % of triangles
    removed (holes, inner boundaries, valence 1..8), unreferenced vertices
    dropped; rest in the x-y plane with z-jitter."""
    rng = np.random.default_rng(seed)
    pos = np.array([[j / (n - 1), -i / (n - 1), 1e-4 * rng.standard_normal()] for i in range(n) for j in range(n)],
                   np.float32)
    tris = []
    for i in range(n - 1):
        for j in range(n - 1):
            a, b, c, d = i * n + j, i * n + j + 1, (i + 1) * n + j, (i + 1) * n + j + 1
            tris += [[a, c, b], [b, c, d]] if rng.random() < 0.5 else [[a, c, d], [a, d, b]]
    tris = np.array(tris, np.int32)
    tris = tris[rng.random(len(tris)) >= drop]
    used = np.unique(tris)
    remap = -np.ones(len(pos), np.int64); remap[used] = np.arange(len(used))
    return pos[used], remap[tris].astype(np.int32)


@pytest.mark.parametrize("kernel", ["persistent", "resident", "resident256", "stream"])
def test_irregular_mesh(pdg, oracle, kernel):
    # mixed valence, holes and inner boundaries: one frame against the f64
    # oracle, and every launch structure bitwise equal to the graph path
    pos, tris = irregular_mesh()
    m = pdg.Mesh.create(pos, tris, density=0.1)
    c = pdg.Constraints(m).build_stretch(1e3).build_bend(1e-2)
    top = np.where(pos[:, 1] > -1e-6)[0]
    c.set_pins(top[[0, -1]])
    cfg = pdg.Config.default(max_iterations=10, rho=0.99, dt=1 / 60, gravity=-9.81, kernel=pdg.KERNEL_GRAPH)
    g = pdg.Solver(cfg, m, c)
    stg = g.step(2)
    a = m.arrays(); ca = c.arrays()
    sc = oracle.Scene(a["rest"], a["tris"], k_stretch=ca["k_stretch"], k_bend=1e-2, pins=ca["pins"], h=cfg.dt,
                      gravity=cfg.gravity)
    x = a["rest"].astype(np.float64).reshape(-1); v = np.zeros_like(x)
    for _ in range(2):
        x, v, _ = sc.step_jacobi(x, v, 10, rho=0.99)
    xg, vg = g.get_state()
    assert rel(xg, x) < REL_ONE_FRAME
    cfg.kernel = KERNELS[kernel.replace("256", "")]
    if kernel == "resident256":
        cfg.block_threads = 256
    s = pdg.Solver(cfg, m, c)
    s.step(2)
    assert all(np.array_equal(u, w) for u, w in zip(g.get_state(), s.get_state()))


def test_batch_with_a_single_triangle_cloth(pdg, oracle):
    # ragged batch: a 3-vertex cloth without hinges beside a regular one;
    # each equals its own single-cloth solve
    tri = pdg.Mesh.create(np.array([[0, 0, 0], [0.1, 0, 0], [0, -0.1, 0.001]], np.float32),
                          np.array([[0, 1, 2]], np.int32))
    ct = pdg.Constraints(tri).build_stretch(100.0).set_pins([0])
    m, c, cfg, sc, a = scene(pdg, oracle, n=9)
    cfg_t = pdg.Config.default(max_iterations=10, rho=0.99, dt=1 / 60, gravity=-9.81)
    singles = []
    for mm, cc, cf in [(tri, ct, cfg_t), (m, c, cfg)]:
        s = pdg.Solver(cf, mm, cc)
        s.step(3, stats=False)
        singles.append(s.get_state())
    for kern in (pdg.KERNEL_GRAPH, pdg.KERNEL_RESIDENT):
        cfg_t.kernel = cfg.kernel = kern
        b = pdg.Solver([cfg_t, cfg], [tri, m], [ct, c])
        b.step(3, stats=False)
        for i in range(2):
            assert all(np.array_equal(u, w) for u, w in zip(b.get_state(i), singles[i]))
    xt = singles[0][0]
    assert np.array_equal(xt[0], np.array([0, 0, 0], np.float32))   # pinned corner stays
    assert np.all(np.isfinite(xt))


def test_set_pins_on_a_live_solver_equals_a_solver_built_with_them(pdg, oracle):
    # Constraints::set_from_list + upload_to_gpu on a running solver: the new
    # pin set (with moved targets) gives the bits of a solver created with it
    n = 17
    m, c, cfg, sc, a = scene(pdg, oracle, n=n, max_iterations=12)
    s = pdg.Solver(cfg, m, c)
    s.step(2, stats=False)
    x, v = s.get_state()
    top = np.arange(n, dtype=np.int32)
    tgt = a["rest"][top] + np.array([0.0, 0.01, 0.02], np.float32)
    _check = pdg._check
    _check(pdg.lib().pdg_solver_set_pins(s.h, 0, pdg._p(top), len(top), pdg._p(np.ascontiguousarray(tgt))))
    s.step(2, stats=False)
    got = s.get_state()
    c2 = pdg.Constraints(m).build_stretch(1e3).build_bend(1e-2).set_pins(top, tgt)
    s2 = pdg.Solver(cfg, m, c2)
    s2.set_state(x, v)
    s2.step(2, stats=False)
    ref = s2.get_state()
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    assert np.allclose(got[0][top], tgt) and np.all(got[1][top] == 0)
    with pytest.raises(pdg.PDGError):
        _check(pdg.lib().pdg_solver_set_pins(s.h, 0, pdg._p(np.array([0, 0], np.int32)), 2, None))
