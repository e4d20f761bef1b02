"""The oracle against the reference's own known answers (CPU).

The reference ships no golden vectors; its unit tests pin invariants of the
setup stage, restated here against the oracle:
  src/tests/test_mesh.cpp:13-70        mass conservation, Dm_inv * Dm = I, dF/dx x = vec(F)
  src/tests/test_topology.cpp:17-61    inner-edge counts, edge validity, vert->tri coverage
  src/tests/test_constraints.cpp:10-27 pin presets
plus checks of the oracle's own algebra (polar vs SVD, LDL^T vs scipy) and
the physical known answers the reference does not test.
"""
import numpy as np
import pytest


def _grid(O, n, m, size, mtype):
    pos, tris = O.generate_grid(n, m, size, mtype)
    return pos, tris


def test_mass_conservation(oracle):
    pos, tris = _grid(oracle, 10, 10, 0.1, 0)
    G, area, mass = oracle.rest_state(pos, tris, 0.1)
    expected = 0.1 * area.sum()
    assert abs(mass.sum() - expected) / expected < 1e-5


@pytest.mark.parametrize("mtype", [0, 1, 2, 3])
def test_dm_inv_inverts_dm(oracle, mtype):
    pos, tris = _grid(oracle, 10, 10, 0.1, mtype)
    G, area, mass = oracle.rest_state(pos, tris, 0.1)
    for t in range(len(tris)):
        i0, i1, i2 = tris[t]
        e = np.stack([pos[i1] - pos[i0], pos[i2] - pos[i0]], 1)
        p0 = e[:, 0] / np.linalg.norm(e[:, 0])
        o = e[:, 1] - e[:, 1].dot(p0) * p0
        P = np.stack([p0, o / np.linalg.norm(o)], 1)
        Dm = P.T @ e
        Ginv = np.array([[G[t, 0], G[t, 2]], [G[t, 1], G[t, 3]]])
        assert np.linalg.norm(Ginv @ Dm - np.eye(2)) < 1e-4


def test_dfdx_maps_rest_to_F(oracle):
    pos, tris = _grid(oracle, 10, 10, 0.1, 0)
    G, area, mass, dfdx = oracle.rest_state(pos, tris, 0.1, with_dfdx=True)
    for t in range(10):
        i0, i1, i2 = tris[t]
        x = np.concatenate([pos[i0], pos[i1], pos[i2]])
        Ginv = np.array([[G[t, 0], G[t, 2]], [G[t, 1], G[t, 3]]])
        F = np.stack([pos[i1] - pos[i0], pos[i2] - pos[i0]], 1) @ Ginv
        assert np.linalg.norm(dfdx[t] @ x - np.concatenate([F[:, 0], F[:, 1]])) < 1e-4


@pytest.mark.parametrize("n,expect", [(3, 8), (4, 21), (10, 225)])
def test_inner_edge_counts_type0(oracle, n, expect):
    pos, tris = _grid(oracle, n, n, 1.0, 0)
    e = oracle.topology(len(pos), tris)
    assert int((e[:, 3] != -1).sum()) == expect


@pytest.mark.parametrize("mtype", [0, 1, 2])
def test_inner_edge_counts_3x3_types(oracle, mtype):
    pos, tris = _grid(oracle, 3, 3, 1.0, mtype)
    e = oracle.topology(len(pos), tris)
    assert int((e[:, 3] != -1).sum()) == 8


def test_edges_valid_and_vert_tri_cover(oracle):
    pos, tris = _grid(oracle, 5, 5, 1.0, 3)
    e = oracle.topology(len(pos), tris)
    assert np.all(e[:, 0] < e[:, 1])
    # every triangle side is an edge whose tri_a/tri_b includes that triangle
    key = {(a, b): (ta, tb) for a, b, ta, tb in e}
    for t, tri in enumerate(tris):
        for s in range(3):
            a, b = sorted((tri[s], tri[(s + 1) % 3]))
            assert t in key[(a, b)]


def test_pin_presets(oracle):
    # Constraints::pin_top_row / pin_corners on a 10x10 grid
    ncols = 10
    top = list(range(ncols))
    corners = [0, ncols - 1]
    pos, tris = _grid(oracle, 10, 10, 0.1, 0)
    sc = oracle.Scene(pos, tris, pins=corners)
    assert list(sc.pins) == corners and np.allclose(sc.pin_targets, pos[corners])
    sc = oracle.Scene(pos, tris, pins=top)
    assert len(sc.pins) == 10 and sc.pins[0] == 0 and sc.pins[9] == 9


def test_flat_rest_bend_norm_zero(oracle):
    pos, tris = _grid(oracle, 6, 6, 0.1, 1)
    sc = oracle.Scene(pos, tris, k_bend=1e-2)
    assert len(sc.hinge) == int((sc.edges[:, 3] != -1).sum())
    assert np.abs(sc.nrest).max() < 1e-5
    # cotangent weights of a hinge sum to zero (translation invariance)
    assert np.abs(sc.w.sum(1)).max() < 1e-4


def _polar_np(F):
    """closest rotation of the Gram-Schmidt-projected F via numpy SVD with
    the determinant fix of src/stretch_reference.cpp:56-65"""
    b0 = F[:, 0] / np.linalg.norm(F[:, 0])
    c1 = F[:, 1] - F[:, 1].dot(b0) * b0
    b1 = c1 / np.linalg.norm(c1)
    B = np.stack([b0, b1], 1)
    U, S, Vt = np.linalg.svd(B.T @ F)
    R2 = U @ Vt
    if np.linalg.det(R2) < 0:
        U[:, 1] *= -1
        R2 = U @ Vt
    return B @ R2


def test_polar_matches_svd(oracle):
    rng = np.random.default_rng(1)
    # single triangle: random deformation of a rest triangle, compare the
    # oracle's stretch residual with the SVD-based projection
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    tris = np.array([[0, 1, 2]], np.int32)
    sc = oracle.Scene(pos, tris, k_stretch=1.0, k_bend=0.0, h=1.0, gravity=0.0)
    G = np.array([[sc.G[0, 0], sc.G[0, 2]], [sc.G[0, 1], sc.G[0, 3]]], np.float64)
    for _ in range(20):
        x = pos.astype(np.float64) + rng.normal(0, 0.3, (3, 3))
        F = np.stack([x[1] - x[0], x[2] - x[0]], 1) @ G
        R = _polar_np(F)
        # r = A^T (F - R) * h^2 wA with y = x  ->  compare the vertex-1 force
        n, r = sc.residual(x.reshape(-1), x.reshape(-1))
        wA = sc.k_stretch[0] * sc.area[0]
        q = wA * (F - R)
        f1 = G[0, 0] * q[:, 0] + G[0, 1] * q[:, 1]
        assert np.allclose(r[3:6], f1, atol=1e-9)


def test_ldlt_matches_scipy(oracle):
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    pos, tris, pins = oracle.hanging_cloth(9, 1.0)
    sc = oracle.Scene(pos, tris, k_stretch=1e3, k_bend=1e-2, pins=pins)
    ri, ci, val = sc.global_matrix(with_bend=True)
    K = sp.csr_matrix((val, (ri, ci)), shape=(3 * sc.N, 3 * sc.N))
    assert abs(K - K.T).max() < 1e-12
    # one direct local/global iteration from rest = K^-1 b; rebuild b here
    x0 = pos.astype(np.float64).reshape(-1)
    v0 = np.zeros_like(x0)
    x1, _ = sc.step_direct(x0, v0, iters=1, pin_elim=1, with_bend=True)
    # residual of the linear system at the oracle's solution must vanish:
    # K x1 = M y + h^2 sum wA A^T R(x0) + h^2 sum k w p(x0) (consistent pins)
    y = sc.predict(x0, v0).reshape(-1)
    r_lin = K @ x1
    # the same right-hand side, formed through the residual function at x0:
    # r(x) = M(x - y) + h^2 (K_s x - b_s)  =>  b = K x0 - r(x0) (free rows)
    n0, r0 = sc.residual(y, x0)
    b = K @ x0 - r0.reshape(-1)
    free = np.ones(sc.N, bool); free[sc.pins] = False
    fd = np.repeat(free, 3)
    assert np.allclose(r_lin[fd], b[fd], rtol=1e-9, atol=1e-12)
    x_sp = spla.spsolve(K.tocsc(), np.where(fd, b, x1))
    assert np.allclose(x_sp, x1, rtol=1e-9, atol=1e-12)


def test_free_fall_known_answer(oracle):
    # no constraints: x_{n+1} = x_n + h v + h^2 g exactly, v_{n+1} = v + h g
    pos, tris = _grid(oracle, 5, 5, 0.1, 1)
    sc = oracle.Scene(pos, tris, k_stretch=0.0, k_bend=0.0, gravity=-9.81, h=0.01)
    x = pos.astype(np.float64).reshape(-1); v = np.zeros_like(x)
    x1, v1, info = sc.step_jacobi(x, v, 5, rho=0.99)
    expect = x.reshape(-1, 3) + np.array([0, -9.81 * 1e-4, 0])
    assert np.allclose(x1.reshape(-1, 3), expect, atol=1e-12)
    assert np.allclose(v1.reshape(-1, 3)[:, 1], -9.81 * 0.01 * 1.0, atol=1e-9)


def test_rest_state_static_consistent(oracle):
    # rest shape, g = 0: the consistent step keeps the cloth still
    # (the reference's literal x = rhs/diag step, src/pd_solver.cu:371-398,
    # does not)
    pos, tris = _grid(oracle, 10, 10, 0.1, 0)
    sc = oracle.Scene(pos, tris, k_stretch=1e3, k_bend=1.0, gravity=0.0, h=0.01, pins=[0, 9])
    x = pos.astype(np.float64).reshape(-1); v = np.zeros_like(x)
    x1, v1, info = sc.step_jacobi(x, v, 50, rho=0.99)
    # the rest constants are float32, so the rest shape is static to ~1e-6 m/s
    assert np.abs(v1).max() < 1e-5
    xl, vl = sc.step_literal(pos.reshape(-1), np.zeros(3 * sc.N, np.float32), 50)
    assert np.abs(vl).max() > 1.0


def test_rigid_motion_invariance(oracle):
    # stretch/bend residual is invariant under rigid motion of a rest mesh
    pos, tris = _grid(oracle, 6, 6, 0.1, 1)
    sc = oracle.Scene(pos, tris, k_stretch=1e3, k_bend=1e-1, gravity=0.0)
    th = 0.7
    Rz = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    x = (pos.astype(np.float64) @ Rz.T + np.array([0.3, -1.0, 2.0])).reshape(-1)
    n, r = sc.residual(x, x)
    n_strained, _ = sc.residual(x * 1.01, x * 1.01)   # 1 % uniform stretch
    assert n < 1e-5 * n_strained


def test_direct_and_jacobi_same_fixed_point(oracle):
    # soft cloth: Chebyshev-Jacobi iterated to convergence reaches the fixed
    # point of the direct local/global solve (consistent pin elimination)
    pos, tris, pins = oracle.hanging_cloth(9, 0.5)
    sc = oracle.Scene(pos, tris, k_stretch=20.0, k_bend=1e-3, pins=pins, h=1 / 60)
    x = pos.astype(np.float64).reshape(-1); v = np.zeros_like(x)
    xd, vd = sc.step_direct(x, v, iters=1000, pin_elim=1, with_bend=True)
    xj, vj, info = sc.step_jacobi(x, v, 4000, tol=1e-12, rho=0.9)
    assert np.linalg.norm(xj - xd) / np.linalg.norm(xd) < 1e-7


def test_reference_pin_elimination_is_inconsistent(oracle):
    # The reference's CPU pin elimination zeroes pinned rows/columns without
    # moving K_fp x_p to the right-hand side, which drags the free vertices
    # toward the origin
    pos, tris = _grid(oracle, 10, 10, 0.1, 0)
    sc = oracle.Scene(pos, tris, k_stretch=1e3, k_bend=0.0, gravity=0.0, h=0.01, pins=[0, 9])
    x = pos.astype(np.float64).reshape(-1); v = np.zeros_like(x)
    _, v_ref = sc.step_direct(x, v, iters=50, pin_elim=0)
    _, v_ok = sc.step_direct(x, v, iters=50, pin_elim=1)
    assert np.abs(v_ref).max() > 1.0
    assert np.abs(v_ok).max() < 1e-5   # float32 rest constants: static to ~1e-6 m/s
