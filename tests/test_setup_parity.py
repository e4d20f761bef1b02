"""Host setup of the library (through the C ABI) against the oracle (CPU).

Covers ClothMesh::precompute_rest_state, MeshTopology::build,
SimConstraints::build_bend / precompute_jacobi_diag, the pin presets and the
generators, on every mesh type and on ragged and single-cell meshes.
Bit-exact: both sides compute the same float32 arithmetic in the same order.
"""
import numpy as np
import pytest


MESHES = [(2, 2, 0), (3, 3, 1), (5, 7, 2), (9, 9, 3), (33, 33, 1), (17, 5, 1)]


@pytest.mark.parametrize("nr,nc,mtype", MESHES)
def test_generator_matches(pdg, oracle, nr, nc, mtype):
    m = pdg.Mesh.generate(nr, nc, 0.05, mtype)
    a = m.arrays()
    pos, tris = oracle.generate_grid(nr, nc, 0.05, mtype)
    assert np.array_equal(a["rest"], pos) and np.array_equal(a["tris"], tris)


@pytest.mark.parametrize("nr,nc,mtype", MESHES)
def test_rest_state_bitexact(pdg, oracle, nr, nc, mtype):
    m = pdg.Mesh.hanging(nr, 0.8, mtype=mtype, jitter=1e-4, seed=3, ncols=nc)
    a = m.arrays()
    G, area, mass, dfdx = oracle.rest_state(a["rest"], a["tris"], 0.1, with_dfdx=True)
    assert np.array_equal(G, a["Dm_inv"])
    assert np.array_equal(area, a["area"])
    assert np.array_equal(mass, a["mass"])
    assert np.array_equal(dfdx, a["dFdx"])


@pytest.mark.parametrize("nr,nc,mtype", MESHES)
def test_topology_and_bend_bitexact(pdg, oracle, nr, nc, mtype):
    m = pdg.Mesh.hanging(nr, 0.8, mtype=mtype, jitter=1e-4, seed=5, ncols=nc)
    a = m.arrays()
    t = m.topology()
    e = oracle.topology(m.N, a["tris"])
    assert np.array_equal(t["edges"], e)
    assert t["num_inner"] == int((e[:, 3] >= 0).sum())
    lens = np.linalg.norm(a["rest"][e[:, 1]] - a["rest"][e[:, 0]], axis=1)
    assert np.allclose(t["rest_len"], lens, rtol=1e-6)
    # vertex -> triangle lists cover every corner, in triangle order
    for v in range(0, m.N, max(1, m.N // 50)):
        lst = t["vt"][t["vt_ptr"][v]:t["vt_ptr"][v + 1]]
        expect = np.nonzero((a["tris"] == v).any(1))[0]
        assert np.array_equal(lst, expect)
    c = pdg.Constraints(m).build_stretch(1e3).build_bend(2e-2)
    ca = c.arrays()
    hinge, w, nr_, hk = oracle.build_bend(a["rest"], a["tris"], e, 2e-2)
    assert np.array_equal(ca["quads"], hinge)
    assert np.array_equal(ca["w"], w) and np.array_equal(ca["n_rest"], nr_) and np.array_equal(ca["bend_k"], hk)
    for dt in (1 / 60, 0.01):
        d = c.jacobi_diag(dt)
        d2 = oracle.jacobi_diag(m.N, a["tris"], a["Dm_inv"], a["area"], ca["k_stretch"], hinge, w, hk, a["mass"],
                                np.float32(dt))
        assert np.array_equal(d, d2)


def test_tri_tri_adjacency(pdg):
    m = pdg.Mesh.generate(4, 4, 1.0, 0)
    a = m.arrays(); t = m.topology()
    for tri in range(m.T):
        for k in range(3):
            nb = t["tri_tri"][tri, k]
            opp = a["tris"][tri, k]
            side = set(a["tris"][tri]) - {opp}
            if nb >= 0:
                assert side <= set(a["tris"][nb]) and nb != tri
            else:   # boundary side: no other triangle holds both vertices
                others = [u for u in range(m.T) if u != tri and side <= set(a["tris"][u])]
                assert others == []


def test_pin_presets(pdg):
    m = pdg.Mesh.generate(10, 10, 0.1, 0)
    c = pdg.Constraints(m).pin_top_row(10)
    ca = c.arrays()
    assert list(ca["pins"]) == list(range(10))
    assert np.array_equal(ca["targets"], m.arrays()["rest"][:10])
    c.pin_corners(10)
    assert list(c.arrays()["pins"]) == [0, 9]


def test_obj_loader(pdg, tmp_path):
    # ClothMesh::load_obj: 1-based indices, "i/t/n" tokens, fan triangulation
    p = tmp_path / "quad.obj"
    p.write_text("# quad\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nf 1/1 2/1 3/1 4/1\n")
    m = pdg.Mesh.load_obj(str(p))
    a = m.arrays()
    assert m.N == 4 and m.T == 2
    assert np.array_equal(a["tris"], [[0, 1, 2], [0, 2, 3]])
    assert np.isclose(a["area"].sum(), 1.0) and np.isclose(a["mass"].sum(), 0.1)


def test_obj_loader_errors(pdg, tmp_path):
    with pytest.raises(pdg.PDGError) as e:
        pdg.Mesh.load_obj(str(tmp_path / "missing.obj"))
    assert e.value.code == pdg.ERR_IO
    p = tmp_path / "bad.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2 9\n")
    with pytest.raises(pdg.PDGError):
        pdg.Mesh.load_obj(str(p))
    p2 = tmp_path / "empty.obj"
    p2.write_text("# nothing\n")
    with pytest.raises(pdg.PDGError):
        pdg.Mesh.load_obj(str(p2))


def test_argument_errors(pdg):
    with pytest.raises(pdg.PDGError):
        pdg.Mesh.generate(1, 5, 0.1, 0)       # nrows >= 2 (src/mesh_generator.cpp:9)
    with pytest.raises(pdg.PDGError):
        pdg.Mesh.generate(3, 3, 0.1, 4)
    with pytest.raises(pdg.PDGError):
        pdg.Mesh.create(np.zeros((3, 3)), np.array([[0, 1, 3]]))
    m = pdg.Mesh.generate(3, 3, 0.1, 0)
    c = pdg.Constraints(m)
    with pytest.raises(pdg.PDGError):
        c.set_pins([0, 99])
    with pytest.raises(pdg.PDGError):
        c.set_pins([1, 1])
    with pytest.raises(pdg.PDGError):
        c.build_stretch(float("nan"))
