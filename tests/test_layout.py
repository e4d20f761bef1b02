"""Patch layout built on the host (no GPU): the properties the sweep kernels
rely on, checked by pdg_layout_check over meshes, batches and patch sizes.

- Reorder and partition: every vertex once, patches inside their cloth.
- Halo and neighbour lists: every owner of a halo vertex is a neighbour, so
  the resident kernel waits for it.
- Boundary vertices first: every owned vertex another patch reads is among
  the first nbnd, which the resident kernel publishes before its interior.
- Contribution slots: each slot of an owned vertex is written exactly once,
  by the phase-A records when the vertex is a boundary one.  This is what
  makes the gather deterministic and race-free.
- Every triangle through an owned vertex is held by the patch.
"""
import numpy as np
import pytest


def cloth(pdg, n, mtype=1, ks=1e3, kb=1e-2, pins="corners", seed=0, ncols=None):
    m = pdg.Mesh.hanging(n, 1.0, mtype=mtype, jitter=1e-4, seed=seed, ncols=ncols)
    c = pdg.Constraints(m).build_stretch(ks)
    if kb > 0:
        c.build_bend(kb)
    if pins == "corners":
        c.pin_corners(ncols or n)
    return m, c


@pytest.mark.parametrize("mtype", [0, 1, 2, 3])
@pytest.mark.parametrize("pv", [16, 32, 128, 448])
def test_layout_of_one_cloth(pdg, mtype, pv):
    m, c = cloth(pdg, 33, mtype=mtype)
    info = pdg.layout_check(pdg.Config.default(), m, c, pv)
    assert info["vertices"] == m.N
    assert info["patches"] == -(-m.N // pv)
    assert info["max_owned"] == min(pv, m.N)
    assert 0 < info["boundary_total"] <= m.N and info["halo_total"] > 0
    assert 0 < info["phase_a_cells"] <= info["cells"]


def test_grid_quads_pair_into_cells(pdg):
    # the two triangles of every grid quad share its diagonal, the longest
    # edge: (n-1)^2 cells, and the hinges of the diagonals are the cells' h0
    n = 17
    m, c = cloth(pdg, n, mtype=1)
    info = pdg.layout_check(pdg.Config.default(), m, c, 64)
    assert m.T == 2 * (n - 1) ** 2
    assert info["cells"] >= (n - 1) ** 2   # a cell held by several patches counts once per patch


def test_single_patch_has_no_halo(pdg):
    m, c = cloth(pdg, 9)
    info = pdg.layout_check(pdg.Config.default(), m, c, 128)
    assert info["patches"] == 1 and info["halo_total"] == 0 and info["boundary_total"] == 0
    assert info["phase_a_cells"] == 0


def test_batch_of_uneven_cloths(pdg):
    # cloths of different sizes, shapes, stiffnesses and pins in one layout:
    # no patch spans two cloths and no halo reaches into another cloth
    specs = [(9, 0, 1e3, 1e-2, "corners"), (33, 1, 5e2, 0.0, "none"), (17, 3, 1e3, 1e-1, "corners"),
             (24, 2, 2e3, 1e-2, "corners")]
    ms, cs = [], []
    for i, (n, mt, ks, kb, pins) in enumerate(specs):
        m, c = cloth(pdg, n, mtype=mt, ks=ks, kb=kb, pins=pins, seed=i)
        ms.append(m); cs.append(c)
    for pv in (16, 64, 480):
        info = pdg.layout_check(pdg.Config.default(), ms, cs, pv)
        assert info["vertices"] == sum(m.N for m in ms)
        assert info["patches"] == sum(-(-m.N // pv) for m in ms)


def test_rectangular_cloth(pdg):
    m, c = cloth(pdg, 20, ncols=45)
    for pv in (32, 100, 256):
        info = pdg.layout_check(pdg.Config.default(), m, c, pv)
        assert info["vertices"] == 20 * 45


def test_irregular_mesh(pdg):
    # a jittered triangulated disc with fan-like valences (not a grid)
    rng = np.random.default_rng(4)
    rings, per = 9, 12
    pos = [[0.0, 0.0, 0.0]]
    for r in range(1, rings + 1):
        k = per * r
        for j in range(k):
            a = 2 * np.pi * (j + 0.5 * (r % 2)) / k
            pos.append([r * np.cos(a) + rng.normal(0, 0.05), r * np.sin(a) + rng.normal(0, 0.05), 0.0])
    pos = np.asarray(pos, np.float32) * 0.05
    Delaunay = pytest.importorskip("scipy.spatial").Delaunay
    tris = Delaunay(pos[:, :2]).simplices.astype(np.int32)
    # consistent counter-clockwise orientation
    e1 = pos[tris[:, 1], :2] - pos[tris[:, 0], :2]
    e2 = pos[tris[:, 2], :2] - pos[tris[:, 0], :2]
    flip = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0] < 0
    tris[flip] = tris[flip][:, [0, 2, 1]]
    m = pdg.Mesh.create(pos, tris)
    c = pdg.Constraints(m).build_stretch(1e3)
    c.build_bend(1e-2)
    c.set_pins([0])
    for pv in (16, 48, 128):
        info = pdg.layout_check(pdg.Config.default(), m, c, pv)
        assert info["vertices"] == len(pos)
        assert info["lone_hinges"] >= 0


def test_headline_layout(pdg):
    # the 257x257 cloth at the resident kernel's 448-vertex patches: one patch
    # per SM of a GB300 (148 of 152) and shared memory within the opt-in limit
    m, c = cloth(pdg, 257)
    info = pdg.layout_check(pdg.Config.default(), m, c, 448)
    assert info["patches"] == 148 and info["max_owned"] == 448
    assert info["smem_resident"] <= 216 * 1024


def test_bad_arguments(pdg):
    m, c = cloth(pdg, 9)
    with pytest.raises(pdg.PDGError) as e:
        pdg.layout_check(pdg.Config.default(), m, c, 8)
    assert e.value.code == pdg.ERR_ARG
    m2, c2 = cloth(pdg, 9, seed=1)
    with pytest.raises(pdg.PDGError) as e:
        pdg.layout_check(pdg.Config.default(), [m, m2], [c2, c], 32)   # constraints of another mesh
    assert e.value.code == pdg.ERR_ARG


# Each planted mistake and the checker's finding (pdg_layout_check_planted
# builds the layout, plants one mistake, then runs the same check).
PLANTED = {
    1: "cloth or caller index out of place",
    2: "is foreign, owned or repeated",
    3: "is read by another patch but not among the first",
    4: "written twice",
    5: "contributions written",
    6: "out of range",
}


@pytest.mark.parametrize("mistake", sorted(PLANTED))
@pytest.mark.parametrize("mtype", [1, 3])
def test_checker_catches_each_planted_mistake(pdg, mistake, mtype):
    m, c = cloth(pdg, 33, mtype=mtype)
    cfg = pdg.Config.default()
    pdg.layout_check(cfg, m, c, 128)   # the built layout itself passes
    with pytest.raises(pdg.PDGError) as e:
        pdg.layout_check_planted(cfg, m, c, 128, mistake)
    assert e.value.code == pdg.ERR_STATE, str(e.value)
    assert PLANTED[mistake] in str(e.value), str(e.value)


def test_planted_mistake_out_of_range_is_an_argument_error(pdg):
    m, c = cloth(pdg, 17)
    with pytest.raises(pdg.PDGError) as e:
        pdg.layout_check_planted(pdg.Config.default(), m, c, 128, 7)
    assert e.value.code == pdg.ERR_ARG
