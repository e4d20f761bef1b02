"""Golden vectors recorded from the reference's own CUDA kernels.

tests/golden/ref_*.npz hold one frame of src/pd_solver.cu's kernels, run on
a GB300 by tests/golden/make_ref_golden.py.  The oracle's literal step must
reproduce them (CPU), and so must the library's reference-literal mode (GPU).
Single-sweep cases are held to 1e-5 relative; the literal iteration amplifies
rounding ~1e5x over 10 sweeps, so multi-sweep cases are held to the spread
the oracle itself shows under 1e-7 perturbations of its input.
"""
import glob
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))


def rel(a, b):
    a = np.asarray(a, np.float64).reshape(-1); b = np.asarray(b, np.float64).reshape(-1)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def load(oracle, path):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_ref_golden as mk
    d = np.load(path)
    meta = json.loads(str(d["meta"]))
    sc, pos = mk.make_scene(tuple(meta["mesh"]), meta["params"])
    return sc, pos, d, meta


def spread(sc, x0, v0, sweeps, seed=0):
    rng = np.random.default_rng(seed)
    xo, _ = sc.step_literal(x0.reshape(-1), v0.reshape(-1), sweeps)
    s = 0.0
    for _ in range(3):
        xp = (x0 * (1 + 1e-7 * rng.standard_normal(x0.shape))).astype(np.float32)
        xp[sc.pins] = x0[sc.pins]
        s = max(s, rel(sc.step_literal(xp.reshape(-1), v0.reshape(-1), sweeps)[0], xo))
    return s


def test_fixtures_present():
    assert len(FILES) >= 4, "golden fixtures missing: run tests/golden/make_ref_golden.py on a GPU box"


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[4:-4] for f in FILES])
def test_oracle_literal_reproduces_reference_kernels(oracle, path):
    sc, pos, d, meta = load(oracle, path)
    x1, v1 = sc.step_literal(d["x0"].reshape(-1), d["v0"].reshape(-1), int(meta["sweeps"]))
    if meta["sweeps"] == 1:
        assert rel(x1, d["x1"]) < 1e-5
        assert rel(v1, d["v1"]) < 1e-3
    else:
        bound = max(10 * spread(sc, d["x0"], d["v0"], int(meta["sweeps"])), 1e-5)
        assert rel(x1, d["x1"]) < bound


@pytest.mark.gpu
@pytest.mark.parametrize("path", [f for f in FILES if f.endswith("_s1.npz")], ids=lambda f: os.path.basename(f)[4:-4])
def test_library_literal_mode_reproduces_reference_kernels(pdg, oracle, path):
    sc, pos, d, meta = load(oracle, path)
    p = meta["params"]
    m = pdg.Mesh.create(pos, sc.tris)
    c = pdg.Constraints(m).build_stretch(p["ks"]).build_bend(p["kb"]).set_pins(sc.pins)
    cfg = pdg.Config.default(max_iterations=1, dt=p["h"], gravity=p["g"], damping=p["damping"],
                             mode=pdg.MODE_REFERENCE_LITERAL)
    s = pdg.Solver(cfg, m, c)
    s.set_state(d["x0"], d["v0"])
    s.step(1, stats=False)
    x, v = s.get_state()
    assert rel(x, d["x1"]) < 1e-5
    assert rel(v, d["v1"]) < 1e-3
