"""Record golden vectors of the reference's own CUDA step (run on a GPU machine).

    python tests/golden/make_ref_golden.py [out_dir] [--missing]

With --missing only the cases whose fixture is not in tests/golden yet are
recorded.

For each case the reference kernels of src/pd_solver.cu (compiled for sm_103a
into oracle/_ref/pd_solver_ref.cubin, launched by oracle/ref_harness.c in the
order of PDSolver::step) advance one frame; the case's parameters, start
state and the reference's output are written to tests/golden/ref_<case>.npz.
The mesh and its setup are regenerated from the parameters by the oracle, so
a fixture is small.  tests/test_golden.py checks the oracle's literal step
(CPU) and the library's literal mode (GPU) against these files.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle")]

import oracle as O  # noqa: E402
import ref_kernels  # noqa: E402

# name: (mesh, params, sweeps, perturbation)
CASES = {
    # 17x17 hanging cloth of the benchmark family (x-y plane, corners pinned)
    "hang17_rest_s1": (("hang", 17, 1.0), dict(ks=1e3, kb=1e-2, h=1 / 60, g=-9.81, damping=0.0), 1, 0.0),
    "hang17_pert_s1": (("hang", 17, 1.0), dict(ks=1e3, kb=1e-2, h=1 / 60, g=-9.81, damping=0.0), 1, 0.01),
    "hang17_rest_s10": (("hang", 17, 1.0), dict(ks=1e3, kb=1e-2, h=1 / 60, g=-9.81, damping=0.0), 10, 0.0),
    # the reference's own test scene (src/tests/test_pd_constraints.cpp:152-187):
    # 10x10 type-3 grid, cell 0.1, stretch 100, bend 1, corners pinned, dt 0.01
    "grid10t3_s1": (("grid", 10, 0.1, 3), dict(ks=100.0, kb=1.0, h=0.01, g=-9.8, damping=0.0), 1, 0.0),
    "grid10t3_pert_s1": (("grid", 10, 0.1, 3), dict(ks=100.0, kb=1.0, h=0.01, g=-9.8, damping=0.2), 1, 0.005),
    # the 33x33 hanging cloth of the small benchmark workload (1,089 vertices)
    "hang33_rest_s1": (("hang", 33, 1.0), dict(ks=1e3, kb=1e-2, h=1 / 60, g=-9.81, damping=0.0), 1, 0.0),
    "hang33_pert_s1": (("hang", 33, 1.0), dict(ks=1e3, kb=1e-2, h=1 / 60, g=-9.81, damping=0.0), 1, 0.01),
}


def make_scene(mesh, p):
    if mesh[0] == "hang":
        pos, tris, pins = O.hanging_cloth(mesh[1], mesh[2], seed=0)
    else:
        n, size, mtype = mesh[1], mesh[2], mesh[3]
        pos, tris = O.generate_grid(n, n, size, mtype)
        pins = np.array([0, n - 1], np.int32)
    sc = O.Scene(pos, tris, k_stretch=p["ks"], k_bend=p["kb"], pins=pins, h=p["h"], gravity=p["g"],
                 damping=p["damping"])
    return sc, pos


def start_state(sc, pos, pert, seed=1):
    rng = np.random.default_rng(seed)
    x = pos.astype(np.float32).copy()
    v = np.zeros_like(x)
    if pert > 0:
        cell = float(np.linalg.norm(pos[sc.tris[0, 1]] - pos[sc.tris[0, 0]]))
        x += (pert * cell * rng.standard_normal(x.shape)).astype(np.float32)
        v += (0.05 * rng.standard_normal(x.shape)).astype(np.float32)
        x[sc.pins] = sc.pin_targets
        v[sc.pins] = 0.0
    return x, v


def main(out_dir=HERE, missing_only=False):
    if not ref_kernels.available():
        raise SystemExit("reference kernels unavailable (oracle/_ref/pd_solver_ref.cubin or the harness missing)")
    os.makedirs(out_dir, exist_ok=True)
    for name, (mesh, p, sweeps, pert) in CASES.items():
        if missing_only and os.path.exists(os.path.join(HERE, "ref_%s.npz" % name)):
            continue
        sc, pos = make_scene(mesh, p)
        x0, v0 = start_state(sc, pos, pert)
        x1, v1 = ref_kernels.ref_step(sc, x0, v0, sweeps)
        meta = json.dumps({"mesh": list(mesh), "params": p, "sweeps": sweeps, "pert": pert})
        np.savez_compressed(os.path.join(out_dir, "ref_%s.npz" % name), x0=x0, v0=v0, x1=x1, v1=v1,
                            meta=np.array(meta))
        print(name, "N=%d" % sc.N, "max|v1|=%.3g" % np.abs(v1).max())


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    main(args[0] if args else HERE, missing_only="--missing" in sys.argv)
