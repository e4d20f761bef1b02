"""How far Chebyshev-Jacobi is from the benchmark's 1e-5 target (CPU oracle).

The batched and large workloads ask for relative residual 1e-5 with a cap of
200 sweeps.  On a swinging 17x17 cloth (stretch k 1e3, bend k 1e-2, wind
(0.5, 0, 0.3), rho 0.99) the float64 iteration does reach 1e-5, so the
method converges to the PD fixed point, but only after well over a thousand
sweeps: it is the 200-sweep cap, not the method, that keeps the workloads
from 1e-5.
"""
import numpy as np


def swinging_cloth(oracle, n=17, frames=10):
    pos, tris, pins = oracle.hanging_cloth(n, 1.0, seed=0)
    sc = oracle.Scene(pos, tris, k_stretch=1e3, k_bend=1e-2, pins=pins, h=1 / 60, gravity=-9.81,
                      wind=(0.5, 0.0, 0.3))
    x = pos.astype(np.float64).reshape(-1); v = np.zeros_like(x)
    for _ in range(frames):   # a deep solve per frame: the cloth falls and swings
        x, v, _ = sc.step_jacobi(x, v, 3000, tol=1e-9, rho=0.99)
    return sc, x, v


def test_sweeps_to_1e5_on_a_small_cloth(oracle):
    sc, x, v = swinging_cloth(oracle)
    _, _, info = sc.step_jacobi(x, v, 8000, tol=1e-5, rho=0.99)
    used = info["used"]
    rel = info["res"][-1] / info["res_y"]
    # converged, after far more sweeps than the benchmark's cap of 200
    assert rel <= 1e-5 and used < 8000
    assert used > 5 * 200, used
    # and after 200 sweeps the same frame is still far above the target
    _, _, info200 = sc.step_jacobi(x, v, 200, tol=0.0, rho=0.99)
    assert info200["res"][-1] / info200["res_y"] > 1e-4
