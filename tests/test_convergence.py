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


def test_residual_judge_after_4_sweeps_rejects_a_start_that_finishes_first(oracle):
    # Cloths of the batched distribution, each frame solved to relative
    # residual 1e-2 from the inertial start (as the benchmark's arms do).  On
    # every later frame two starts are compared: the inertial one and the
    # previous frame's offset.  Always taking the previous offset needs
    # fewer sweeps on average, but a judge that compares the two residuals
    # after 4 sweeps keeps it too rarely to get that gain: the previous
    # offset carries high-frequency error that dominates the early residual.
    import scenes

    def sweeps_to(info, tol, cap):
        k = np.nonzero(info["res"] / info["res_y"] <= tol)[0]
        return int(k[0]) if len(k) else cap

    tol, cap, K = 1e-2, 200, 4
    inertial, prev, judged = [], [], []
    for p in scenes.batch_params(3, seed=7, n_range=(17, 25)):
        pos, tris, _ = oracle.hanging_cloth(p["n"], p["size"], seed=p["mesh_seed"])
        sc = oracle.Scene(pos, tris, k_stretch=p["ks"], k_bend=p["kb"], pins=p["pins"], h=1 / 60, gravity=-9.81,
                          wind=tuple(p["wind"]))
        x = pos.astype(np.float64).reshape(-1); v = np.zeros_like(x); d1 = None
        for f in range(8):
            y = sc.predict(x, v)
            if d1 is not None:
                _, _, ii = sc.step_jacobi(x, v, cap, rho=0.99)
                _, _, ip = sc.step_jacobi(x, v, cap, rho=0.99, init=2, x0=y + d1)
                si, sp = sweeps_to(ii, tol, cap), sweeps_to(ip, tol, cap)
                inertial.append(si); prev.append(sp)
                judged.append(sp if ip["res"][K - 1] < ii["res"][K - 1] else si)
            xa, va, _ = sc.step_jacobi(x, v, cap, tol=tol, rho=0.99)
            d1 = xa - y
            x, v = xa, va
    mi, mp, mj = np.mean(inertial), np.mean(prev), np.mean(judged)
    assert mp < 0.9 * mi, (mp, mi)       # the previous offset finishes first
    assert mj > mp + 0.5 * (mi - mp), (mj, mp, mi)   # the judge keeps less than half of that gain


def test_always_keeping_the_previous_offset_is_unstable_in_closed_loop(oracle):
    # The same kind of cloth when every frame starts from the previous
    # frame's offset and the trajectory continues from that solve (stopped at
    # 1e-2).  A solve stopped at a tolerance leaves error in the direction of
    # its start: from the inertial start the offset comes out too small and
    # the cloth loses energy; from the previous offset it repeats the last
    # frame's internal force and the cloth gains energy.  Within 20 frames
    # the cloth (which the wind accelerates either way) runs to more than
    # twice the inertial trajectory's peak speed and its frames stop
    # converging, while the inertial start's trajectory stays converged.
    import scenes
    p = scenes.batch_params(3, seed=7, n_range=(17, 33))[2]
    pos, tris, _ = oracle.hanging_cloth(p["n"], p["size"], seed=p["mesh_seed"])
    sc = oracle.Scene(pos, tris, k_stretch=p["ks"], k_bend=p["kb"], pins=p["pins"], h=1 / 60, gravity=-9.81,
                      wind=tuple(p["wind"]))
    out = {}
    for mode in ("inertial", "previous"):
        x = pos.astype(np.float64).reshape(-1); v = np.zeros_like(x); d1 = None
        speeds, failed = [], 0
        for f in range(20):
            y = sc.predict(x, v)
            if mode == "previous" and d1 is not None:
                xa, va, info = sc.step_jacobi(x, v, 200, tol=1e-2, rho=0.99, init=2, x0=y + d1)
            else:
                xa, va, info = sc.step_jacobi(x, v, 200, tol=1e-2, rho=0.99)
            failed += int(info["res"][-1] > 1e-2 * info["res_y"])
            d1 = xa - y
            x, v = xa, va
            speeds.append(np.abs(v).max())
        out[mode] = (speeds, failed)
    si, fi = out["inertial"]
    sp, fp = out["previous"]
    assert fi == 0, fi
    assert fp >= 2 and max(sp) > 2 * max(si), (fp, max(sp), max(si))
