"""Train and evaluate the learned warm start on data the PD solver generates.

    python cloth-cuda_gb300/train_warmstart.py [--trajectories 256] [--frames 64]
        [--batch 32] [--lr 1e-3] [--smoothness 0] [--eval-seeds 128] [--out params.npy] [--json result.json]

Training data: trajectories of cloths drawn from the batched-workload
distribution (scenes.batch), `batch` cloths per solver; every frame of every
trajectory is one training batch: inputs (x_n, v_n, y), target the solver's
frame result x_{n+1} - y, computed with a deep solve (cap 400 sweeps, relative
residual 1e-6) so the target is close to the converged positions.  Loss: MSE
plus --smoothness times the squared error differences over the mesh edges;
Adam.  Evaluation on `eval_seeds` held-out cloths: for each, the same frames
are solved from the inertial start, from the learned start kept only where
its residual is lower, and from the learned start always kept, to relative
residual --eval-tol (1e-5) with cap 200; the script reports the
start-residual ratio, iterations, convergence and the vertex-steps/s of
each, and the sweeps saved on the frames both starts solve.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import pdg  # noqa: E402
import scenes  # noqa: E402


def train(args, log=print):
    w = pdg.WarmStart(seed=args.seed).set_smoothness(args.smoothness)
    nbatches = max(1, args.trajectories // args.batch)
    losses = []
    t0 = time.time()
    for b in range(nbatches):
        ms, cs, cfgs, _ = scenes.batch(args.batch, seed=1000 + b, max_iterations=args.target_cap,
                                       tolerance=args.target_tol, kernel=pdg.KERNEL_GRAPH, n_range=args.n_range)
        s = pdg.Solver(cfgs, ms, cs)
        w.attach(s)
        bl = [w.train_frame(s, args.lr) for _ in range(args.frames)]
        losses.append(float(np.mean(bl)))
        log("batch %d/%d  mean loss %.4f  (%.1f s)" % (b + 1, nbatches, losses[-1], time.time() - t0))
        s.close()
        w.solver = None
    return w, losses


def score(params, args, seeds=2, frames=32, base_seed=500000):
    """Mean squared offset error (lr = 0, no smoothness term) of `params` on
    held-out trajectories."""
    out = []
    for b in range(seeds):
        ms, cs, cfgs, _ = scenes.batch(args.batch, seed=base_seed + b, max_iterations=args.target_cap,
                                       tolerance=args.target_tol, kernel=pdg.KERNEL_GRAPH, n_range=args.n_range)
        s = pdg.Solver(cfgs, ms, cs)
        w = pdg.WarmStart(seed=0)
        w.set_params(params)
        w.attach(s)
        out += [w.train_frame(s, 0.0) for _ in range(frames)]
        s.close(); w.close()
    return float(np.mean(out))


def evaluate(params, args, log=print):
    res = {"inertial": [], "learned": [], "learned_kept": []}
    times = {"inertial": 0.0, "learned": 0.0, "learned_kept": 0.0}
    verts = {"inertial": 0, "learned": 0, "learned_kept": 0}
    nb = max(1, args.eval_seeds // args.batch)
    for b in range(nb):
        for mode in ("inertial", "learned", "learned_kept"):
            init = {"inertial": pdg.INIT_INERTIAL, "learned": pdg.INIT_WARMSTART,
                    "learned_kept": pdg.INIT_WARMSTART_KEEP}[mode]
            ms, cs, cfgs, _ = scenes.batch(args.batch, seed=900000 + b, max_iterations=200,
                                           tolerance=args.eval_tol, kernel=pdg.KERNEL_GRAPH, init=init,
                                           n_range=args.n_range)
            s = pdg.Solver(cfgs, ms, cs)
            w = None
            if mode != "inertial":
                w = pdg.WarmStart(seed=0)
                w.set_params(params)
                w.attach(s)
            N = sum(m.N for m in ms)
            for f in range(args.eval_frames):
                t0 = time.perf_counter()
                st = s.step(1)
                times[mode] += time.perf_counter() - t0
                verts[mode] += N
                res[mode] += [dict(frame=f, **x) for x in st]
            s.close()
            if w is not None:
                w.close()
    out = {}
    for mode in res:
        r = res[mode]
        out[mode] = dict(
            iterations_mean=float(np.mean([x["iterations"] for x in r])),
            converged_fraction=float(np.mean([x["converged"] for x in r])),
            start_ratio_mean=float(np.mean([x["res_initial"] / max(x["res_inertial"], 1e-30) for x in r])),
            rel_residual_median=float(np.median([x["rel_residual"] for x in r])),
            learned_start_kept=float(np.mean([x["warm_start_used"] for x in r])),
            vertex_steps_per_s_host_timed=verts[mode] / max(times[mode], 1e-9))
        log(mode, json.dumps(out[mode]))
    # sweeps to the tolerance on the frames both starts reach it
    for mode in ("learned", "learned_kept"):
        both = [(xi["iterations"], xl["iterations"]) for xi, xl in zip(res["inertial"], res[mode])
                if xi["converged"] and xl["converged"]]
        out["%s_iterations_saved_on_frames_both_converge" % mode] = (
            float(1 - np.sum([b for _, b in both]) / max(np.sum([a for a, _ in both]), 1)) if both else None)
        out["%s_frames_both_converge" % mode] = len(both)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--trajectories", type=int, default=256)
    ap.add_argument("--frames", type=int, default=64)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--smoothness", type=float, default=0.0,
                    help="weight of the neighbour-difference term of the training loss")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--target-cap", type=int, default=400)
    ap.add_argument("--target-tol", type=float, default=1e-6)
    ap.add_argument("--eval-seeds", type=int, default=128)
    ap.add_argument("--eval-frames", type=int, default=16)
    ap.add_argument("--eval-tol", type=float, default=1e-5, help="relative residual the evaluation solves to")
    ap.add_argument("--n-min", type=int, default=17)
    ap.add_argument("--n-max", type=int, default=129)
    ap.add_argument("--out", default="")
    ap.add_argument("--json", default="")
    args = ap.parse_args()
    args.n_range = (args.n_min, args.n_max)
    w, losses = train(args)
    params = w.get_params()
    if args.out:
        np.save(args.out, params)
    held_out = score(params, args, frames=args.frames)
    zero = score(np.zeros_like(params), args, frames=args.frames)
    print("held-out loss: trained %.4f, zero predictor (inertial start) %.4f" % (held_out, zero))
    ev = evaluate(params, args)
    result = dict(args={k: v for k, v in vars(args).items() if k != "n_range"}, train_loss=losses,
                  held_out_loss=held_out, zero_predictor_loss=zero, eval=ev)
    print(json.dumps(result))
    if args.json:
        json.dump(result, open(args.json, "w"), indent=1)


if __name__ == "__main__":
    main()
