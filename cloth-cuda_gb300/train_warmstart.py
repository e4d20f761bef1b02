"""Train and evaluate the learned warm start on data the PD solver generates.

    python cloth-cuda_gb300/train_warmstart.py [--trajectories 2000] [--frames 64]
        [--batch 32] [--lr 1e-3] [--smoothness 0] [--energy-norm] [--eval-seeds 128]
        [--eval-frames 16] [--eval-cap 200] [--judge 0,4] [--out params.npy] [--json result.json]

The committed parameters (cloth-cuda_gb300/warmstart_params.npy) were made by

    python cloth-cuda_gb300/train_warmstart.py --trajectories 2000 --frames 64 --batch 32 \\
        --val-judge 4 --eval-seeds 128 --eval-frames 16 --eval-tols 3e-2,1e-2,1e-5 --judge 4 \\
        --out cloth-cuda_gb300/warmstart_params.npy --json train.json

(validation then judged after 4 sweeps; the selected checkpoint, the zero decoder, is also the
best one judged on the start residuals, the default now)

Training data: 2,000 trajectories of 64 frames of cloths drawn from the
batched-workload distribution (scenes.batch: grid side 17..129, 0.5-2 m,
1-4 boundary pins, stretch k 1e2..1e4, bend k 1e-3..1e-1, wind N(0, 2)),
`batch` cloths per solver and per Adam step; every frame of every trajectory
is one training batch: inputs (x_n, v_n, y, d_prev) of the trajectory, which
is solved as in use (cap --traj-cap sweeps, tolerance --traj-tol), target
x* - y - d_prev from a deep solve of the same frame from the same state (cap
--target-cap sweeps, relative residual --target-tol) so the target is close
to the converged positions (pdg_warmstart_train_pair).
Loss: MSE, plus --smoothness times the squared error differences over the
mesh edges (weighted by the PD system's stiffness with --energy-norm); Adam,
lr 1e-3.  The network starts with a zero decoder (it then predicts the
previous frame's offset); before training and every --select-every batches
it is validated by the mean sweeps its judged start needs to --val-tol on
--val-seeds validation cloths, and the checkpoint with the fewest sweeps is
kept (a lower offset error does not by itself mean fewer sweeps).
Evaluation on --eval-seeds held-out cloths (seeds disjoint from training and
validation): the same frames are solved from the inertial start and from the
judged learned start (judge after K sweeps for each K of --judge) to each
relative residual of --eval-tols with cap --eval-cap (200); the script reports sweeps,
convergence, the fraction of cloth-frames where the learned start was kept,
and the sweeps saved on the frames both starts solve.
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

PARAMS = os.path.join(HERE, "warmstart_params.npy")
TRAIN_SEED0 = 1000          # training batches: seeds 1000, 1001, ...
VAL_SEED0 = 700000          # validation batches (checkpoint selection)
EVAL_SEED0 = 900000         # held-out evaluation batches


def load_params(path=PARAMS):
    """The committed network parameters (float32, pdg_warmstart layout)."""
    return np.load(path).astype(np.float32)


def _pair(args, seed):
    """The trajectory solver (solved as in use: cap --traj-cap, tolerance
    --traj-tol) and the deep solver of the targets, over the same cloths."""
    out = []
    for cap, tol in ((args.traj_cap, args.traj_tol), (args.target_cap, args.target_tol)):
        ms, cs, cfgs, _ = scenes.batch(args.batch, seed=seed, max_iterations=cap, tolerance=tol,
                                       kernel=pdg.KERNEL_STREAM, patch_verts=128, block_threads=128,
                                       n_range=args.n_range)
        out.append(pdg.Solver(cfgs, ms, cs))
    return out


def validate(params, args):
    """Mean sweeps to --val-tol (cap 200) of the judged learned start with
    `params` on the validation cloths (seeds disjoint from training and
    evaluation); the checkpoint selection's measure."""
    rows = []
    for b in range(max(1, args.val_seeds // args.batch)):
        r, _, _ = solve_frames(params, dict(max_iterations=200, tolerance=args.val_tol, kernel=pdg.KERNEL_STREAM,
                                            patch_verts=128, block_threads=128, init=pdg.INIT_WARMSTART),
                               VAL_SEED0 + b, args.batch, args.val_frames, args.n_range, judge=args.val_judge)
        rows += r
    return float(np.mean([x["iterations"] for x in rows]))


def train(args, log=print):
    """Adam on the training trajectories; every --select-every batches (and
    before the first) the network is validated by sweeps and the best
    checkpoint is kept.  Returns (best parameters, losses, validation log)."""
    w = pdg.WarmStart(seed=args.seed).set_smoothness(args.smoothness).set_energy_norm(args.energy_norm)
    nbatches = max(1, args.trajectories // args.batch)
    losses, val = [], []
    best = None
    t0 = time.time()

    def checkpoint(b):
        nonlocal best
        if not args.select_every:
            return
        p = w.get_params()
        sw = validate(p, args)
        val.append(dict(batch=b, sweeps=sw))
        log("checkpoint after %d batches: validation sweeps %.2f" % (b, sw))
        if best is None or sw < best[1]:
            best = (p, sw, b)

    checkpoint(0)
    for b in range(nbatches):
        traj, deep = _pair(args, TRAIN_SEED0 + b)
        w.attach(traj)
        bl = [w.train_pair(traj, deep, args.lr) for _ in range(args.frames)]
        losses.append(float(np.mean(bl)))
        if b % 8 == 0 or b == nbatches - 1:
            log("batch %d/%d  mean loss %.4f  (%.1f s)" % (b + 1, nbatches, losses[-1], time.time() - t0))
        traj.close(); deep.close()
        w.solver = None
        if args.select_every and ((b + 1) % args.select_every == 0 or b == nbatches - 1):
            checkpoint(b + 1)
    if best is None:
        return w.get_params(), losses, val, nbatches
    return best[0], losses, val, best[2]


def score(params, args, seeds=2, frames=32, base_seed=500000):
    """Mean squared error (lr = 0, no smoothness term) of the prediction of
    `params` on held-out trajectories: the target is the change of the
    converged offset since the previous frame, so zero parameters score the
    previous frame's offset as the prediction."""
    out = []
    for b in range(seeds):
        traj, deep = _pair(args, base_seed + b)
        w = pdg.WarmStart(seed=0)
        w.set_params(params)
        w.attach(traj)
        out += [w.train_pair(traj, deep, 0.0) for _ in range(frames)]
        traj.close(); deep.close(); w.close()
    return float(np.mean(out))


def solve_frames(params, cfg_kw, seed, count, frames, n_range, judge=1):
    """Per-cloth frame stats of `frames` frames of one held-out batch, and
    the host time of the frames (each step call synchronises)."""
    ms, cs, cfgs, _ = scenes.batch(count, seed=seed, n_range=n_range, **cfg_kw)
    s = pdg.Solver(cfgs, ms, cs)
    w = None
    if params is not None:
        w = pdg.WarmStart(seed=0)
        w.set_params(params)
        w.set_judge_sweeps(judge)
        w.attach(s)
    st_all, t = [], 0.0
    for f in range(frames):
        t0 = time.perf_counter()
        st = s.step(1)
        t += time.perf_counter() - t0
        st_all += [dict(frame=f, **x) for x in st]
    N = sum(m.N for m in ms)
    s.close()
    if w is not None:
        w.close()
    return st_all, N * frames, t


def summarize(rows):
    return dict(iterations_mean=float(np.mean([x["iterations"] for x in rows])),
                converged_fraction=float(np.mean([x["converged"] for x in rows])),
                rel_residual_median=float(np.median([x["rel_residual"] for x in rows])),
                learned_start_kept=float(np.mean([x["warm_start_used"] for x in rows])))


def evaluate(params, args, log=print):
    """Inertial vs judged learned start on held-out cloths, per tolerance and
    judge sweep count."""
    nb = max(1, args.eval_seeds // args.batch)
    out = {}
    for tol in args.eval_tols:
        common = dict(max_iterations=args.eval_cap, tolerance=tol, kernel=pdg.KERNEL_STREAM, patch_verts=128,
                      block_threads=128)
        arms = {"inertial": dict(params=None, init=pdg.INIT_INERTIAL, judge=0)}
        for K in args.judge:
            arms["learned_judge%d" % K] = dict(params=params, init=pdg.INIT_WARMSTART, judge=K)
        res = {}
        for name, arm in arms.items():
            rows, vs, t = [], 0, 0.0
            for b in range(nb):
                r, v_, t_ = solve_frames(arm["params"], dict(common, init=arm["init"]), EVAL_SEED0 + b, args.batch,
                                         args.eval_frames, args.n_range, judge=arm["judge"])
                rows += r; vs += v_; t += t_
            res[name] = rows
            out.setdefault("tol_%g" % tol, {})[name] = dict(summarize(rows), vertex_steps_per_s_host_timed=vs / t)
            log("tol %g %s %s" % (tol, name, json.dumps(out["tol_%g" % tol][name])))
        for name in res:
            if name == "inertial":
                continue
            both = [(a["iterations"], b["iterations"]) for a, b in zip(res["inertial"], res[name])
                    if a["converged"] and b["converged"]]
            out["tol_%g" % tol][name]["sweeps_saved_on_frames_both_converge"] = (
                float(1 - sum(b for _, b in both) / max(sum(a for a, _ in both), 1)) if both else None)
            out["tol_%g" % tol][name]["frames_both_converge"] = len(both)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--trajectories", type=int, default=2000)
    ap.add_argument("--frames", type=int, default=64)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--smoothness", type=float, default=0.0,
                    help="weight of the neighbour-difference term of the training loss")
    ap.add_argument("--energy-norm", action="store_true",
                    help="weigh that term by the PD system's stiffness (energy norm of the error)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--target-cap", type=int, default=1000)
    ap.add_argument("--target-tol", type=float, default=1e-7)
    ap.add_argument("--traj-cap", type=int, default=200, help="sweep cap of the training trajectories' frames")
    ap.add_argument("--traj-tol", type=float, default=1e-5, help="tolerance of the training trajectories' frames")
    ap.add_argument("--eval-seeds", type=int, default=128)
    ap.add_argument("--eval-frames", type=int, default=16)
    ap.add_argument("--eval-tols", default="1e-2,1e-5", help="relative residuals the evaluation solves to")
    ap.add_argument("--eval-cap", type=int, default=200, help="sweep cap of the evaluation's frames")
    ap.add_argument("--judge", default="0,4", help="judge sweep counts to evaluate")
    ap.add_argument("--n-min", type=int, default=17)
    ap.add_argument("--n-max", type=int, default=129)
    ap.add_argument("--params", default="", help="evaluate these parameters instead of training")
    ap.add_argument("--select-every", type=int, default=8,
                    help="validate every this many batches and keep the checkpoint with the fewest sweeps (0: keep the last)")
    ap.add_argument("--val-seeds", type=int, default=64)
    ap.add_argument("--val-frames", type=int, default=8)
    ap.add_argument("--val-tol", type=float, default=1e-2)
    ap.add_argument("--val-judge", type=int, default=1)
    ap.add_argument("--out", default="")
    ap.add_argument("--json", default="")
    args = ap.parse_args()
    args.n_range = (args.n_min, args.n_max)
    args.eval_tols = [float(x) for x in args.eval_tols.split(",") if x]
    args.judge = [int(x) for x in args.judge.split(",") if x]
    t0 = time.time()
    losses, val, chosen = [], [], None
    if args.params:
        params = np.load(args.params).astype(np.float32)
    else:
        params, losses, val, chosen = train(args)
        if args.out:
            np.save(args.out, params)
    t_train = time.time() - t0
    held_out = score(params, args, frames=args.frames)
    zero = score(np.zeros_like(params), args, frames=args.frames)
    print("held-out loss: trained %.4f, zero parameters (previous offset) %.4f" % (held_out, zero))
    ev = evaluate(params, args)
    result = dict(args={k: v for k, v in vars(args).items() if k != "n_range"}, train_seconds=t_train,
                  train_loss=losses, validation=val, chosen_checkpoint_batches=chosen, held_out_loss=held_out,
                  zero_params_loss=zero, eval=ev)
    print(json.dumps(result))
    if args.json:
        json.dump(result, open(args.json, "w"), indent=1)


if __name__ == "__main__":
    main()
