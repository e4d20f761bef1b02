"""Synthetic workloads of the PD cloth solver (meshes, constraints, configs).

All scenes are generated from seeds through the C ABI; no dataset is involved.

  hanging(n, side, ...)   square cloth in the x-y plane, row 0 on top, two top
                          corners pinned, alternating diagonals, z jitter
                          N(0, 1e-4) -- the plain single-cloth workloads
  batch(count, seed)      many cloths of uneven size: grid side n ~ U{17..129},
                          size ~ U[0.5, 2] m, 1-4 random boundary pins, stretch
                          k log-uniform [1e2, 1e4], bend k log-uniform
                          [1e-3, 1e-1], constant wind N(0, 2 m/s^2) per axis
"""
from __future__ import annotations

import numpy as np

import pdg

H = 1.0 / 60.0
G = -9.81


def hanging(n, side, ks=1e3, kb=1e-2, seed=0, mtype=1, jitter=1e-4, pins="corners"):
    m = pdg.Mesh.hanging(n, side, mtype=mtype, jitter=jitter, seed=seed)
    c = pdg.Constraints(m).build_stretch(ks)
    if kb > 0:
        c.build_bend(kb)
    if pins == "corners":
        c.pin_corners(n)
    elif pins == "top":
        c.pin_top_row(n)
    return m, c


def boundary_vertices(n):
    """Indices of the boundary vertices of an n x n grid (generator order)."""
    idx = [j for j in range(n)] + [(n - 1) * n + j for j in range(n)]
    idx += [i * n for i in range(1, n - 1)] + [i * n + n - 1 for i in range(1, n - 1)]
    return np.array(sorted(set(idx)), np.int32)


def shard(sizes, rank, world):
    """Contiguous split of cloths (vertex counts `sizes`) over `world` ranks,
    balanced by vertices: rank r gets the cloths whose cumulative vertex
    count midpoint falls in [r/world, (r+1)/world) of the total.  Cloths are
    independent, so a sharded batch needs no exchange between ranks."""
    sizes = np.asarray(sizes, np.float64)
    total = sizes.sum()
    mid = (np.cumsum(sizes) - 0.5 * sizes) / max(total, 1.0)
    owner = np.minimum((mid * world).astype(int), world - 1)
    return [i for i in range(len(sizes)) if owner[i] == rank]


def batch_params(count, seed=0, *, n_range=(17, 129), size_range=(0.5, 2.0)):
    """Per-cloth parameters of `count` cloths drawn from the batched-workload
    distribution (numpy only; batch() builds the meshes from them)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        size = float(rng.uniform(*size_range))
        ks = float(10 ** rng.uniform(2, 4))
        kb = float(10 ** rng.uniform(-3, -1))
        wind = rng.normal(0.0, 2.0, 3).astype(np.float32)
        npins = int(rng.integers(1, 5))
        pins = rng.choice(boundary_vertices(n), size=npins, replace=False).astype(np.int32)
        mesh_seed = int(rng.integers(1 << 31))
        out.append(dict(n=n, size=size, ks=ks, kb=kb, wind=wind.tolist(), pins=pins.tolist(), mesh_seed=mesh_seed))
    return out


def batch(count, seed=0, *, max_iterations=200, tolerance=1e-5, rho=0.99, n_range=(17, 129),
          size_range=(0.5, 2.0), **cfg_kw):
    """(meshes, constraints, configs, params) of `count` cloths drawn from
    the batched-workload distribution."""
    meshes, cons, cfgs = [], [], []
    params = batch_params(count, seed, n_range=n_range, size_range=size_range)
    for p in params:
        n = p["n"]
        m = pdg.Mesh.hanging(n, p["size"], mtype=1, jitter=1e-4, seed=p["mesh_seed"])
        c = pdg.Constraints(m).build_stretch(p["ks"]).build_bend(p["kb"]).set_pins(np.array(p["pins"], np.int32))
        cfg = pdg.Config.default(max_iterations=max_iterations, tolerance=tolerance, rho=rho, dt=H, gravity=G,
                                 wind=tuple(float(w) for w in p["wind"]), **cfg_kw)
        meshes.append(m); cons.append(c); cfgs.append(cfg)
    return meshes, cons, cfgs, params
