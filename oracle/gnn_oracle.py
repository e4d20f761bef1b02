"""Float64 restatement of the warm-start network -- TEST INFRASTRUCTURE ONLY.

The network has no counterpart in the reference; the tests compare the
library's hand-written CUDA forward/backward/Adam kernels with this module.

Network (hidden H = 64), on the mesh graph (both directions of every edge):
    h0    = relu(We x + be)                          x: 14 node features
    for l = 1, 2:
      P, Q  = A_l h, B_l h
      m_ij  = relu(P_i + Q_j + C_l e_ij + c_l)         e_ij: 4 edge features
      a_i   = mean_{j in N(i)} m_ij
      h     = h + relu(U_l [h; a] + u_l)
    out   = Wd h + bd                                 3 outputs (offset change / scale)
Loss: mean over free vertices and the 3 components of (out - target)^2, plus
an optional weighted edge term (loss_and_grad).
Parameter shapes follow the library's layout (pdg_warmstart_get_params):
    We (64, 14), be (64), then per layer A (64, 64), B (64, 64), C (64, 4),
    c (64), U (64, 128), u (64), then Wd (3, 64), bd (3).
"""
from __future__ import annotations

import numpy as np

H = 64
NF = 14
EF = 4
NO = 3


def shapes():
    s = [("We", (H, NF)), ("be", (H,))]
    for l in range(2):
        s += [("A%d" % l, (H, H)), ("B%d" % l, (H, H)), ("C%d" % l, (H, EF)), ("c%d" % l, (H,)),
              ("U%d" % l, (H, 2 * H)), ("u%d" % l, (H,))]
    s += [("Wd", (NO, H)), ("bd", (NO,))]
    return s


def unflatten(flat):
    out, o = {}, 0
    for name, shp in shapes():
        n = int(np.prod(shp))
        out[name] = np.asarray(flat[o:o + n], np.float64).reshape(shp)
        o += n
    return out


def flatten(d):
    return np.concatenate([np.asarray(d[n], np.float64).reshape(-1) for n, _ in shapes()])


def count():
    return sum(int(np.prod(s)) for _, s in shapes())


def forward(p, x, e, src, dst, deg):
    """x (N, NF), e (Ed, EF) per directed edge dst <- src, deg (N,).
    Returns (out, cache)."""
    relu = lambda z: np.maximum(z, 0.0)
    z0 = x @ p["We"].T + p["be"]
    h = relu(z0)
    cache = dict(x=x, z0=z0, layers=[])
    for l in range(2):
        P = h @ p["A%d" % l].T
        Q = h @ p["B%d" % l].T
        zm = P[dst] + Q[src] + e @ p["C%d" % l].T + p["c%d" % l]
        m = relu(zm)
        a = np.zeros_like(h)
        np.add.at(a, dst, m)
        a /= np.maximum(deg, 1)[:, None]
        cat = np.concatenate([h, a], 1)
        zu = cat @ p["U%d" % l].T + p["u%d" % l]
        cache["layers"].append(dict(h=h, zm=zm, cat=cat, zu=zu))
        h = h + relu(zu)
    out = h @ p["Wd"].T + p["bd"]
    cache["h"] = h
    return out, cache


def loss_and_grad(p, x, e, src, dst, deg, target, free, lam=0.0, ew=None):
    """Loss = [sum_i |d_i|^2 + lam/2 sum_(a->b) k_ab w_a w_b |d_a - d_b|^2] / cnt
    with d = (out - target) * free over the directed edges (both directions
    of every mesh edge), edge weights k (ew, one per directed edge; None: 1),
    and its gradient with respect to every parameter."""
    out, c = forward(p, x, e, src, dst, deg)
    cnt = max(int(free.sum()) * NO, 1)
    diff = (out - target) * free[:, None]
    kab = np.ones(len(src)) if ew is None else np.asarray(ew, np.float64)
    wab = (free[src] * free[dst] * kab)[:, None]
    de = (diff[src] - diff[dst]) * wab
    loss = float(((diff ** 2).sum() + 0.5 * lam * ((diff[src] - diff[dst]) ** 2 * wab).sum()) / cnt)
    g = {n: np.zeros(s) for n, s in shapes()}
    gd = 2.0 * diff
    if lam:
        np.add.at(gd, src, lam * de)
        np.add.at(gd, dst, -lam * de)
    dout = gd * free[:, None] / cnt
    g["Wd"] = dout.T @ c["h"]
    g["bd"] = dout.sum(0)
    dh = dout @ p["Wd"]
    for l in (1, 0):
        L = c["layers"][l]
        dzu = dh * (L["zu"] > 0)
        g["U%d" % l] = dzu.T @ L["cat"]
        g["u%d" % l] = dzu.sum(0)
        dcat = dzu @ p["U%d" % l]
        dh_prev = dh + dcat[:, :H]
        da = dcat[:, H:] / np.maximum(deg, 1)[:, None]
        dm = da[dst] * (L["zm"] > 0)
        dP = np.zeros_like(dh); np.add.at(dP, dst, dm)
        dQ = np.zeros_like(dh); np.add.at(dQ, src, dm)
        g["C%d" % l] = dm.T @ e
        g["c%d" % l] = dm.sum(0)
        g["A%d" % l] = dP.T @ L["h"]
        g["B%d" % l] = dQ.T @ L["h"]
        dh = dh_prev + dP @ p["A%d" % l] + dQ @ p["B%d" % l]
    dz0 = dh * (c["z0"] > 0)
    g["We"] = dz0.T @ x
    g["be"] = dz0.sum(0)
    return loss, g, out


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) on flat float64 arrays; t counts from 1."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
