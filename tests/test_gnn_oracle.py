"""The float64 network oracle checks itself against finite differences (CPU)."""
import numpy as np
import pytest


def grid_graph(n):
    """4-neighbour grid adjacency as a symmetric CSR, plus directed edge lists."""
    N = n * n
    nbr = [[] for _ in range(N)]
    for i in range(n):
        for j in range(n):
            v = i * n + j
            if j + 1 < n:
                nbr[v].append(v + 1); nbr[v + 1].append(v)
            if i + 1 < n:
                nbr[v].append(v + n); nbr[v + n].append(v)
    ptr = np.zeros(N + 1, np.int32)
    adj = []
    for v in range(N):
        s = sorted(nbr[v])
        adj += s
        ptr[v + 1] = len(adj)
    adj = np.array(adj, np.int32)
    dst = np.repeat(np.arange(N), np.diff(ptr))
    return ptr, adj, dst, adj.copy(), np.diff(ptr).astype(np.float64)


def random_problem(seed=0, n=5):
    import gnn_oracle as G
    rng = np.random.default_rng(seed)
    ptr, adj, dst, src, deg = grid_graph(n)
    N = n * n
    x = rng.normal(size=(N, G.NF))
    e = rng.normal(size=(len(adj), G.EF))
    target = rng.normal(size=(N, 3))
    free = (rng.random(N) > 0.1).astype(np.float64)
    p = {k: rng.normal(scale=0.3, size=s) for k, s in G.shapes()}
    return G, p, x, e, src, dst, deg, target, free, ptr, adj


@pytest.mark.parametrize("lam,weighted", [(0.0, False), (0.7, False), (0.7, True)])
def test_oracle_gradients_match_finite_differences(lam, weighted):
    G, p, x, e, src, dst, deg, target, free, _, _ = random_problem(0)
    # symmetric positive edge weights (the energy-norm term's form)
    ew = None
    if weighted:
        a = np.random.default_rng(5).uniform(0.5, 3.0, len(deg))
        ew = 0.5 * (a[src] + a[dst])
    loss, g, _ = G.loss_and_grad(p, x, e, src, dst, deg, target, free, lam, ew)
    flat = G.flatten(p)
    gflat = G.flatten(g)
    rng = np.random.default_rng(1)
    idx = rng.choice(len(flat), 60, replace=False)
    eps = 1e-6
    for k in idx:
        fp = flat.copy(); fp[k] += eps
        fm = flat.copy(); fm[k] -= eps
        lp = G.loss_and_grad(G.unflatten(fp), x, e, src, dst, deg, target, free, lam, ew)[0]
        lm = G.loss_and_grad(G.unflatten(fm), x, e, src, dst, deg, target, free, lam, ew)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - gflat[k]) <= 1e-6 + 1e-4 * abs(fd), (k, fd, gflat[k])


def test_oracle_adam_matches_formula():
    import gnn_oracle as G
    p = np.array([1.0, -2.0]); g = np.array([0.5, 0.25]); m = np.zeros(2); v = np.zeros(2)
    p1, m1, v1 = G.adam(p, g, m, v, 1, 1e-3)
    # first step of Adam moves each parameter by lr against its gradient sign
    assert np.allclose(p1, p - 1e-3 * np.sign(g), atol=1e-9)
