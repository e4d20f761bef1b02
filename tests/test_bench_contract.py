"""The benchmark script's fixed parts, without a GPU: the algorithmic bytes
per fused sweep that the roofline divides by, the workload table and the
measured traffic it reads.

Per sweep (the reference solve's data, read and written once): x^k, x^(k-1),
x^(k+1), y as float4 and 1/diag per vertex; 3 indices, Dm_inv and wA per
triangle; 4 indices, 4 weights, n and k per bend hinge; and the vertex-to-
corner CSR (4 (N + 1) + 12 T).  The grid sizes are those of the hanging
cloths of the small, single-cloth and large workloads (alternating-diagonal
grids: N = n^2, T = 2 (n - 1)^2, inner edges E = 3 (n - 1)^2 - 2 (n - 1)),
the inner-edge counts that src/tests/test_topology.cpp:24-35 checks.
"""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def grid(n):
    return n * n, 2 * (n - 1) ** 2, 3 * (n - 1) ** 2 - 2 * (n - 1)


@pytest.mark.parametrize("n,expected", [(33, 288_844), (257, 18_366_540), (1025, 293_666_892)])
def test_algorithmic_bytes_per_sweep(n, expected):
    import bench
    N, T, E = grid(n)
    assert bench.algorithmic_bytes_per_sweep(N, T, E) == expected
    # about 265-280 bytes per vertex
    assert 260 < expected / N < 285


def test_grid_counts_match_the_workloads():
    assert grid(33) == (1089, 2048, 3008)
    assert grid(257) == (66049, 131072, 196096)
    assert grid(1025) == (1050625, 2097152, 3143680)


def test_workload_table_and_measured_traffic():
    import bench
    wl = bench.WORKLOADS
    assert set(bench.METRICS) == set(wl)
    b = wl["batch512"]
    assert (b["count"], b["iters"], b["tol"], b["reach"]) == (512, 200, 1e-5, 1e-2)
    assert b["plan"] == (256, 256) and b["learned"]
    assert (wl["large1025"]["iters"], wl["large1025"]["tol"]) == (200, 1e-6)
    assert (wl["plain257"]["iters"], wl["hang33"]["iters"]) == (32, 10)
    # the traffic the roofline reports comes from ncu captures of the bench's
    # own kernels: within 20 % of the algorithmic bytes of the same sweep
    tr = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    alg_1025 = 293_666_892
    assert 0.8 < tr["large1025"]["k_stream"] / alg_1025 < 1.2
    assert 0.8 < tr["batch512"]["k_stream"] / 902_000_344 < 1.2
