"""sim_cloth driver (the reference's command line, src/tools/sim_cloth.cpp) on the GPU."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "cloth-cuda_gb300", "bin", "sim_cloth")


def run(args):
    return subprocess.run([EXE] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=120)


def read_ply(path):
    lines = open(path).read().splitlines()
    nv = int(next(l for l in lines if l.startswith("element vertex")).split()[-1])
    start = lines.index("end_header") + 1
    return np.array([[float(t) for t in l.split()] for l in lines[start:start + nv]])


def test_sim_cloth_runs_and_exports(pdg, tmp_path):
    p = run(["20", "20", "0.05", "--steps", "20", "--iter", "30", "--pin", "top", "--stiffness", "100",
             "--bend", "0.1", "--type", "3", "--export", str(tmp_path), "--verbose"])
    assert p.returncode == 0, p.stderr
    assert "Simulation complete" in p.stdout and "Final energy" in p.stdout
    assert "Pinned vertices: 20" in p.stdout
    frames = sorted(f for f in os.listdir(tmp_path) if f.endswith(".ply"))
    assert "frame_0000.ply" in frames and "frame_final.ply" in frames and len(frames) >= 11
    x0 = read_ply(tmp_path / "frame_0000.ply")
    x1 = read_ply(tmp_path / "frame_final.ply")
    assert x0.shape == x1.shape == (20 * 20 + 19 * 19, 3)
    assert np.allclose(x1[:20], x0[:20], atol=1e-5)      # top row pinned
    assert x1[20:, 1].min() < -1e-3                      # the rest falls along -y


def test_sim_cloth_literal_mode_and_errors(pdg, tmp_path):
    p = run(["10", "10", "0.1", "--steps", "5", "--iter", "5", "--mode", "literal", "--pin", "corners"])
    assert p.returncode == 0, p.stderr
    p = run(["10", "10", "0.1", "--stretch-backend", "cpu-ref"])
    assert p.returncode == 2 and "not available" in p.stderr
    p = run(["1", "10", "0.1"])
    assert p.returncode == 3
