"""The C-ABI library loads and exports every symbol include/pdg.h declares
(CPU only: no compute calls)."""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exports_every_declared_symbol(pdg):
    names = pdg.exported_symbols()
    assert len(names) > 30
    L = pdg.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert missing == []


def test_dynamic_symbol_table(pdg):
    out = subprocess.run(["nm", "-D", "--defined-only", pdg.LIB_PATH], stdout=subprocess.PIPE, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for n in pdg.exported_symbols():
        assert n in exported, n


def test_version_and_defaults(pdg):
    assert b"sm_103a" in pdg.lib().pdg_version()
    c = pdg.Config.default()
    # PDSolverConfig defaults (include/pd_solver.h:4-15)
    assert c.max_iterations == 50 and c.use_chebyshev == 1
    assert abs(c.rho - 0.9) < 1e-7 and abs(c.gravity + 9.8) < 1e-6 and abs(c.dt - 0.01) < 1e-9
    assert c.damping == 0.0 and c.mode == pdg.MODE_CONSISTENT


def test_last_error_is_set(pdg):
    L = pdg.lib()
    rc = L.pdg_config_default(None)
    assert rc == pdg.ERR_ARG
    assert b"null" in L.pdg_last_error_string()


def test_no_product_import_of_oracle():
    # the product path must not route through the oracle
    for root, _, files in os.walk(os.path.join(ROOT, "cloth-cuda_gb300")):
        for f in files:
            if f.endswith((".py", ".cpp", ".cu", ".h", ".cuh")):
                txt = open(os.path.join(root, f), errors="ignore").read()
                assert "oracle" not in txt.lower() or f == "build.py", f


def test_cli_driver_built(pdg):
    exe = os.path.join(ROOT, "cloth-cuda_gb300", "bin", "sim_cloth")
    if not os.path.exists(exe):
        pytest.skip("sim_cloth not built")
    p = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert p.returncode == 1 and "Usage" in p.stderr
