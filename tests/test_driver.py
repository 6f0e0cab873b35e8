"""The C++ driver (cpp/topopt_driver.cpp over the grid::HierarchyGrid facade)."""
import json
import os
import subprocess

import numpy as np
import pytest

from topoptspline3d_gb300 import build, capi, workloads
from tests.helpers import setup_oracle


def _driver():
    capi.load()
    assert os.path.exists(build.DRIVER_PATH)
    return build.DRIVER_PATH


def test_driver_rejects_bad_arguments():
    r = subprocess.run([_driver(), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown argument" in r.stderr


@pytest.mark.gpu
def test_driver_matches_oracle_history(oracle_mod):
    r = subprocess.run([_driver(), "--case", "cantilever", "--nx", "16", "--ny", "8", "--nz", "8", "--lattice",
                        "7", "5", "5", "--iters", "4", "--mode", "pcg64"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    summary = json.loads(r.stdout.strip().splitlines()[-1])
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    co = []
    for _ in range(4):
        o.update_operators()
        o.pcg(2, 2, 1e-6, 300, 1)
        co.append(o.compliance())
        o.sensitivity(); o.filter(2.0); o.spline_adjoint(); o.oc_update(0.4)
    assert np.allclose(summary["compliance"], co, rtol=1e-6, atol=0), (summary["compliance"], co)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "vcycle"])
def test_driver_modes_run(mode):
    r = subprocess.run([_driver(), "--case", "mbb", "--nx", "32", "--ny", "16", "--nz", "16", "--lattice",
                        "11", "7", "7", "--iters", "3", "--mode", mode], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    c = json.loads(r.stdout.strip().splitlines()[-1])["compliance"]
    assert all(np.isfinite(c)) and c[-1] < c[0]


def test_driver_rejects_bad_optimizer():
    r = subprocess.run([_driver(), "--optimizer", "sqp"], capture_output=True, text=True)
    assert r.returncode == 2 and "--optimizer" in r.stderr


@pytest.mark.gpu
def test_driver_mma_matches_oracle_history(oracle_mod):
    """--optimizer mma (the reference's testOrdinarySplineTopoptMMA loop) against the
    oracle chain with the oracle MMA, 4 design iterations."""
    from oracle.oracle import OracleMMA
    r = subprocess.run([_driver(), "--case", "cantilever", "--nx", "16", "--ny", "8", "--nz", "8", "--lattice",
                        "7", "5", "5", "--iters", "4", "--mode", "pcg64", "--optimizer", "mma"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    summary = json.loads(r.stdout.strip().splitlines()[-1])
    assert summary["optimizer"] == "mma"
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    nc = o.num_coeffs()
    _, _, _, _, nge = o.gs_maps(0)
    o.put("sens", np.where(o.get("eactive") != 0, 1e3 / nge, 0.0))
    o.spline_adjoint()
    dv = o.get("csens")[None, :]
    om = OracleMMA(nc, 1, 1e-3, 1.0)
    co = []
    for _ in range(4):
        o.put("coeff", om.x)
        o.coeff_to_density()
        vol = o.volume(True)
        o.update_operators()
        o.pcg(2, 2, 1e-6, 300, 1)
        co.append(o.compliance())
        o.sensitivity(); o.filter(2.0); o.spline_adjoint()
        om.update(o.get("csens"), dv, [1e3 * (vol - 0.4)])
    assert np.allclose(summary["compliance"], co, rtol=1e-6, atol=0), (summary["compliance"], co)


def test_driver_projection_needs_mma():
    r = subprocess.run([_driver(), "--selfsupport"], capture_output=True, text=True)
    assert r.returncode == 2 and "--optimizer mma" in r.stderr


@pytest.mark.gpu
def test_driver_mma_with_projection_and_constraints():
    """--optimizer mma --heaviside 4 --selfsupport: the reference's README
    example path (projection, volume + self-support + drip constraints) runs,
    stays finite and is repeatable."""
    cmd = [_driver(), "--case", "cantilever", "--nx", "24", "--ny", "12", "--nz", "12", "--lattice", "9", "6", "6",
           "--iters", "6", "--mode", "pcg64", "--optimizer", "mma", "--heaviside", "4", "--selfsupport",
           "--surface-lattice", "24"]
    runs = [subprocess.run(cmd, capture_output=True, text=True, timeout=300) for _ in range(2)]
    for r in runs:
        assert r.returncode == 0, r.stderr
    s = [json.loads(r.stdout.strip().splitlines()[-1]) for r in runs]
    assert s[0]["compliance"] == s[1]["compliance"]
    assert all(np.isfinite(s[0]["compliance"]))
    lines = [ln for ln in runs[0].stdout.splitlines() if ln.startswith("-- iter")]
    assert len(lines) == 6 and all("ss = " in ln for ln in lines)
