"""Reference precision (topo_set_reference_precision): the reference stores rho,
coefficients and sensitivities in FP32 and takes rho^p with powf
(grid/Grid.cu:1739).  With the switch on, those arrays hold FP32 values at the
points where the reference stores them, and a design run's distance from the
FP64 path is measured: it is the FP32 storage gap the FP64 oracle parity does
not show."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import setup_gpu, rel

pytestmark = pytest.mark.gpu


def _is_f32(a):
    a = np.asarray(a, dtype=np.float64)
    return np.array_equal(a, a.astype(np.float32).astype(np.float64))


def _case():
    return workloads.small_cases()["cantilever16"]


def test_arrays_hold_fp32_values():
    wl = _case()
    g = setup_gpu(wl)
    g.set_reference_precision(1)
    g.put("coeff", np.random.default_rng(4).uniform(0.05, 0.95, g.num_coeffs()))
    g.coeff_to_density()
    rho = g.get("rho")
    assert _is_f32(g.get("coeff")) and _is_f32(rho)
    ea = wl.eactive if wl.eactive is not None else np.ones(wl.nx * wl.ny * wl.nz, np.uint8)
    ref = np.where(ea != 0, np.power(rho.astype(np.float32), np.float32(3.0)), 0).astype(np.float64)
    g.update_operators()  # rho^p in FP32 by powf
    assert rel(g.get("rhop"), ref) < 1e-6
    g.solve(mode=capi.SOLVE_PCG64, rtol=1e-8, max_iter=300)
    g.sensitivity()
    assert _is_f32(g.get("sens"))
    g.filter(wl.filter_radius)
    assert _is_f32(g.get("sens"))
    g.spline_adjoint()
    assert _is_f32(g.get("csens"))
    g.close()


def test_design_run_gap_to_fp64():
    """Ten design iterations from the same start with and without reference
    precision: the compliance trajectories agree to the FP32 storage level."""
    wl = _case()
    runs = []
    for ref in (0, 1):
        g = setup_gpu(wl)
        g.set_reference_precision(ref)
        g.coeff_to_density()
        comp = []
        for _ in range(10):
            s = g.design_iteration(solve=dict(mode=capi.SOLVE_PCG64, rtol=1e-9, max_iter=300),
                                   oc=dict(vgoal=wl.vgoal), filter_radius=wl.filter_radius)
            comp.append(s["compliance"])
        runs.append((np.array(comp), g.get("coeff")))
        g.close()
    (c64, k64), (c32, k32) = runs
    gap = np.abs(c32 - c64) / np.abs(c64)
    print("compliance gap per iteration:", " ".join(f"{x:.1e}" for x in gap),
          f"coefficients {rel(k32, k64):.1e}")
    assert gap.max() < 1e-4 and gap.max() > 0
    assert rel(k32, k64) < 1e-3
