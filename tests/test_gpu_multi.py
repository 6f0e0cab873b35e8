"""Multi-right-hand-side solve (many load cases as right-hand sides of one
V-cycle) against the oracle's single-right-hand-side FP64 MG-PCG, per load."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import rel, random_coeff, setup_oracle

pytestmark = pytest.mark.gpu


def _problem(wl, coeff):
    p = capi.Problem(wl.nx, wl.ny, wl.nz)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", coeff)
    p.coeff_to_density()
    p.set_operator_precision(2)
    p.update_operators()
    return p


@pytest.mark.parametrize("nrhs", [1, 5])
def test_multi_rhs_matches_oracle(oracle_mod, nrhs):
    wl = workloads.cantilever(48, 24, 24)
    nc = int(np.prod([q + wl.order for q in wl.partition]))
    coeff = random_coeff(nc, seed=21)
    F = workloads.patch_loads(wl.nx, wl.ny, wl.nz, nrhs, seed0=1000, patch=8)
    p = _problem(wl, coeff)
    p.multi_reserve(8)
    U, st, rr = p.solve_multi(F, rtol=1e-9, max_iter=300)
    assert st["max_relres"] <= 1e-9 and (rr <= 1e-9).all()
    o = setup_oracle(wl, coeff)
    o.update_operators()
    for k in range(nrhs):
        o.put("f", F[k])
        o.put("u", np.zeros_like(F[k]))
        o.pcg(2, 2, 1e-11, 400, 1)
        uo = o.get("u")
        assert rel(U[k], uo) < 1e-6, k
        assert abs(F[k] @ U[k] - F[k] @ uo) <= 1e-8 * abs(F[k] @ uo)


@pytest.mark.parametrize("inner_max", [4, 6])
def test_multi_rhs_inner_cg_matches_oracle(oracle_mod, inner_max):
    """With a batched FP32 inner CG per outer step each load still matches the
    oracle, in fewer outer (FP64) iterations than one V-cycle per step."""
    wl = workloads.cantilever(48, 24, 24)
    nc = int(np.prod([q + wl.order for q in wl.partition]))
    coeff = random_coeff(nc, seed=23)
    F = workloads.patch_loads(wl.nx, wl.ny, wl.nz, 5, seed0=2000, patch=8)
    p = _problem(wl, coeff)
    p.multi_reserve(8)
    U1, st1, _ = p.solve_multi(F, rtol=1e-9, max_iter=300)
    U, st, rr = p.solve_multi(F, rtol=1e-9, max_iter=300, inner_max=inner_max, inner_rtol=0.05)
    assert st["max_relres"] <= 1e-9 and (rr <= 1e-9).all()
    assert st["iterations"] < st1["iterations"]
    o = setup_oracle(wl, coeff)
    o.update_operators()
    for k in range(5):
        o.put("f", F[k])
        o.put("u", np.zeros_like(F[k]))
        o.pcg(2, 2, 1e-11, 400, 1)
        uo = o.get("u")
        assert rel(U[k], uo) < 1e-6, k
        assert abs(F[k] @ U[k] - F[k] @ uo) <= 1e-8 * abs(F[k] @ uo)


def test_multi_rhs_equals_single_solves():
    """Each right-hand side of the batch converges like its own single solve."""
    wl = workloads.cantilever(32, 16, 16, lattice=(11, 7, 7))
    nc = int(np.prod([q + wl.order for q in wl.partition]))
    coeff = random_coeff(nc, seed=5)
    F = workloads.patch_loads(wl.nx, wl.ny, wl.nz, 4, seed0=77, patch=6)
    p = _problem(wl, coeff)
    p.multi_reserve(4)
    U, st, rr = p.solve_multi(F, rtol=1e-8)
    for k in range(4):
        p.put("f", F[k])
        p.put("u", np.zeros_like(F[k]))
        s = p.solve(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-8, max_iter=300, inner_max=1)
        assert s["relres"] <= 1e-8
        assert rel(U[k], p.get("u")) < 1e-6


def test_multi_rhs_errors():
    import ctypes as C
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    nc = int(np.prod([q + wl.order for q in wl.partition]))
    p = _problem(wl, np.full(nc, 0.5))
    o = capi.SolveOpts(capi.SOLVE_MIXED, capi.SMOOTH_CHEBYSHEV, 2, 2, 1e-6, 100, 0.1, 2, 0.3, 1.1, 1, 0, 0.0)
    st = capi.MultiStats()
    assert p.lib.topo_solve_multi(p.h, 1, C.byref(o), C.byref(st), None) == capi.TOPO_E_STATE
    p.multi_reserve(2)
    assert p.lib.topo_solve_multi(p.h, 3, C.byref(o), C.byref(st), None) == capi.TOPO_E_BAD_INPUT
    o.smoother = capi.SMOOTH_GS
    assert p.lib.topo_solve_multi(p.h, 1, C.byref(o), C.byref(st), None) == capi.TOPO_E_BAD_INPUT
    o.smoother, o.mode = capi.SMOOTH_CHEBYSHEV, capi.SOLVE_PCG64
    assert p.lib.topo_solve_multi(p.h, 1, C.byref(o), C.byref(st), None) == capi.TOPO_E_BAD_INPUT
