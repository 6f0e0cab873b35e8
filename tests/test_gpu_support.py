"""Heaviside projection and the self-support / drip constraints on the GPU
against the oracle restatement (oracle/support_oracle.py) on the same seeded
spline designs: projected density and its sensitivity chain at 1e-12,
surface points and normals at 1e-12, constraint values and coefficient
gradients at 1e-10 (FP64 on both sides), and the MMA design loop with the
projection and all three constraints (testOrdinarySplineTopoptMMA,
utils/test_utils.cpp:972-1217)."""
import numpy as np
import pytest

from oracle import support_oracle as so
from tests.helpers import rel, setup_gpu, setup_oracle
from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _pair(seed=3, dims=(12, 6, 6), lattice=(6, 5, 5)):
    wl = workloads.cantilever(*dims, lattice=lattice)
    nc = int(np.prod([q + wl.order for q in wl.partition]))
    coeff = np.random.default_rng(seed).uniform(0.15, 0.85, nc)
    return wl, coeff, setup_gpu(wl, coeff), setup_oracle(wl, coeff)


@pytest.mark.parametrize("beta", [1.0, 4.0, 16.0])
def test_heaviside_projection_chain(oracle_mod, beta):
    wl, coeff, g, o = _pair(dims=(16, 8, 8), lattice=(7, 5, 5))
    rho0 = o.get("rho")
    g.heaviside_project(beta)
    assert rel(g.get("rho_init"), rho0) < 1e-13
    act = o.get("eactive").astype(bool)
    proj = np.where(act, np.clip(so.heaviside(rho0, beta), 1e-3, 1.0), 0.0)
    assert rel(g.get("rho"), proj) < 1e-13
    o.put("rho", proj)
    for p in (g, o):
        p.update_operators()
    g.solve(mode=capi.SOLVE_PCG64, rtol=1e-10, max_iter=300)
    o.pcg(2, 2, 1e-10, 300, 0)
    g.sensitivity()
    o.sensitivity()
    g.heaviside_sensitivity(beta)
    o.put("sens", o.get("sens") * np.where(act, so.dirac(rho0, beta), 0.0))
    assert rel(g.get("sens"), o.get("sens")) < 1e-8
    g.put("sens", o.get("sens"))
    for p in (g, o):
        p.filter(2.0)
        p.spline_adjoint()
    assert rel(g.get("csens"), o.get("csens")) < 1e-12
    # projected volume: scale / den * dH/drho, filtered, adjoint
    den = o.gs_maps(0)[4]
    g.heaviside_volume_csens(beta, filter_radius=2.0, scale=1e3)
    o.put("sens", np.where(act, 1e3 / den * so.dirac(rho0, beta), 0.0))
    o.filter(2.0)
    o.spline_adjoint()
    assert rel(g.get("volcsens"), o.get("csens")) < 1e-12
    g.close()


CASES = [
    dict(ss_mode=4, drip_mode=6, drip_version=0, print_angle=0.75),
    dict(ss_mode=2, drip_mode=7, drip_version=1, print_angle=0.75, hfunction_c=10.0),
    dict(ss_mode=0, drip_mode=6, drip_version=1, print_angle=0.7, reference_quirks=1),
    dict(ss_mode=5, drip_mode=7, drip_version=0, print_angle=0.8, drip_beta=8.0, drip_mu=4.0, drip_beta_scale=1.0,
         reference_quirks=1),
    dict(ss_mode=3, drip_mode=4, print_angle=0.0),
]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("max_points", [400, 60])
def test_support_constraints_match_oracle(oracle_mod, case, max_points):
    opts = dict(CASES[case], lattice=10, max_points=max_points, beta=4.0)
    wl, coeff, g, o = _pair()
    bmin, bmax = wl.spline_box()
    spl = so.Spline(o, wl.order, wl.partition, bmin, bmax, coeff)
    count, pts = so.surface_points(o, spl, (wl.nx, wl.ny, wl.nz), 1.0, o.get("eactive"), 10, max_points)
    st = g.support_constraints(**opts)
    assert st["candidates"] == count and st["points"] == len(pts)
    gp = g.get("surf_points").reshape(3, -1).T
    assert np.abs(gp - pts).max() <= 1e-12
    ref = so.constraints(spl, pts, opts, 4.0, coeff.size)
    assert st["flipped"] == int(ref["flipped"]) and st["overhang_points"] == ref["down"]
    assert np.abs(g.get("surf_normals").reshape(3, -1).T - ref["normals"]).max() <= 1e-12 * np.abs(ref["normals"]).max()
    assert abs(st["ss_value"] - ref["ss"]) <= 1e-10 * max(1.0, abs(ref["ss"]))
    assert abs(st["drip_value"] - ref["drip"]) <= 1e-10 * max(1.0, abs(ref["drip"]))
    for name, key in (("sscsens", "gss"), ("dripcsens", "gdrip")):
        a, b = g.get(name), ref[key]
        assert np.abs(a - b).max() <= 1e-10 * max(np.abs(b).max(), 1e-30), (name, np.abs(a - b).max())
    g.close()


def test_mma_loop_with_projection_and_constraints():
    """Five MMA iterations with the Heaviside projection (beta 4) and the
    volume, self-support and drip constraints at the reference's scales
    (1e3, 1e-1, 1e2); two runs are bit for bit the same."""
    def run():
        wl, coeff, g, _ = _pair(seed=5, dims=(16, 8, 8), lattice=(7, 5, 5))
        g.put("coeff", np.full(coeff.size, 0.4))
        mma = capi.MMA.for_problem(g, 3, lb=1e-3, ub=1.0)
        dev = capi.load()
        hist = []
        for it in range(5):
            mma.get_x(g.device_ptr("coeff"))
            g.coeff_to_density()
            g.heaviside_project(4.0)
            vol = g.volume()
            g.update_operators()
            g.solve(mode=capi.SOLVE_PCG64, rtol=1e-8, max_iter=300)
            c = g.compliance()
            st = g.support_constraints(lattice=16, max_points=2000, beta=4.0, ss_mode=4, drip_mode=6,
                                       print_angle=0.75)
            g.sensitivity()
            g.heaviside_sensitivity(4.0)
            g.filter(2.0)
            g.spline_adjoint()
            g.heaviside_volume_csens(4.0, filter_radius=2.0, scale=1e3)
            ssc = g.get("sscsens") * 1e-1
            drc = g.get("dripcsens") * 1e2
            g.put("sscsens", ssc)
            g.put("dripcsens", drc)
            gv = [1e3 * (vol - wl.vgoal), 1e-1 * (st["ss_value"] - 1.0), 1e2 * st["drip_value"]]
            s = mma.update(g.device_ptr("csens"), [g.device_ptr("volcsens"), g.device_ptr("sscsens"),
                                                   g.device_ptr("dripcsens")], gv)
            hist.append((c, vol, st["ss_value"], st["drip_value"], st["points"], s["subiterations"]))
            assert np.isfinite(c) and np.isfinite(st["ss_value"]) and np.isfinite(st["drip_value"])
        x = mma.x
        mma.close()
        g.close()
        return hist, x
    h1, x1 = run()
    h2, x2 = run()
    assert h1 == h2 and np.array_equal(x1, x2)
    assert h1[-1][0] != h1[0][0]
