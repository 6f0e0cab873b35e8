"""GPU parity: the CUDA library against the CPU FP64 oracle on identical seeded
inputs, through the C ABI.  Tolerances: FP64 kernels 1e-12 relative per
operation and 1e-8 for solver outputs (compliance, displacements, sensitivities);
FP32 kernels 1e-5; the mixed-precision solve 1e-6 on compliance."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import setup_gpu, setup_oracle, rel, random_masked_u, random_coeff

pytestmark = pytest.mark.gpu

CASES = ["cantilever16", "mbb32", "cantilever48"]


def _case(name):
    return workloads.small_cases()[name]


@pytest.fixture(params=CASES)
def pair(request, oracle_mod):
    wl = _case(request.param)
    nc = int(np.prod([p + wl.order for p in wl.partition]))
    coeff = random_coeff(nc, seed=11)
    return wl, setup_gpu(wl, coeff), setup_oracle(wl, coeff)


def test_hierarchy_and_template(pair):
    wl, g, o = pair
    assert g.num_levels() == o.num_levels()
    for l in range(o.num_levels()):
        assert g.level_dims(l)[0] == tuple(o.level_dims(l))
        assert np.array_equal(g.get("eactive", l), o.get("eactive", l))
    assert np.array_equal(g.get("vmask"), o.get("vmask"))
    assert rel(g.get("ke"), o.get("ke")) < 1e-13


def test_density(pair):
    wl, g, o = pair
    assert rel(g.get("rho"), o.get("rho")) < 1e-13


def test_fine_operator_fp64_fp32(pair):
    wl, g, o = pair
    u = random_masked_u(wl.nv, o.get("vmask"), 5)
    o.update_penalised()
    y_o = o.apply_fine(u)
    assert rel(g.apply_fine(u, 0), y_o) < 1e-12   # modal FP64 kernel
    assert rel(g.apply_fine(u, 2), y_o) < 1e-12   # dense-row FP64 kernel
    assert rel(g.apply_fine(u, 1), y_o) < 1e-5    # modal FP32 kernel
    # double-float modal kernel: ~48-bit significands; elementwise against FP64
    y_df, y_64 = g.apply_fine(u, 3), g.apply_fine(u, 0)
    assert rel(y_df, y_o) < 1e-12
    assert np.abs(y_df - y_64).max() <= 1e-12 * np.abs(y_64).max()


def test_galerkin_levels(pair):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    for l in range(1, o.num_levels()):
        assert rel(g.get("kelem", l), o.get("kelem", l)) < 1e-12, l
        assert rel(g.get("stencil", l), o.get("stencil", l)) < 1e-12, l


def test_smoother_transfers_coarsest(pair):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    u = random_masked_u(wl.nv, o.get("vmask"), 9) * 1e-6
    for p in (g, o):
        p.put("u", u)
        p.smooth(0, 1)
    assert rel(g.get("u"), o.get("u")) < 1e-12
    for p in (g, o):
        p.smooth(0, 1, reverse=True)
        p.residual(0)
    assert rel(g.get("r"), o.get("r")) < 1e-10
    nl = o.num_levels()
    for l in range(1, nl):
        for p in (g, o):
            p.restrict(l)
        assert rel(g.get("f", l), o.get("f", l)) < 1e-12
        if l < nl - 1:
            for p in (g, o):
                p.put("u", np.zeros(3 * g.size("u", l) // 3), l)
                p.smooth(l, 2)
                p.residual(l)
            assert rel(g.get("u", l), o.get("u", l)) < 1e-11
    for p in (g, o):
        p.coarsest_solve()
    assert rel(g.get("u", nl - 1), o.get("u", nl - 1)) < 1e-9
    for p in (g, o):
        p.prolong(nl - 2)
    assert rel(g.get("u", nl - 2), o.get("u", nl - 2)) < 1e-9


def test_reference_vcycle_sequence(pair):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    for k in range(3):
        rg, ro = g.vcycle(5, 5), o.vcycle(5, 5)
        assert abs(rg - ro) < 1e-8 * ro, (k, rg, ro)
    assert rel(g.get("u"), o.get("u")) < 1e-8


@pytest.mark.parametrize("smoother", [capi.SMOOTH_GS, capi.SMOOTH_CHEBYSHEV])
def test_pcg64_matches_oracle(pair, smoother):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    st = g.solve(mode=capi.SOLVE_PCG64, smoother=smoother, rtol=1e-6, max_iter=200)
    it_o, rr_o = o.pcg(2, 2, 1e-6, 200, smoother)
    assert st["relres"] <= 1e-6 and rr_o <= 1e-6
    assert abs(st["iterations"] - it_o) <= 1
    assert abs(g.compliance() - o.compliance()) < 1e-8 * abs(o.compliance())
    assert rel(g.get("u"), o.get("u")) < 1e-8


@pytest.mark.parametrize("smoother", [capi.SMOOTH_GS, capi.SMOOTH_CHEBYSHEV])
def test_mixed_solve_tolerance(pair, smoother):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    st = g.solve(mode=capi.SOLVE_MIXED, smoother=smoother, rtol=1e-6, max_iter=400)
    assert st["relres"] <= 1e-6
    o.pcg(2, 2, 1e-10, 400, 0)
    assert abs(g.compliance() - o.compliance()) < 1e-6 * abs(o.compliance())
    assert rel(g.get("u"), o.get("u")) < 1e-4


def test_sensitivity_filter_adjoint(pair):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    g.solve(mode=capi.SOLVE_PCG64, rtol=1e-8, max_iter=300)
    o.pcg(2, 2, 1e-8, 300, 0)
    for p in (g, o):
        p.sensitivity()
    assert rel(g.get("sens"), o.get("sens")) < 1e-8
    # same U on both sides for the remaining chain
    g.put("sens", o.get("sens"))
    for p in (g, o):
        p.filter(wl.filter_radius)
    assert rel(g.get("sens"), o.get("sens")) < 1e-13
    for p in (g, o):
        p.spline_adjoint()
    assert rel(g.get("csens"), o.get("csens")) < 1e-13


@pytest.mark.parametrize("twice", [False, True])
def test_oc_update(pair, twice):
    wl, g, o = pair
    o.update_operators()
    o.pcg(2, 2, 1e-8, 300, 0)
    o.sensitivity()
    o.filter(wl.filter_radius)
    o.spline_adjoint()
    g.put("csens", o.get("csens"))
    tg, lg = g.oc_update(0.3, apply_twice=twice)
    to, lo = o.oc_update(0.3, apply_twice=twice)
    assert tg == to and abs(lg - lo) <= 1e-12 * abs(lo)
    assert rel(g.get("coeff"), o.get("coeff")) < 1e-12
    assert rel(g.get("rho"), o.get("rho")) < 1e-12
    assert abs(g.volume() - o.volume()) < 1e-12


def test_design_iterations_history(oracle_mod):
    wl = _case("cantilever16")
    g, o = setup_gpu(wl), setup_oracle(wl)
    cg, co = [], []
    for it in range(6):
        s = g.design_iteration(solve=dict(mode=capi.SOLVE_PCG64, rtol=1e-8, max_iter=300),
                               oc=dict(vgoal=wl.vgoal))
        cg.append(s["compliance"])
        o.update_operators()
        o.pcg(2, 2, 1e-8, 300, 0)
        co.append(o.compliance())
        o.sensitivity(); o.filter(wl.filter_radius); o.spline_adjoint(); o.oc_update(wl.vgoal)
    assert np.allclose(cg, co, rtol=1e-7, atol=0), (cg, co)
    assert rel(g.get("coeff"), o.get("coeff")) < 1e-6


@pytest.mark.parametrize("smoother", [capi.SMOOTH_GS, capi.SMOOTH_CHEBYSHEV])
def test_masked_domain_and_odd_sizes(oracle_mod, smoother):
    nx, ny, nz = 37, 21, 13
    wl = workloads.cantilever(nx, ny, nz, lattice=(9, 6, 5))
    wl.eactive = workloads.perforated(nx, ny, nz, holes=6, radius=(2.0, 4.0), seed=5)
    g, o = setup_gpu(wl), setup_oracle(wl)
    assert np.array_equal(g.get("vmask"), o.get("vmask"))
    assert rel(g.get("rho"), o.get("rho")) < 1e-13
    g.update_operators(); o.update_operators()
    for l in range(1, o.num_levels()):
        assert rel(g.get("stencil", l), o.get("stencil", l)) < 1e-12
    st = g.solve(mode=capi.SOLVE_PCG64, smoother=smoother, rtol=1e-6, max_iter=300)
    it, rr = o.pcg(2, 2, 1e-6, 300, smoother)
    assert rr <= 1e-6 and st["relres"] <= 1e-6 and abs(st["iterations"] - it) <= 1
    assert abs(g.compliance() - o.compliance()) < 1e-8 * abs(o.compliance())
    st = g.solve(mode=capi.SOLVE_MIXED, smoother=smoother, rtol=1e-6, max_iter=300)
    assert st["relres"] <= 1e-6
    assert abs(g.compliance() - o.compliance()) < 1e-6 * abs(o.compliance())


def test_floating_parts_coarsest_pseudo_inverse(oracle_mod):
    # disjoint ellipsoids: parts without supports make the coarse operators
    # singular; both sides drop the same null directions of the coarsest matrix
    nx, ny, nz = 40, 24, 16
    wl = workloads.cantilever(nx, ny, nz, lattice=(9, 7, 5))
    wl.eactive = workloads.ellipsoid_union(nx, ny, nz, n=5, seed=5, axes=(3, 8), fill=(0.05, 0.6))
    from tests.test_oracle_known_answers import _stencil_to_matrix
    g, o = setup_gpu(wl), setup_oracle(wl)
    g.update_operators(); o.update_operators()
    nl = o.num_levels()
    A = _stencil_to_matrix(o.get("stencil", nl - 1), o.level_dims(nl - 1))
    # right-hand side in the range of the (singular) coarsest operator, SoA layout
    x = np.random.default_rng(2).standard_normal(A.shape[0])
    f = A @ x
    for p in (g, o):
        p.put("f", f, nl - 1)
        p.coarsest_solve()
        u = p.get("u", nl - 1)
        assert np.isfinite(u).all()
        assert np.linalg.norm(A @ u - f) <= 1e-6 * np.linalg.norm(f)


def test_reference_gs_maps_on_device_handle(pair):
    wl, g, o = pair
    for l in range(o.num_levels()):
        a, b = g.gs_maps(l), o.gs_maps(l)
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))


def test_determinism_bitwise(oracle_mod):
    wl = _case("mbb32")
    runs = []
    for _ in range(2):
        g = setup_gpu(wl, random_coeff(11 * 7 * 7, seed=4))
        s = g.design_iteration(solve=dict(mode=capi.SOLVE_MIXED, rtol=1e-6), oc=dict(vgoal=0.35))
        runs.append((s["compliance"], g.get("u"), g.get("coeff")))
        g.close()
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][1], runs[1][1]) and np.array_equal(runs[0][2], runs[1][2])


def test_error_codes():
    wl = _case("cantilever16")
    g = capi.Problem(wl.nx, wl.ny, wl.nz)
    with pytest.raises(capi.TopoError) as e:
        g.update_operators()
    assert e.value.code == capi.TOPO_E_STATE
    g.set_bc(wl.fixed, wl.loads)
    with pytest.raises(capi.TopoError) as e:
        g.coeff_to_density()
    assert e.value.code == capi.TOPO_E_STATE
    with pytest.raises(capi.TopoError) as e:
        g.put("rho", np.zeros(3))
    assert e.value.code == capi.TOPO_E_BAD_INPUT
    bad = wl.loads.copy(); bad[5] = np.nan
    with pytest.raises(capi.TopoError) as e:
        g.set_bc(wl.fixed, bad)
    assert e.value.code == capi.TOPO_E_BAD_INPUT
    # zero load: the solve returns U = 0 immediately
    g.set_bc(wl.fixed, np.zeros_like(wl.loads))
    g.update_operators()
    s = g.solve(mode=capi.SOLVE_PCG64)
    assert s["relres"] == 0.0 and not g.get("u").any()
    # iteration cap: TOPO_E_NOT_CONVERGED, state still usable
    g.set_bc(wl.fixed, wl.loads)
    g.update_operators()
    s = g.solve(mode=capi.SOLVE_PCG64, rtol=1e-14, max_iter=2, check=False)
    assert s["rc"] == capi.TOPO_E_NOT_CONVERGED and s["iterations"] == 2
    s = g.solve(mode=capi.SOLVE_PCG64, rtol=1e-6, max_iter=200)
    assert s["relres"] <= 1e-6


@pytest.mark.parametrize("mode", [capi.SOLVE_MIXED, capi.SOLVE_PCG64])
def test_design_iteration_energy_sensitivity(oracle_mod, mode):
    """topo_design_iteration takes the sensitivity from the element energies of
    the solve's final double-float residual; the step-by-step calls take it from
    topo_sensitivity.  Same solve, so the designs agree to rounding."""
    wl = _case("mbb32")
    nc = int(np.prod([p + wl.order for p in wl.partition]))
    coeff = random_coeff(nc, seed=5)
    a, b = setup_gpu(wl, coeff), setup_gpu(wl, coeff)
    opts = dict(mode=mode, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-8, max_iter=300, inner_max=4)
    sa = a.design_iteration(solve=opts, oc=dict(vgoal=wl.vgoal))
    b.update_operators()
    b.solve(**opts)
    cb = b.compliance()
    b.sensitivity()
    b.filter(2.0)
    b.spline_adjoint()
    b.oc_update(wl.vgoal)
    assert abs(sa["compliance"] - cb) <= 1e-14 * abs(cb)
    assert rel(a.get("coeff"), b.get("coeff")) < 1e-12
    assert rel(a.get("rho"), b.get("rho")) < 1e-12
