"""The loops that run on the device inside CUDA graphs (the mixed solve's outer
FP64 CG with the inner FP32 CG nested in it, the OC bisection) against the same
loops run from the host: their stopping rules (tolerance, iteration cap, a
non-finite residual) give the same outcome, and a failed solve leaves the
handle usable."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

SOLVE = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-6, max_iter=300, inner_max=4)


def _make(graphs):
    wl = workloads.small_cases()["mbb32"]
    p = capi.Problem(wl.nx, wl.ny, wl.nz)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), wl.coeff0))
    p.coeff_to_density()
    p.set_operator_precision(2)
    p.set_graphs(graphs)
    p.update_operators()
    return p


@pytest.mark.parametrize("graphs", [0, 1])
def test_inner_cap(graphs):
    """An inner tolerance that is never met: every inner solve stops at the cap,
    so the V-cycle count is the cap times the outer iterations."""
    p = _make(graphs)
    s = p.solve(**dict(SOLVE, inner_rtol=1e-30, inner_max=3))
    assert s["relres"] <= 1e-6
    assert s["vcycles"] == 3 * s["iterations"]


@pytest.mark.parametrize("graphs", [0, 1])
def test_nonfinite_inner_residual(graphs):
    """A start vector of random values of size 1e30 (not a rigid translation,
    so K u is of that size too) is finite in FP64, but the residual's squares
    overflow the FP32 inner solver: both loop forms stop and report a
    non-finite residual, and the next solve from zero converges on the same
    handle."""
    p = _make(graphs)
    n3 = p.get("u").size
    p.put("u", 1e30 * np.random.default_rng(0).uniform(-1.0, 1.0, n3))
    with pytest.raises(capi.TopoError) as e:
        p.solve(**SOLVE)
    assert e.value.code == capi.TOPO_E_NONFINITE
    p.put("u", np.zeros(n3))
    s = p.solve(**SOLVE)
    assert s["relres"] <= 1e-6


@pytest.mark.parametrize("inner_max", [1, 4])
def test_outer_loop_on_device_matches_host(inner_max):
    """The outer CG as one graph launch (one V-cycle per outer iteration, or the
    graphed inner CG as a nested WHILE loop) runs the host loop's kernels in
    the host loop's order: the same iteration and V-cycle counts and the same
    solution bit for bit, on the first solve (capture) and on a replay."""
    res = []
    for graphs in (1, 0):
        p = _make(graphs)
        u0 = p.get("u")
        runs = []
        for _ in range(2):
            p.put("u", u0)
            s = p.solve(**dict(SOLVE, inner_max=inner_max))
            runs.append((s["iterations"], s["vcycles"], s["relres"], p.get("u")))
        state = p.graph_state()
        if graphs:  # the outer loop ran as a graph, with the inner CG nested in it
            assert state["solve"] and state["nested_inner"] == (inner_max > 1) and not state["inner"]
        else:
            assert not any(state.values())
        res.append(runs)
    for (it_g, vc_g, rr_g, u_g), (it_h, vc_h, rr_h, u_h) in zip(res[0], res[1]):
        assert (it_g, vc_g, rr_g) == (it_h, vc_h, rr_h)
        assert np.array_equal(u_g, u_h)
    assert res[0][0][2] <= 1e-6


@pytest.mark.parametrize("graphs", [0, 1])
def test_outer_cap(graphs):
    """A tolerance that is never met: the outer loop stops at max_iter in both
    forms and the solve reports that it did not converge."""
    p = _make(graphs)
    s = p.solve(**dict(SOLVE, rtol=1e-30, max_iter=5, inner_max=2), check=False)
    assert s["rc"] == capi.TOPO_E_NOT_CONVERGED
    assert s["iterations"] == 5 and s["vcycles"] <= 10


def test_oc_loop_matches_host():
    """Same sensitivities and volume goal: the device bisection and the host one
    take the same number of trials to the same threshold and coefficients."""
    res = []
    for graphs in (0, 1):
        p = _make(graphs)
        p.solve(**SOLVE)
        p.sensitivity()
        p.filter(2.0)
        p.spline_adjoint()
        trials, lam = p.oc_update(0.3)
        res.append((trials, lam, p.get("coeff"), p.get("rho")))
    assert res[0][0] == res[1][0] and res[0][1] == res[1][1]
    assert np.array_equal(res[0][2], res[1][2]) and np.array_equal(res[0][3], res[1][3])
