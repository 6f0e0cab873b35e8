"""The autotuner (topo_autotune): kernel z-march depth and mixed-solver schedule
picked by timing on the live problem state."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def test_autotune_picks_converging_schedule_and_restores_state():
    wl = workloads.half_mbb(64, 32, 32, lattice=(17, 9, 9))
    p = capi.Problem(64, 32, 32)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), wl.coeff0))
    p.coeff_to_density()
    p.set_operator_precision(2)
    p.update_operators()
    u0 = p.get("u")
    base = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-6, max_iter=300, inner_max=4)
    best, rep = p.autotune(base)
    assert np.array_equal(p.get("u"), u0)
    assert rep["tz32"] in (4, 8, 16, 32) and rep["tz64"] in (4, 8, 16, 32)
    # 4 inner counts x 2 smoothing counts x 2 degrees x 2 lower interval ends x 2 inner
    # tolerances, then two coordinate passes of 3 lower ends, 1 tolerance and 1 degree,
    # then 3 degrees x 3 lower ends x 2 tolerances jointly, then 2 inner counts x 2
    # inner tolerances and the next degree
    assert rep["candidates"] == 97 and rep["best_ms"] <= rep["base_ms"]
    # the fastest FP32 Chebyshev step over the depths, both element-product forms
    # and the three tile heights of the modal form
    rows_ms = rep["cheb_rows_ms"]
    fastest = min(rep["cheb_ms"] + rep["cheb_tc_ms"] + rows_ms[4] + rows_ms[16])
    k = (4, 8, 16, 32).index(rep["tz32"])
    assert rep["rows32"] in (4, 8, 16) and not (rep["tc"] and rep["rows32"] != 8)
    chosen = rep["cheb_tc_ms"] if rep["tc"] else rows_ms.get(rep["rows32"], rep["cheb_ms"])
    assert fastest == chosen[k]
    assert best["mode"] == capi.SOLVE_MIXED and best["rtol"] == 1e-6
    assert best["inner_max"] in (1, 2, 3, 4, 5, 6, 8, 10) and best["pre"] in (1, 2)
    assert 2 <= best["cheb_degree"] <= 5
    assert best["cheb_lo"] in (0.02, 0.04, 0.05, 0.06, 0.1, 0.2, 0.3)
    assert best["inner_rtol"] in (0.1, 0.05, 0.03, 0.02, 0.01)
    s = p.solve(**best)
    assert s["relres"] <= 1e-6
    # the tuned z-march depth is used by the solver and gives the same operator
    u = np.random.default_rng(1).standard_normal(3 * p.nv) * np.repeat((p.get("vmask") & 8) != 0, 3)
    assert np.allclose(p.apply_fine(u, 3), p.apply_fine(u, 0), rtol=0, atol=1e-12 * np.abs(p.apply_fine(u, 0)).max())


def test_autotune_rejects_other_modes():
    wl = workloads.small_cases()["cantilever16"]
    p = capi.Problem(wl.nx, wl.ny, wl.nz)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), 0.5))
    p.coeff_to_density()
    p.update_operators()
    with pytest.raises(capi.TopoError) as e:
        p.autotune(dict(mode=capi.SOLVE_PCG64))
    assert e.value.code == capi.TOPO_E_BAD_INPUT
