"""Many independent designs of uneven sizes at once (topo_design_batch): the
concurrent run (a host thread per design, each design iteration one graph
launch after the first) reproduces, bit for bit, each design run on its own."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

SOLVE = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-6, max_iter=300, inner_max=4)


def _make(wl):
    p = capi.Problem(wl.nx, wl.ny, wl.nz)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), wl.coeff0))
    p.coeff_to_density()
    p.set_operator_precision(2)
    return p


def test_batch_equals_sequential():
    wls = workloads.batch_cantilevers(6, seed0=2000, nx_range=(24, 48), nyz_range=(16, 24))
    ocs = [dict(vgoal=w.vgoal) for w in wls]
    batch = [_make(w) for w in wls]
    last, bs = capi.design_batch(batch, 3, threads=6, solve=SOLVE, ocs=ocs)
    assert bs["failures"] == 0 and bs["wall_ms"] > 0
    # after each design's first iteration (host sequence) its iterations ran as one graph each
    assert all(q.graph_state()["iteration"] for q in batch)
    for k, w in enumerate(wls):
        p = _make(w)
        for _ in range(3):
            s = p.design_iteration(solve=SOLVE, oc=ocs[k])
        assert s["compliance"] == last[k]["compliance"], k
        assert np.array_equal(p.get("coeff"), batch[k].get("coeff")), k


@pytest.mark.parametrize("inner_rtol", [1e-1, 1e-3])
def test_graphs_do_not_change_results(inner_rtol):
    """Graphs on: the V-cycle replays as one graph, and the inner FP32 CG and
    the OC bisection each run as one graph whose loop is decided on the device
    (the CG stopping on the inner tolerance, or on the iteration cap with the
    tighter one).  Graphs off: the same kernels launched one by one with the
    loops on the host.  Results, iteration, V-cycle and trial counts agree
    exactly, over design iterations whose spectral bounds differ."""
    wl = workloads.small_cases()["mbb32"]
    solve = dict(SOLVE, inner_rtol=inner_rtol)
    runs = []
    for g in (0, 1):
        p = _make(wl)
        p.set_graphs(g)
        s = [p.design_iteration(solve=solve, oc=dict(vgoal=0.35)) for _ in range(3)]
        runs.append(([(x["compliance"], x["iterations"], x["vcycles"], x["relres"], x["oc_trials"], x["volume"])
                      for x in s], p.get("u"), p.get("coeff")))
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][1], runs[1][1]) and np.array_equal(runs[0][2], runs[1][2])
    assert all(x[2] > x[1] for x in runs[1][0])  # several inner iterations per outer one


def test_material_must_match_live_handles():
    a = capi.Problem(8, 8, 8)
    with pytest.raises(capi.TopoError):
        capi.Problem(8, 8, 8, E=2e6)
    b = capi.Problem(8, 8, 8)  # same material is fine
    del a, b
