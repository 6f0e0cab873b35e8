"""A whole design iteration as one CUDA graph (topo_design_iteration with
graphs on: operator update, spectral bounds with device-side restarts, the
mixed solve's nested device loops, compliance, sensitivity, filter, adjoint,
OC bisection) against the same iteration run from the host, kernel for kernel:
the same designs, compliances, iteration counts and OC trials bit for bit;
checkpoint/resume and a failed solve behave as on the host."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _make(graphs, wl=None):
    wl = wl or workloads.small_cases()["mbb32"]
    p = capi.Problem(wl.nx, wl.ny, wl.nz, eactive=wl.eactive)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), wl.coeff0))
    p.coeff_to_density()
    p.set_operator_precision(2)
    p.set_graphs(graphs)
    return wl, p


def _opts(wl, inner_max):
    solve = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, pre=1, post=1, rtol=1e-6, max_iter=300,
                 inner_max=inner_max, inner_rtol=0.05, cheb_degree=3, cheb_lo=0.1)
    return dict(solve=solve, oc=dict(vgoal=wl.vgoal))


def _run(p, opts, n):
    out = []
    for _ in range(n):
        s = p.design_iteration(**opts)
        out.append((s["compliance"], s["iterations"], s["vcycles"], s["relres"], s["oc_trials"], s["volume"]))
    return out, p.get("coeff"), p.get("rho"), p.get("u")


CASES = {
    "mbb32": lambda: workloads.small_cases()["mbb32"],
    "perforated37": lambda: _perforated(),
}


def _perforated():
    w = workloads.cantilever(37, 21, 13, lattice=(9, 6, 5))
    w.eactive = workloads.perforated(37, 21, 13, holes=6, radius=(2.0, 4.0), seed=5)
    return w


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("inner_max", [1, 4])
def test_iteration_graph_matches_host(case, inner_max):
    res = {}
    for graphs in (1, 0):
        wl, p = _make(graphs, CASES[case]())
        res[graphs] = _run(p, _opts(wl, inner_max), 5)
        state = p.graph_state()
        assert state["iteration"] == bool(graphs), p.last_error()
    (s1, c1, r1, u1), (s0, c0, r0, u0) = res[1], res[0]
    assert s1 == s0
    assert np.array_equal(c1, c0) and np.array_equal(r1, r0) and np.array_equal(u1, u0)
    assert all(x[3] <= 1e-6 for x in s1)


def test_graph_modes_agree():
    """topo_set_graphs 1 (whole-iteration graph), 3 (outer solve graph, no
    iteration graph), 2 (outer loop on the host) and 0 (no graphs): the same
    design iterations bit for bit, each mode holding the graphs it names."""
    res = {}
    want = {1: {"iteration"}, 3: {"solve", "nested_inner", "oc"}, 2: {"inner", "oc"}, 0: set()}
    for mode in (1, 3, 2, 0):
        wl, p = _make(mode)
        res[mode] = _run(p, _opts(wl, 4), 4)
        held = {k for k, v in p.graph_state().items() if v}
        assert want[mode] <= held, (mode, held, p.last_error())
    for mode in (3, 2, 0):
        assert res[mode][0] == res[1][0], mode
        assert np.array_equal(res[mode][1], res[1][1]), mode


def test_graph_mode_argument_checked():
    _, p = _make(1)
    for bad in (-1, 4):
        with pytest.raises(capi.TopoError):
            p.set_graphs(bad)


def test_iteration_graph_resume(tmp_path):
    """Checkpoint after two graphed iterations, three more, then a fresh
    handle resumed from the checkpoint runs the same three bit for bit (its
    first iteration on the host, the rest as graphs)."""
    wl, p = _make(1)
    opts = _opts(wl, 4)
    _run(p, opts, 2)
    path = str(tmp_path / "it.ckpt")
    p.checkpoint_save(path)
    ref = _run(p, opts, 3)
    _, q = _make(1)
    q.checkpoint_load(path)
    got = _run(q, opts, 3)
    assert got[0] == ref[0]
    assert np.array_equal(got[1], ref[1])


def test_iteration_graph_failed_solve_keeps_design():
    """A start vector whose residual overflows the FP32 inner solver: the
    iteration fails with a non-finite residual in both forms, coefficients and
    density stay those the iteration started from, and the next iteration
    from a zero start runs."""
    out = {}
    for graphs in (1, 0):
        wl, p = _make(graphs)
        opts = _opts(wl, 4)
        _run(p, opts, 2)
        c0, r0 = p.get("coeff"), p.get("rho")
        n3 = p.get("u").size
        p.put("u", 1e30 * np.random.default_rng(0).uniform(-1.0, 1.0, n3))
        with pytest.raises(capi.TopoError) as e:
            p.design_iteration(**opts)
        assert e.value.code == capi.TOPO_E_NONFINITE
        assert np.array_equal(p.get("coeff"), c0) and np.array_equal(p.get("rho"), r0)
        p.put("u", np.zeros(n3))
        s = p.design_iteration(**opts)
        assert s["relres"] <= 1e-6
        out[graphs] = (s["compliance"], p.get("coeff"))
    assert out[1][0] == out[0][0] and np.array_equal(out[1][1], out[0][1])
