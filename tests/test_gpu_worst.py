"""Worst-case compliance on the GPU (block Rayleigh-Ritz over multi-RHS solves)
against the exact worst case from the oracle: the largest eigenpair of
M = S^T K^-1 S (oracle/worst_oracle.py), loads along the end-face normal or in
any direction.  Tolerances: compliance 1e-6 relative (FP64 rel-res 1e-8 final
solve), load direction 1e-6 where the leading eigenvalue is simple."""
import numpy as np
import pytest

from oracle import worst_oracle
from tests.helpers import rel, setup_gpu, setup_oracle
from tests.test_oracle_worst import end_face
from topoptspline3d_gb300 import workloads

pytestmark = pytest.mark.gpu


def _pair(dims):
    wl = workloads.cantilever(*dims, lattice=(7, 5, 5))
    g, o = setup_gpu(wl), setup_oracle(wl)
    g.update_operators()
    o.update_operators()
    return wl, g, o


@pytest.mark.parametrize("free", [False, True])
@pytest.mark.parametrize("block", [1, 8])
def test_worst_compliance_matches_largest_eigenpair(oracle_mod, free, block):
    dims = (16, 10, 6)
    wl, g, o = _pair(dims)
    vid, nrm = end_face(*dims)
    lam, vec, w = worst_oracle.dense_worst(o, vid, nrm, free)
    g.set_load_region(vid, nrm)
    st = g.worst_compliance(block=block, free_direction=free, tol=1e-7, rtol=1e-8, max_iter=400, seed=5)
    assert abs(st["compliance"] - lam) <= 1e-6 * lam, (st, lam)
    if block > 1:
        assert abs(st["second"] - w[1]) <= 1e-4 * lam
    # F holds the unit worst load, U its displacement
    f, u = g.get("f"), g.get("u")
    assert abs(np.linalg.norm(f) - 1.0) <= 1e-12
    x = worst_oracle.gather(o, vid, nrm, f, free)
    assert abs(abs(np.dot(x, vec)) - 1.0) <= 1e-6
    assert abs(np.dot(f, u) - st["compliance"]) <= 1e-9 * lam
    g.close()


def test_equal_leading_loads(oracle_mod):
    """A square section has two equal bending loads: the compliance is still
    the largest eigenvalue, and the block finds both."""
    dims = (16, 8, 8)
    wl, g, o = _pair(dims)
    vid, nrm = end_face(*dims)
    lam, vec, w = worst_oracle.dense_worst(o, vid, nrm, False)
    assert abs(w[1] - w[0]) <= 1e-9 * w[0]
    g.set_load_region(vid, nrm)
    st = g.worst_compliance(block=4, tol=1e-6, rtol=1e-8, max_iter=400, seed=2)
    assert abs(st["compliance"] - lam) <= 1e-6 * lam
    assert abs(st["second"] - lam) <= 1e-6 * lam
    g.close()


def test_robust_design_chain(oracle_mod):
    """The design chain after the worst-case solve acts on the worst load: the
    sensitivities, filter and spline adjoint equal the oracle's for that load."""
    dims = (16, 10, 6)
    wl, g, o = _pair(dims)
    vid, nrm = end_face(*dims)
    g.set_load_region(vid, nrm)
    st = g.worst_compliance(block=8, tol=1e-7, rtol=1e-10, max_iter=400, seed=5)
    o.put("f", g.get("f"))
    o.put("u", np.zeros(3 * wl.nv))
    o.pcg(2, 2, 1e-11, 500, 0)
    assert abs(o.compliance() - st["compliance"]) <= 1e-8 * st["compliance"]
    for p in (g, o):
        p.sensitivity()
        p.filter(wl.filter_radius)
        p.spline_adjoint()
    assert rel(g.get("csens"), o.get("csens")) <= 1e-8
    tg, _ = g.oc_update(wl.vgoal)
    to, _ = o.oc_update(wl.vgoal)
    assert tg == to
    assert rel(g.get("coeff"), o.get("coeff")) <= 1e-8
    g.close()
