"""GPU MMA (topo_mma_*, one cooperative kernel per update) against the oracle's
restatement of the reference MMA (optimization/mma_t.*).

Both compute in FP64 and differ only in the order of the grid-wide sums, so the
iterates agree to rounding: the tests compare them step by step.  Device
buffers for the standalone optimiser come from torch (plumbing only)."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from oracle.oracle import OracleMMA
from tests.helpers import setup_gpu, setup_oracle, rel

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def _sync():
    import torch
    torch.cuda.synchronize()


def _case3():
    s3 = np.sqrt(3.0)

    def df(v):
        x, y = v
        e = np.exp(10 * (x - y) ** 2)
        return np.array([0.5 + 20 * (x - y) * e, s3 / 2 + 20 * (y - x) * e])

    def g(v):
        x, y = v
        return np.array([x * x + y * y - 1, x * x - 0.75, y * y - 0.75, (x + y) ** 2 - 1])

    def dg(v):
        x, y = v
        return np.array([[2 * x, 2 * y], [2 * x, 0.0], [0.0, 2 * y], [2 * (x + y), 2 * (x + y)]])

    return df, g, dg


def _step_both(gm, om, df, dg, g):
    dfd = _dev(df)
    dgd = [_dev(r) for r in dg]
    _sync()
    st = gm.update(dfd.data_ptr(), [t.data_ptr() for t in dgd], g)
    conv_o = om.update(df, dg, g)
    return st, conv_o


def test_reference_case3_trajectory():
    """The reference's MMA self-test problem (2 variables, 4 constraints), run
    to convergence on the GPU and the oracle side by side."""
    df, g, dg = _case3()
    gm = capi.MMA(2, 4, lb=-1.0, ub=1.0)
    om = OracleMMA(2, 4, -1.0, 1.0)
    assert np.allclose(gm.x, om.x, rtol=1e-14, atol=0)
    for it in range(100):
        x = om.x
        st, conv_o = _step_both(gm, om, df(x), dg(x), g(x))
        so = om.stats()
        assert st["subiterations"] == so["subiterations"], it
        assert np.abs(gm.x - om.x).max() <= 1e-12 * (1 + np.abs(om.x).max()), it
        assert st["converged"] == conv_o
        if conv_o:
            break
    assert conv_o and it < 100


@pytest.mark.parametrize("n,m", [(1000, 1), (100_000, 2), (70_785, 3), (5000, 4)])
def test_random_updates_multiblock(n, m):
    """Several updates on random gradients; n large enough for one CTA per SM."""
    rng = np.random.default_rng(n + m)
    lb = rng.uniform(0.0, 0.2, n)
    ub = lb + rng.uniform(0.5, 1.0, n)
    gm = capi.MMA(n, m, lb=lb, ub=ub)
    om = OracleMMA(n, m, lb, ub)
    # the device contracts multiply-adds, the oracle does not: last-bit differences
    assert np.allclose(gm.x, om.x, rtol=1e-14, atol=0)
    for it in range(4):
        df = rng.standard_normal(n) * rng.uniform(0.1, 10.0)
        dg = rng.standard_normal((m, n)) / n
        g = rng.uniform(-0.5, 0.5, m)
        st, _ = _step_both(gm, om, df, dg, g)
        so = om.stats()
        assert not st["overflow"]
        assert st["subiterations"] == so["subiterations"], it
        assert rel(gm.x, om.x) < 1e-11, it
        assert abs(st["dx_norm"] - so["dx_norm"]) <= 1e-10 * so["dx_norm"]


def test_spline_mma_design_loop_parity():
    """MMA on the spline coefficients of a cantilever (the reference's
    testOrdinarySplineTopoptMMA loop, utils/test_utils.cpp:1047-1186) for 6
    design iterations, GPU against the oracle chain."""
    wl = workloads.small_cases()["cantilever16"]
    nc = int(np.prod([q + wl.order for q in wl.partition]))
    p = setup_gpu(wl)
    o = setup_oracle(wl)
    vol_scale, vf, cmin = 1e3, 0.4, 1e-3
    gm = capi.MMA.for_problem(p, 1, lb=cmin, ub=1.0)
    om = OracleMMA(nc, 1, cmin, 1.0)
    assert np.allclose(gm.x, om.x, rtol=1e-14, atol=0)
    # d volume / d coefficient (topo_volume_csens into the handle's array; the
    # oracle by its adjoint of the constant 1/den field)
    p.volume_csens(scale=vol_scale)
    p.sync()
    ne_pad = _padded_elements(o)
    o.put("sens", np.where(o.get("eactive") != 0, vol_scale / ne_pad, 0.0))
    o.spline_adjoint()
    dv_o = o.get("csens")
    assert rel(p.get("volcsens"), dv_o) < 1e-13
    for it in range(6):
        s = capi.mma_design_iteration(p, gm, vf, solve=dict(mode=capi.SOLVE_PCG64, rtol=1e-10, max_iter=400))
        # oracle side of the same iteration
        o.put("coeff", om.x)
        o.coeff_to_density()
        vol = o.volume(True)
        o.update_operators()
        o.pcg(2, 2, 1e-10, 400, 0)
        c = o.compliance()
        o.sensitivity()
        o.filter(2.0)
        o.spline_adjoint()
        om.update(o.get("csens"), dv_o[None, :], [vol_scale * (vol - vf)])
        assert abs(s["volume"] - vol) <= 1e-12, it
        assert abs(s["compliance"] - c) <= 1e-8 * c, it
        assert rel(gm.x, om.x) < 1e-8, it
    assert abs(s["volume"] - vf) < abs(0.5 - vf)


def _padded_elements(o):
    _, _, _, _, nge = o.gs_maps(0)
    return nge


def test_mma_errors():
    with pytest.raises(capi.TopoError) as e:
        capi.MMA(10, 5)
    assert e.value.code == capi.TOPO_E_BAD_INPUT
    gm = capi.MMA(10, 1)
    d = _dev(np.zeros(10))
    _sync()
    with pytest.raises(capi.TopoError) as e:
        gm.update(d.data_ptr(), [d.data_ptr()], [0.0])
    assert e.value.code == capi.TOPO_E_STATE
    with pytest.raises(capi.TopoError) as e:
        gm.init(1.0, 0.5)
    assert e.value.code == capi.TOPO_E_BAD_INPUT
    gm.init(0.0, 1.0)
    with pytest.raises(capi.TopoError) as e:
        gm.update(d.data_ptr(), [d.data_ptr()], [float("nan")])
    assert e.value.code == capi.TOPO_E_BAD_INPUT
