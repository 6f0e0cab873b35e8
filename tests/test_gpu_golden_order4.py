"""GPU parity pinned by the reference's own code, cubic (order 4) splines on the
GPU, and the full 50-iteration plain-method run (config 0).

- The CUDA spline density, spline adjoint and filter against the golden vectors
  of the reference's coeff2density, ddensity2dcoeff_update and filterSensitivity
  (tests/golden, FP32 in the reference: tolerances at FP32 rounding).
- Order 4 (cubic, 4 taps per axis, 64 coefficients per element) density,
  adjoint and OC update against the oracle at 1e-12 on the three small cases.
- 48x24x24 cantilever, lattice 13x7x7, 50 design iterations of plain FP64
  MG-PCG with the OC update (utils/test_utils.cpp:928-958 with a rel-res 1e-6
  solve): compliance per iteration within 1e-8 of the oracle's.
"""
import numpy as np
import pytest

from tests import golden
from tests.helpers import rel, random_coeff, setup_gpu, setup_oracle
from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

G = golden.load()
N = int(G["cube"])


def _cube(mask, order, part):
    p = capi.Problem(N, N, N, eactive=mask)
    p.set_spline(order, part, (0.0, 0.0, 0.0), (float(N),) * 3)
    return p


@pytest.mark.parametrize("i", range(int(G["n_dens"])))
def test_density_adjoint_vs_reference_code(i):
    order, part = int(G[f"dens_{i}_order"]), [int(p) for p in G[f"dens_{i}_part"]]
    mask = golden.words_to_mask(G[f"dens_{i}_words"], N)
    act = mask.astype(bool)
    p = _cube(mask, order, part)
    p.put("coeff", G[f"dens_{i}_coeff"].astype(np.float64))
    p.coeff_to_density()
    assert np.abs(p.get("rho")[act] - G[f"dens_{i}_rho"]).max() <= 2e-6
    sens = np.zeros(N ** 3)
    sens[act] = G[f"adj_{i}_sens"]
    p.put("sens", sens)
    p.spline_adjoint()
    assert rel(p.get("csens"), G[f"adj_{i}_csens"]) <= 1e-5
    p.close()


@pytest.mark.parametrize("i", range(int(G["n_filt"])))
def test_filter_vs_reference_code(i):
    mask = golden.words_to_mask(G[f"filt_{i}_words"], N)
    act = mask.astype(bool)
    p = _cube(mask, 3, [3, 3, 3])
    sens = np.zeros(N ** 3)
    sens[act] = G[f"filt_{i}_sens"]
    p.put("sens", sens)
    p.filter(float(G[f"filt_{i}_radius"]))
    assert rel(p.get("sens")[act], G[f"filt_{i}_out"]) <= 1e-6
    p.close()


def _order4_cases():
    return {
        "cantilever16": workloads.cantilever(16, 8, 8, lattice=(7, 5, 5), order=4),
        "mbb32": workloads.half_mbb(32, 16, 16, lattice=(11, 7, 7), order=4),
        "cantilever48": workloads.cantilever(lattice=(13, 7, 7), order=4),
    }


@pytest.mark.parametrize("name", ["cantilever16", "mbb32", "cantilever48"])
def test_order4_density_adjoint_oc(oracle_mod, name):
    wl = _order4_cases()[name]
    assert wl.order == 4
    nc = int(np.prod([q + 4 for q in wl.partition]))
    coeff = random_coeff(nc, seed=21)
    g, o = setup_gpu(wl, coeff), setup_oracle(wl, coeff)
    assert rel(g.get("rho"), o.get("rho")) < 1e-12
    sens = -np.abs(np.random.default_rng(4).standard_normal(wl.nx * wl.ny * wl.nz))
    for p in (g, o):
        p.put("sens", sens)
        p.spline_adjoint()
    assert rel(g.get("csens"), o.get("csens")) < 1e-12
    for twice in (False, True):
        for p in (g, o):
            p.put("coeff", coeff)
            p.coeff_to_density()
        tg, lg = g.oc_update(0.3, apply_twice=twice)
        to, lo = o.oc_update(0.3, apply_twice=twice)
        assert tg == to and abs(lg - lo) <= 1e-12 * abs(lo)
        assert rel(g.get("coeff"), o.get("coeff")) < 1e-12
        assert rel(g.get("rho"), o.get("rho")) < 1e-12
    g.close()


def test_order4_design_iterations(oracle_mod):
    wl = _order4_cases()["cantilever16"]
    g, o = setup_gpu(wl), setup_oracle(wl)
    for _ in range(4):
        s = g.design_iteration(solve=dict(mode=capi.SOLVE_PCG64, rtol=1e-8, max_iter=300), oc=dict(vgoal=wl.vgoal))
        o.update_operators()
        o.pcg(2, 2, 1e-8, 300, 0)
        c = o.compliance()
        o.sensitivity(); o.filter(wl.filter_radius); o.spline_adjoint(); o.oc_update(wl.vgoal)
        assert abs(s["compliance"] - c) <= 1e-7 * abs(c)
    assert rel(g.get("coeff"), o.get("coeff")) < 1e-7
    g.close()


def test_config0_fifty_iterations(oracle_mod):
    """Config 0 in full: 48x24x24 cantilever (x = 0 fixed, total force 1 down on
    the bottom edge at x = 48), lattice 13x7x7, coefficients 0.4, filter radius 2,
    OC damp 0.5 / move 0.03 / Vf 0.4, FP64 MG-PCG to rel-res 1e-6 warm-started,
    50 design iterations on the GPU and on the oracle side by side.  Each
    iteration is compared on the same input: the oracle's coefficients and U are
    copied into the GPU before it, so every iteration's error is its own (not
    50 iterations of amplified round-off)."""
    wl = workloads.cantilever()
    g, o = setup_gpu(wl), setup_oracle(wl)
    worst_c, worst_coeff, trial_mismatch = 0.0, 0.0, 0
    comp = []
    for it in range(50):
        g.put("coeff", o.get("coeff"))
        g.coeff_to_density()
        g.put("u", o.get("u"))
        s = g.design_iteration(solve=dict(mode=capi.SOLVE_PCG64, rtol=1e-6, max_iter=300), oc=dict(vgoal=wl.vgoal))
        o.update_operators()
        o.pcg(2, 2, 1e-6, 300, 0)
        c = o.compliance()
        o.sensitivity(); o.filter(wl.filter_radius); o.spline_adjoint()
        trials, _ = o.oc_update(wl.vgoal)
        comp.append(c)
        worst_c = max(worst_c, abs(s["compliance"] - c) / abs(c))
        # both solves stop somewhere below rel-res 1e-6, so sensitivities differ
        # at that level; where the OC bisection then takes a different number
        # of trials (a volume within its 1e-4 tolerance either way) the
        # coefficients legitimately differ at the bracket's width
        if s["oc_trials"] == trials:
            worst_coeff = max(worst_coeff, rel(g.get("coeff"), o.get("coeff")))
        else:
            trial_mismatch += 1
    assert worst_c <= 1e-8, worst_c
    assert worst_coeff <= 1e-6, worst_coeff
    assert trial_mismatch <= 2, trial_mismatch
    # the design improves: compliance falls from the first to the last iteration
    assert comp[-1] < comp[0]
    g.close()
