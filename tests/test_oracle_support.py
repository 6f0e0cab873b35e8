"""The restated constraint derivatives (oracle/support_oracle.py) against
finite differences of the restated values, points held fixed: self-support
modes 2-5 (the mean of the point values) and drip modes 6/7 of both versions,
on seeded spline designs of a small cantilever.  The reference's own
derivative formulas are what the oracle restates; this pins them to the
values they differentiate (without the reference's drip-gradient slips, which
the oracle reproduces behind reference_quirks)."""
import numpy as np
import pytest

from oracle import support_oracle as so
from tests.helpers import setup_oracle
from topoptspline3d_gb300 import workloads


def _design(seed=3):
    wl = workloads.cantilever(12, 6, 6, lattice=(6, 5, 5))
    nc = int(np.prod([q + wl.order for q in wl.partition]))
    coeff = np.random.default_rng(seed).uniform(0.15, 0.85, nc)
    o = setup_oracle(wl, coeff)
    bmin, bmax = wl.spline_box()
    spl = so.Spline(o, wl.order, wl.partition, bmin, bmax, coeff)
    count, pts = so.surface_points(o, spl, (wl.nx, wl.ny, wl.nz), 1.0, o.get("eactive"), 10, 400)
    return wl, spl, coeff, pts, count


@pytest.mark.parametrize("opts", [
    dict(ss_mode=2, drip_mode=6, drip_version=0, print_angle=0.75, hfunction_c=10.0),
    dict(ss_mode=3, drip_mode=7, drip_version=1, print_angle=0.7),
    dict(ss_mode=4, drip_mode=6, drip_version=1, print_angle=0.75),
    dict(ss_mode=5, drip_mode=7, drip_version=0, print_angle=0.8, drip_beta=8.0, drip_mu=4.0, drip_beta_scale=1.0),
])
def test_gradients_match_finite_differences(oracle_mod, opts):
    wl, spl, coeff, pts, count = _design()
    assert count > 50 and len(pts) > 50
    nc = coeff.size
    base = so.constraints(spl, pts, opts, 4.0, nc)
    rng = np.random.default_rng(1)
    for _ in range(3):
        d = rng.standard_normal(nc)
        eps = 1e-6
        vals = []
        for sgn in (1, -1):
            s2 = so.Spline.__new__(so.Spline)
            s2.__dict__.update(spl.__dict__)
            s2.c = coeff + sgn * eps * d
            r = so.constraints(s2, pts, opts, 4.0, nc)
            assert r["flipped"] == base["flipped"] and r["down"] == base["down"]
            vals.append((r["ss"], r["drip"]))
        fd_ss = (vals[0][0] - vals[1][0]) / (2 * eps)
        fd_drip = (vals[0][1] - vals[1][1]) / (2 * eps)
        # central differences: truncation ~ eps^2, round-off ~ 1e-16 |value| / eps
        tol_ss = 1e-5 * abs(fd_ss) + 1e-9 * (1 + abs(base["ss"]))
        tol_drip = 1e-5 * abs(fd_drip) + 1e-9 * (1 + abs(base["drip"]))
        assert abs(fd_ss - base["gss"] @ d) <= tol_ss, (fd_ss, base["gss"] @ d)
        assert abs(fd_drip - base["gdrip"] @ d) <= tol_drip, (fd_drip, base["gdrip"] @ d)


def test_projection_derivative():
    s = np.linspace(0, 1, 101)
    for beta in (1.0, 4.0, 16.0):
        fd = (so.heaviside(s + 1e-7, beta) - so.heaviside(s - 1e-7, beta)) / 2e-7
        assert np.abs(fd - so.dirac(s, beta)).max() <= 1e-6 * beta
        assert abs(so.heaviside(0.0, beta)) < 1e-15 and abs(so.heaviside(1.0, beta) - 1) < 1e-15
