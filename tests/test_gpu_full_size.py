"""The design trajectory at the bench's full size: 256x128x128 half-MBB beam
(12.8 M DOFs, lattice 65x33x33), the GPU against the FP64 oracle for three
design iterations.  Each iteration starts both sides from the oracle's
coefficients and U, so each iteration's error is its own.  The plain FP64
MG-PCG solve matches the oracle's compliance to 1e-8 and its coefficients to
1e-6; the mixed solve (FP32 multigrid under FP64 flexible CG) matches the
compliance to 1e-6, the tolerance the mixed solve is held to."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import rel, setup_gpu, setup_oracle

pytestmark = pytest.mark.gpu


def test_half_mbb_256_trajectory(oracle_mod):
    wl = workloads.half_mbb()
    g, o = setup_gpu(wl), setup_oracle(wl)
    mixed = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-6, max_iter=300, inner_max=6,
                 inner_rtol=0.1, pre=1, post=1, cheb_lo=0.1)
    plain = dict(mode=capi.SOLVE_PCG64, smoother=capi.SMOOTH_GS, rtol=1e-6, max_iter=300)
    for it in range(3):
        start_coeff, start_u = o.get("coeff"), o.get("u")
        o.update_operators()
        it_o, rr_o = o.pcg(2, 2, 1e-6, 300, 0)
        c = o.compliance()
        o.sensitivity(); o.filter(wl.filter_radius); o.spline_adjoint()
        trials, _ = o.oc_update(wl.vgoal)
        for opts, tol in ((plain, 1e-8), (mixed, 1e-6)):
            g.put("coeff", start_coeff)
            g.coeff_to_density()
            g.put("u", start_u)
            s = g.design_iteration(solve=opts, oc=dict(vgoal=wl.vgoal), filter_radius=wl.filter_radius)
            assert s["relres"] <= 1e-6
            err = abs(s["compliance"] - c) / abs(c)
            print(f"iteration {it} {'PCG64' if opts is plain else 'mixed'}: compliance rel. error {err:.2e}, "
                  f"{s['iterations']} iterations (oracle {it_o})")
            assert err <= tol, (it, opts["mode"], err)
            if opts is plain and s["oc_trials"] == trials:
                assert rel(g.get("coeff"), o.get("coeff")) < 1e-6
    g.close()
