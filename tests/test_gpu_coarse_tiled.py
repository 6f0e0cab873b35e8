"""The FP32 level-1 stencil kernels on a grid whose first coarse level uses
the tiled FP32 stencil layout (at least 32,768 vertices; the small parity cases
never reach it), against the FP64 stencil kernels on the same level and input,
through the C ABI (topo_apply_level).  Tolerances: 1e-5 relative for the FP32
operator, 1e-6 on the mixed solve's compliance against the FP64 MG-PCG."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import setup_gpu, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big():
    # level 1 of 256x96x96 is 65 x 25 x 25 = 40,625 vertices: tiled FP32 stencil
    wl = workloads.half_mbb(256, 96, 96, lattice=(65, 25, 25))
    g = setup_gpu(wl)
    g.set_operator_precision(3)
    g.update_operators()
    return wl, g


def test_level1_is_tiled(big):
    _, g = big
    (ex, ey, ez), fct = g.level_dims(1)
    assert fct == 4 and (ex + 1) * (ey + 1) * (ez + 1) >= 32768


@pytest.mark.parametrize("seed", [1, 2])
def test_fp32_level_operator_matches_fp64(big, seed):
    _, g = big
    vm = g.get("vmask", 1)
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((3, vm.size))
    for c in range(3):
        u[c] *= ((vm >> c) & 1) & ((vm >> 3) & 1)
    y64 = g.apply_level(1, u.ravel(), 0)
    y32 = g.apply_level(1, u.ravel(), 1)
    assert np.abs(y64).max() > 0
    assert rel(y32, y64) < 1e-5


def test_mixed_solve_with_tiled_stencils(big):
    _, g = big
    u0 = g.get("u")
    st = g.solve(mode=capi.SOLVE_PCG64, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-8, max_iter=300)
    c64 = g.compliance()
    g.put("u", u0)
    st = g.solve(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-6, max_iter=300, inner_max=6,
                 cheb_degree=4, cheb_lo=0.05, inner_rtol=0.03)
    assert st["relres"] <= 1e-6
    assert abs(g.compliance() - c64) <= 1e-6 * abs(c64)
    assert st["iterations"] <= 8
