"""CTA tile heights of the FP32 modal fine kernels (topo_set_fine_tile_rows):
tiles of 4, 8 and 16 element rows, marched in z, through the C ABI.  Every
vertex sum is formed in the same order whatever the tile height, so the FP32
operator is the same bit for bit across heights and within the FP32 kernels'
1e-5 relative of the CPU FP64 oracle; mixed solves (whose dot products are
summed per CTA, so in another order) reach rel-res 1e-6 and compliance within
1e-6 of the oracle's solve to 1e-10."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import setup_gpu, setup_oracle, rel, random_masked_u, random_coeff

pytestmark = pytest.mark.gpu


def _cases():
    c = dict(workloads.small_cases())
    # a y extent that is no multiple of 3, 7 or 15 owned rows, several CTAs along x
    c["mbb96"] = workloads.half_mbb(96, 50, 40, lattice=(25, 13, 11))
    masked = workloads.cantilever(37, 21, 13, lattice=(9, 6, 5))
    masked.eactive = workloads.perforated(37, 21, 13, holes=6, radius=(2.0, 4.0), seed=5)
    c["perforated37"] = masked
    return c


CASES = ["cantilever16", "mbb32", "cantilever48", "mbb96", "perforated37"]


@pytest.fixture(params=CASES)
def pair(request, oracle_mod):
    wl = _cases()[request.param]
    nc = int(np.prod([p + wl.order for p in wl.partition]))
    coeff = random_coeff(nc, seed=12)
    return wl, setup_gpu(wl, coeff), setup_oracle(wl, coeff)


@pytest.mark.parametrize("tz", [4, 8, 16])
def test_fp32_operator_same_across_tile_heights(pair, tz):
    wl, g, o = pair
    u = random_masked_u(wl.nv, o.get("vmask"), 6)
    o.update_penalised()
    y_o = o.apply_fine(u)
    g.set_tiles(tz, 16)
    ys = {}
    for rows in (8, 4, 16):
        g.set_fine_tile_rows(rows)
        ys[rows] = g.apply_fine(u, 1)
    g.set_fine_tile_rows(8)
    assert rel(ys[8], y_o) < 1e-5
    assert np.array_equal(ys[4], ys[8])
    assert np.array_equal(ys[16], ys[8])


@pytest.mark.parametrize("smoother", [capi.SMOOTH_CHEBYSHEV, capi.SMOOTH_GS])
@pytest.mark.parametrize("rows", [4, 16])
def test_mixed_solve_with_tile_height(pair, rows, smoother):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    u0 = g.get("u")
    st_8 = g.solve(mode=capi.SOLVE_MIXED, smoother=smoother, rtol=1e-6, max_iter=400, inner_max=4)
    g.put("u", u0)
    g.set_fine_tile_rows(rows)
    st_r = g.solve(mode=capi.SOLVE_MIXED, smoother=smoother, rtol=1e-6, max_iter=400, inner_max=4)
    c_r = g.compliance()
    g.set_fine_tile_rows(8)
    o.pcg(2, 2, 1e-10, 400, 0)
    c_o = o.compliance()
    assert st_r["relres"] <= 1e-6
    assert abs(c_r - c_o) < 1e-6 * abs(c_o)
    assert abs(st_r["iterations"] - st_8["iterations"]) <= 1


def test_rejects_other_heights(oracle_mod):
    g = setup_gpu(workloads.small_cases()["cantilever16"])
    for rows in (0, 2, 6, 12, 32):
        with pytest.raises(capi.TopoError):
            g.set_fine_tile_rows(rows)


def test_checkpoint_keeps_tile_height(tmp_path, oracle_mod):
    """A checkpoint carries the tile height with the z-march depths and the
    tensor-core choice: a handle resumed from it launches the same tiles (the
    graph cache keys on them) and gives the same design iterations bit for bit."""
    wl = workloads.half_mbb(64, 32, 32, lattice=(17, 9, 9))
    opts = dict(solve=dict(mode=capi.SOLVE_MIXED, rtol=1e-6, max_iter=300, inner_max=4), oc=dict(vgoal=0.4))
    g = setup_gpu(wl)
    g.set_fine_tile_rows(16)
    g.design_iteration(**opts)
    path = str(tmp_path / "rows.ckpt")
    g.checkpoint_save(path)
    ref = [g.design_iteration(**opts)["compliance"] for _ in range(2)]
    g2 = setup_gpu(wl)
    g2.checkpoint_load(path)
    got = [g2.design_iteration(**opts)["compliance"] for _ in range(2)]
    assert got == ref
