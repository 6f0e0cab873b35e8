"""Fine kernels on a domain with void: the z march of each fine tile covers only
the vertex planes next to its active elements, and the planes cut away get the
operator's output for zero forces.  On a union-of-ellipsoids domain (tiles that
are entirely void, tiles active over part of their height) every form of the
fine operator, the Chebyshev smoother inside the mixed solve, and the element
energies of the sensitivity are checked against the FP64 oracle, which has no
such skip."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import setup_gpu, setup_oracle, rel, random_masked_u

pytestmark = pytest.mark.gpu

NX, NY, NZ = 64, 40, 48


def _tile_zranges(ea, nx, ny, nz, tx=32, ty=8):
    """Active element z range per fine tile (31 x 7 owned vertex columns and the
    element columns around them), or None for a void tile."""
    e3 = ea.reshape(nz, ny, nx).astype(bool)
    out = []
    for by in range((ny + 1 + ty - 2) // (ty - 1)):
        for bx in range((nx + 1 + tx - 2) // (tx - 1)):
            x0, y0 = bx * (tx - 1), by * (ty - 1)
            box = e3[:, max(0, y0 - 1):y0 + ty - 1, max(0, x0 - 1):x0 + tx - 1]
            zs = np.flatnonzero(box.any(axis=(1, 2)))
            out.append((zs.min(), zs.max()) if zs.size else None)
    return out


@pytest.fixture(scope="module")
def pair(oracle_mod):
    wl = workloads.large_ellipsoids(NX, NY, NZ, nloads=4)
    zr = _tile_zranges(wl.eactive, NX, NY, NZ)
    # the case exercises both kinds of cut: void tiles, and partly active ones
    assert any(r is None for r in zr)
    assert any(r is not None and (r[0] > 0 or r[1] < NZ - 1) for r in zr)
    return wl, setup_gpu(wl), setup_oracle(wl)


def test_fine_operator_forms(pair):
    wl, g, o = pair
    u = random_masked_u(wl.nv, o.get("vmask"), 3)
    o.update_penalised()
    y_o = o.apply_fine(u)
    assert rel(g.apply_fine(u, 0), y_o) < 1e-12  # modal FP64
    assert rel(g.apply_fine(u, 2), y_o) < 1e-12  # dense-row FP64 (no tiles)
    assert rel(g.apply_fine(u, 3), y_o) < 1e-12  # double-float
    assert rel(g.apply_fine(u, 1), y_o) < 1e-5   # FP32
    for tz in (4, 8, 32):  # z blocks that start and end inside and outside the active range
        g.set_tiles(tz, tz)
        assert rel(g.apply_fine(u, 0), y_o) < 1e-12, tz
        assert rel(g.apply_fine(u, 3), y_o) < 1e-12, tz
        assert rel(g.apply_fine(u, 1), y_o) < 1e-5, tz
    g.set_tiles(16, 16)


@pytest.mark.parametrize("mode", [capi.SOLVE_PCG64, capi.SOLVE_MIXED])
def test_chebyshev_solves(pair, mode):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    g.put("u", np.zeros(3 * wl.nv))
    st = g.solve(mode=mode, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-8, max_iter=400)
    assert st["relres"] <= 1e-8
    o.put("u", np.zeros(3 * wl.nv))
    o.pcg(2, 2, 1e-10, 400, 0)
    assert abs(g.compliance() - o.compliance()) < 1e-7 * abs(o.compliance())


def test_design_iterations_element_energies(oracle_mod):
    """Design iterations take the sensitivity from the element energies of the
    final double-float residual launch; void layers must read zero there."""
    wl = workloads.large_ellipsoids(NX, NY, NZ, nloads=4)
    g, o = setup_gpu(wl), setup_oracle(wl)
    for it in range(2):
        s = g.design_iteration(solve=dict(mode=capi.SOLVE_PCG64, smoother=capi.SMOOTH_CHEBYSHEV, rtol=1e-9,
                                          max_iter=400), oc=dict(vgoal=wl.vgoal),
                               filter_radius=wl.filter_radius)
        o.update_operators()
        o.pcg(2, 2, 1e-10, 400, 0)
        assert abs(s["compliance"] - o.compliance()) < 1e-7 * abs(o.compliance()), it
        o.sensitivity(); o.filter(wl.filter_radius); o.spline_adjoint(); o.oc_update(wl.vgoal)
    assert rel(g.get("coeff"), o.get("coeff")) < 1e-6


def test_tensor_core_choice_keeps_void_skipping(pair):
    """On a level with void planes the FP32 kernels keep the modal element
    products in 8-row tiles (the tensor-core kernel's tiles and the other tile
    heights do not carry the per-tile z ranges):
    with the tensor-core choice set, the FP32 operator is the modal one bit for
    bit, and still the oracle's to 1e-5."""
    wl, g, o = pair
    u = random_masked_u(wl.nv, o.get("vmask"), 4)
    o.update_penalised()
    y_o = o.apply_fine(u)
    y_modal = g.apply_fine(u, 1)
    g.set_fine_tensor_cores(1)
    y_tc = g.apply_fine(u, 1)
    g.set_fine_tensor_cores(0)
    assert np.array_equal(y_tc, y_modal)
    assert rel(y_tc, y_o) < 1e-5
    # likewise the tile heights: the void-skipping kernel keeps its 8-row tiles
    for rows in (4, 16):
        g.set_fine_tile_rows(rows)
        assert np.array_equal(g.apply_fine(u, 1), y_modal)
    g.set_fine_tile_rows(8)
