"""CPU tests of the C-ABI library: it loads, exports every declared symbol, and its
host-side set-up (element template, level plan, spline tables, reference GS
ordering) agrees with the oracle.  No kernel runs here."""
import ctypes
import os
import re

import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "topo_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(topo_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    syms = declared_symbols()
    assert len(syms) >= 40
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(capi.EXPORTED) == syms


def test_element_template_matches_oracle(oracle_mod):
    for E, nu, h in [(1e6, 0.4, 1.0), (2.5, 0.3, 0.37), (210e9, 0.25, 2.0)]:
        K_lib = capi.element_template(E, nu, h)
        K_orc = oracle_mod.ke_template(E, nu, h)
        assert np.abs(K_lib - K_orc).max() <= 1e-12 * np.abs(K_orc).max()


@pytest.mark.parametrize("dims", [(48, 24, 24), (256, 128, 128), (37, 21, 9), (7, 5, 3), (16, 8, 8)])
def test_level_plan_matches_oracle(oracle_mod, dims):
    nx, ny, nz = dims
    d_lib, f_lib = capi.plan_levels(nx, ny, nz)
    if nx * ny * nz <= 8 * 10 ** 6 and nx * ny * nz < 300000:
        o = oracle_mod.Oracle(nx, ny, nz)
        assert [tuple(o.level_dims(l)) for l in range(o.num_levels())] == [tuple(int(v) for v in d) for d in d_lib]
        assert [o.level_factor(l) for l in range(o.num_levels())] == [int(v) for v in f_lib]
    if dims == (256, 128, 128):
        assert [tuple(int(v) for v in d) for d in d_lib] == [(256, 128, 128), (64, 32, 32), (32, 16, 16), (16, 8, 8), (8, 4, 4)]
    if dims == (48, 24, 24):
        assert [tuple(int(v) for v in d) for d in d_lib] == [(48, 24, 24), (12, 6, 6), (6, 3, 3)]


def test_level_plan_masked_domain(oracle_mod):
    mask = workloads.ellipsoid_union(40, 24, 20, n=4, seed=7, axes=(4, 12))
    d_lib, f_lib = capi.plan_levels(40, 24, 20, mask)
    o = oracle_mod.Oracle(40, 24, 20, eactive=mask)
    assert [tuple(o.level_dims(l)) for l in range(o.num_levels())] == [tuple(int(v) for v in d) for d in d_lib]


@pytest.mark.parametrize("order,part,n", [(3, 10, 48), (3, 4, 24), (3, 62, 256), (4, 9, 48), (2, 12, 48)])
def test_spline_tables_match_oracle(oracle_mod, order, part, n):
    knots, i0, N = capi.spline_axis(order, part, 0.0, float(n), n)
    o = oracle_mod.Oracle(n, 4, 4)
    o.set_spline(order, (part, 1, 1), (0, 0, 0), (n, 4, 4))
    assert np.array_equal(knots, o.knots(0, order, part))
    inside = i0 >= 0
    assert inside.all()
    # partition of unity and non-negativity of the basis values
    assert np.abs(N.sum(1) - 1.0).max() < 1e-12 and (N >= -1e-15).all()
    # coefficient = i0 + r reproduces the index: the density of c_i = i equals sum_r (i0+r) N_r
    coef = np.arange(order + part, dtype=float)
    o.put("coeff", np.tile(coef, (order + 1) * (order + 1)).ravel()[: o.num_coeffs()] if False else
          np.broadcast_to(coef[None, None, :], (order + 1, order + 1, order + part)).ravel())
    o.coeff_to_density()
    rho_o = o.get("rho").reshape(4, 4, n)[0, 0]
    rho_l = np.clip((N * (i0[:, None] + np.arange(order))).sum(1), 1e-3, 1.0)
    assert np.abs(rho_o - rho_l).max() < 1e-12


@pytest.mark.parametrize("dims,masked", [((5, 3, 2), False), ((16, 8, 8), False), ((40, 24, 20), True)])
def test_reference_gs_maps_match_oracle(oracle_mod, dims, masked):
    nx, ny, nz = dims
    mask = workloads.ellipsoid_union(nx, ny, nz, n=4, seed=7, axes=(4, 12)) if masked else None
    o = oracle_mod.Oracle(nx, ny, nz, eactive=mask)
    for level in range(o.num_levels()):
        vid_o, eid_o, gsn_o, ngv_o, nge_o = o.gs_maps(level)
        vid, eid, gsn, ngv, nge = capi.plan_gs_maps(nx, ny, nz, level, mask)
        assert np.array_equal(vid, vid_o) and np.array_equal(eid, eid_o)
        assert np.array_equal(gsn, gsn_o) and ngv == ngv_o and nge == nge_o


def test_bad_inputs_return_status_without_gpu():
    lib = capi.load()
    out = np.zeros(576)
    assert lib.topo_element_template(1.0, 0.5, 1.0, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == capi.TOPO_E_BAD_INPUT
    n = ctypes.c_int()
    assert lib.topo_plan_levels(0, 1, 1, None, 400, 16, ctypes.byref(n), None, None) == capi.TOPO_E_BAD_INPUT
    assert lib.topo_create(None, None, None) == capi.TOPO_E_BAD_INPUT
