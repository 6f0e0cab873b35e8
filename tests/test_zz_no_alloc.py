"""The allocation-free spline adjoint (topo_spline_adjoint_noalloc) against the
regular entry point.

topo_spline_adjoint_noalloc is for callers that must not allocate device memory
when they ask for a gradient (a fixed memory budget, a loop that must stay out
of the CUDA allocator, memory owned by another component).  It keeps its
intermediate planes in one fixed device array, so these tests check that two
calls in a row, each with its own input, reproduce topo_spline_adjoint, and that
a problem larger than the fixed array is refused rather than run.
"""
import ctypes as C

import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import setup_gpu, random_coeff

pytestmark = pytest.mark.gpu


def _adjoint_both(p, sens, nc):
    """Regular adjoint of `sens`, then the allocation-free one into the WORK buffer."""
    p.put("sens", sens)
    p.spline_adjoint()
    ref = p.get("csens")
    rc = p.lib.topo_spline_adjoint_noalloc(p.h, C.c_void_p(p.device_ptr("sens")), C.c_void_p(p.device_ptr("work")))
    assert rc == capi.TOPO_OK, p.lib.topo_last_error(p.h).decode()
    p.sync()
    out = p.get("work")[:nc]
    return ref, out


def test_noalloc_adjoint_matches_regular_twice():
    wl = workloads.small_cases()["mbb32"]
    p = setup_gpu(wl, random_coeff(11 * 7 * 7, seed=3))
    p.update_operators()
    p.solve(mode=capi.SOLVE_PCG64, rtol=1e-6, max_iter=200)
    p.sensitivity()
    p.filter(2.0)
    nc = p.num_coeffs()
    s1 = p.get("sens")
    rng = np.random.default_rng(9)
    s2 = s1 * rng.uniform(0.5, 2.0, s1.size) - 1e-3 * np.abs(s1).max()
    ref1, out1 = _adjoint_both(p, s1, nc)
    ref2, out2 = _adjoint_both(p, s2, nc)
    for ref, out in ((ref1, out1), (ref2, out2)):
        assert np.linalg.norm(out - ref) <= 1e-13 * np.linalg.norm(ref)
    assert np.linalg.norm(out2 - out1) > 1e-3 * np.linalg.norm(out1)


def test_noalloc_adjoint_refuses_oversized_problem():
    wl = workloads.cantilever(8, 64, 64, lattice=(603, 4, 4))
    p = setup_gpu(wl)
    rc = p.lib.topo_spline_adjoint_noalloc(p.h, C.c_void_p(p.device_ptr("sens")), C.c_void_p(p.device_ptr("work")))
    assert rc == capi.TOPO_E_BAD_INPUT
    assert "scratch" in p.lib.topo_last_error(p.h).decode()
