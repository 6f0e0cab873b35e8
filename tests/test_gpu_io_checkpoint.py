"""Files and checkpoints on the GPU library: a handle made from the reference's
bit-mask domain equals one made from the element mask; raw records
(bio::write_vector, utils/binaryIO.h:70-108) and the FP32 coefficient file of
HierarchyGrid::writeCoeff (grid/Grid.cpp:2139-2156) round-trip; and a design
run resumed from a checkpoint repeats the uninterrupted run bit for bit (OC
and MMA)."""
import os

import numpy as np
import pytest

from tests.helpers import setup_gpu
from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def test_bitmask_handle_equals_mask_handle(tmp_path):
    nx, ny, nz = 37, 21, 13
    ea = workloads.perforated(nx, ny, nz, holes=6, radius=(2.0, 4.0), seed=5).astype(np.uint8)
    reso = (64, 32, 16)
    w = capi.eactive_to_bitmask(nx, ny, nz, ea, reso)
    a = capi.Problem(nx, ny, nz, eactive=ea)
    b = capi.Problem(nx, ny, nz, bitmask=(reso, w))
    assert a.num_levels() == b.num_levels()
    for l in range(a.num_levels()):
        assert np.array_equal(a.get("eactive", l), b.get("eactive", l))
        assert np.array_equal(a.get("vmask", l), b.get("vmask", l))
    a.close(); b.close()


def test_records_round_trip(tmp_path):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    wl.eactive = workloads.perforated(16, 8, 8, holes=2, radius=(1.5, 2.5), seed=1)
    p = setup_gpu(wl, coeff=np.random.default_rng(3).uniform(0.1, 0.9, 7 * 5 * 5))
    coeff = p.get("coeff")
    f32 = str(tmp_path / "coeff")
    p.write_array("coeff", f32, fp32=True)
    raw = np.fromfile(f32, dtype=np.float32)
    assert np.array_equal(raw, coeff.astype(np.float32))
    p.put("coeff", np.zeros_like(coeff))
    p.read_array("coeff", f32, fp32=True)
    assert np.array_equal(p.get("coeff"), raw.astype(np.float64))
    f64 = str(tmp_path / "rho64")
    p.write_array("rho", f64)
    assert np.array_equal(np.fromfile(f64, dtype=np.float64), p.get("rho"))
    with pytest.raises(capi.TopoError):
        p.read_array("u", f64)  # wrong size
    rec = str(tmp_path / "density.rec")
    n = p.write_active_records("rho", rec)
    r = np.fromfile(rec, dtype=np.float32).reshape(-1, 4)
    ea = p.get("eactive").astype(bool)
    assert n == ea.sum() == r.shape[0]
    x, y, z = (r[:, k].astype(int) for k in range(3))
    e = x + 16 * (y + 8 * z)
    assert ea[e].all()
    assert np.array_equal(r[:, 3], p.get("rho")[e].astype(np.float32))
    p.close()


SOLVE = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, pre=1, post=1, rtol=1e-6, max_iter=300,
             inner_max=4, inner_rtol=0.1, cheb_degree=2)


def _run(p, wl, n):
    out = []
    for _ in range(n):
        s = p.design_iteration(solve=SOLVE, oc=dict(vgoal=wl.vgoal))
        out.append((s["compliance"], s["iterations"], s["oc_trials"]))
    return out


@pytest.mark.parametrize("graphs", [True, False])
def test_resume_is_bit_exact(tmp_path, graphs):
    wl = workloads.half_mbb(32, 16, 16, lattice=(11, 7, 7))
    a = setup_gpu(wl)
    a.set_graphs(int(graphs))
    full = _run(a, wl, 6)
    ref_coeff, ref_u = a.get("coeff"), a.get("u")
    a.close()
    b = setup_gpu(wl)
    b.set_graphs(int(graphs))
    first = _run(b, wl, 3)
    ck = str(tmp_path / "run.ckpt")
    b.checkpoint_save(ck, user=b"iteration=3")
    b.close()
    c = setup_gpu(wl)
    c.set_graphs(int(graphs))
    c.put("coeff", np.zeros(c.num_coeffs()))
    assert c.checkpoint_load(ck) == b"iteration=3"
    rest = _run(c, wl, 3)
    assert first + rest == full
    assert np.array_equal(c.get("coeff"), ref_coeff)
    assert np.array_equal(c.get("u"), ref_u)
    c.close()


def test_checkpoint_refuses_another_grid(tmp_path):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    p = setup_gpu(wl)
    ck = str(tmp_path / "a.ckpt")
    p.checkpoint_save(ck)
    q = setup_gpu(workloads.cantilever(16, 8, 16, lattice=(7, 5, 7)))
    with pytest.raises(capi.TopoError):
        q.checkpoint_load(ck)
    p.close(); q.close()


def test_mma_resume_is_bit_exact(tmp_path):
    """The MMA design loop (testOrdinarySplineTopoptMMA) resumed from the
    handle's and the MMA's checkpoints repeats the uninterrupted run."""
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    solve = dict(mode=capi.SOLVE_PCG64, rtol=1e-8, max_iter=300)

    def steps(p, mma, n):
        out = []
        for _ in range(n):
            s = capi.mma_design_iteration(p, mma, wl.vgoal, solve=solve)
            out.append((s["compliance"], s["volume"], s["subiterations"]))
        return out

    def fresh():
        p = setup_gpu(wl)
        p.volume_csens(scale=1e3)
        return p, capi.MMA.for_problem(p, 1, lb=1e-3, ub=1.0)

    a, ma = fresh()
    full = steps(a, ma, 5)
    ref = ma.x
    b, mb = fresh()
    first = steps(b, mb, 2)
    ck, mk = str(tmp_path / "p.ckpt"), str(tmp_path / "m.ckpt")
    b.checkpoint_save(ck)
    mb.checkpoint_save(mk)
    c, mc = fresh()
    c.checkpoint_load(ck)
    mc.checkpoint_load(mk)
    rest = steps(c, mc, 3)
    assert first + rest == full
    assert np.array_equal(mc.x, ref)
    for o in (ma, mb, mc):
        o.close()
    for p in (a, b, c):
        p.close()
