"""FP32 fine kernels with the element products on the tcgen05 tensor cores
(three-term TF32, fp32 accumulators in tensor memory) against the CPU FP64
oracle and against the modal FP32 kernels on the same inputs, through the C
ABI.  Tolerances as for the FP32 kernels: 1e-5 relative per operation, and the
mixed solve 1e-6 on compliance against the oracle's solve to 1e-10."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads
from tests.helpers import setup_gpu, setup_oracle, rel, random_masked_u, random_coeff

pytestmark = pytest.mark.gpu


def _cases():
    c = dict(workloads.small_cases())
    # several CTAs along x (30 owned vertex columns per CTA) and an uneven last z block
    c["mbb96"] = workloads.half_mbb(96, 48, 40, lattice=(25, 13, 11))
    masked = workloads.cantilever(37, 21, 13, lattice=(9, 6, 5))
    masked.eactive = workloads.perforated(37, 21, 13, holes=6, radius=(2.0, 4.0), seed=5)
    c["perforated37"] = masked
    return c


CASES = ["cantilever16", "mbb32", "cantilever48", "mbb96", "perforated37"]


@pytest.fixture(params=CASES)
def pair(request, oracle_mod):
    wl = _cases()[request.param]
    nc = int(np.prod([p + wl.order for p in wl.partition]))
    coeff = random_coeff(nc, seed=11)
    return wl, setup_gpu(wl, coeff), setup_oracle(wl, coeff)


@pytest.mark.parametrize("tz", [4, 8, 16])
def test_fp32_operator_on_tensor_cores(pair, tz):
    wl, g, o = pair
    u = random_masked_u(wl.nv, o.get("vmask"), 5)
    o.update_penalised()
    y_o = o.apply_fine(u)
    g.set_tiles(tz, 16)
    y_modal = g.apply_fine(u, 1)
    g.set_fine_tensor_cores(1)
    y_tc = g.apply_fine(u, 1)
    g.set_fine_tensor_cores(0)
    assert rel(y_tc, y_o) < 1e-5
    assert rel(y_modal, y_o) < 1e-5
    # a different kernel ran: the products are summed in another order
    assert not np.array_equal(y_tc, y_modal)
    assert np.abs(y_tc - y_modal).max() <= 1e-5 * np.abs(y_o).max()


@pytest.mark.parametrize("smoother", [capi.SMOOTH_CHEBYSHEV, capi.SMOOTH_GS])
def test_mixed_solve_on_tensor_cores(pair, smoother):
    wl, g, o = pair
    g.update_operators()
    o.update_operators()
    u0 = g.get("u")
    st_m = g.solve(mode=capi.SOLVE_MIXED, smoother=smoother, rtol=1e-6, max_iter=400, inner_max=4)
    c_m = g.compliance()
    g.put("u", u0)
    g.set_fine_tensor_cores(1)
    st_t = g.solve(mode=capi.SOLVE_MIXED, smoother=smoother, rtol=1e-6, max_iter=400, inner_max=4)
    c_t = g.compliance()
    g.set_fine_tensor_cores(0)
    o.pcg(2, 2, 1e-10, 400, 0)
    c_o = o.compliance()
    assert st_t["relres"] <= 1e-6
    assert abs(c_t - c_o) < 1e-6 * abs(c_o)
    assert abs(c_m - c_o) < 1e-6 * abs(c_o)
    # the same preconditioner up to FP32 rounding: iteration counts agree closely
    assert abs(st_t["iterations"] - st_m["iterations"]) <= 1
    assert abs(st_t["vcycles"] - st_m["vcycles"]) <= max(2, st_m["vcycles"] // 10)


def test_design_iterations_deterministic_on_tensor_cores(oracle_mod):
    wl = workloads.half_mbb(64, 32, 32, lattice=(17, 9, 9))
    runs = []
    for _ in range(2):
        g = setup_gpu(wl)
        g.set_fine_tensor_cores(1)
        s = [g.design_iteration(solve=dict(mode=capi.SOLVE_MIXED, rtol=1e-6, max_iter=300, inner_max=6),
                                oc=dict(vgoal=0.4)) for _ in range(3)]
        runs.append((np.array([x["compliance"] for x in s]), g.get("coeff")))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


def test_multi_rhs_on_tensor_cores(oracle_mod):
    wl = workloads.cantilever(32, 16, 16, lattice=(9, 5, 5))
    rng = np.random.default_rng(3)
    g = setup_gpu(wl)
    g.update_operators()
    nv = g.nv
    F = np.zeros((4, 3 * nv))
    vm = g.get("vmask")
    for k in range(4):
        f = rng.standard_normal((3, nv)) * 1e-3
        for c in range(3):
            f[c] *= ((vm >> c) & 1) & ((vm >> 3) & 1)
        F[k] = f.ravel()
    g.multi_reserve(4)
    U_m, st_m, _ = g.solve_multi(F, rtol=1e-6)
    g.set_fine_tensor_cores(1)
    U_t, st_t, rel_t = g.solve_multi(F, rtol=1e-6)
    g.set_fine_tensor_cores(0)
    assert st_t["max_relres"] <= 1e-6 and np.all(rel_t <= 1e-6)
    for k in range(4):
        assert rel(U_t[k], U_m[k]) < 1e-5


def test_checkpoint_keeps_tensor_core_choice(tmp_path, oracle_mod):
    """A checkpoint carries the FP32 element-product choice with the z-march
    depths: a handle resumed from it runs the same kernel bit for bit."""
    wl = workloads.half_mbb(64, 32, 32, lattice=(17, 9, 9))
    u = random_masked_u(wl.nv, setup_oracle(wl).get("vmask"), 9)
    g = setup_gpu(wl)
    g.set_tiles(8, 16)
    g.set_fine_tensor_cores(1)
    y_tc = g.apply_fine(u, 1)
    path = str(tmp_path / "tc.ckpt")
    g.checkpoint_save(path)
    g2 = setup_gpu(wl)
    y_modal = g2.apply_fine(u, 1)
    g2.checkpoint_load(path)
    y_resumed = g2.apply_fine(u, 1)
    assert np.array_equal(y_resumed, y_tc)
    assert not np.array_equal(y_modal, y_tc)
