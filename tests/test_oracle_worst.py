"""The reference's modified power method for the worst-case load
(optimization/optimization.cpp:213-351), restated on the CPU oracle, against
the exact worst case: the largest eigenpair of M = S^T K^-1 S built column by
column.  The reference stops at a 1e-4 change of the load with rel-res 1e-2, so
it reaches the largest eigenvalue to about 1e-3."""
import numpy as np
import pytest

from oracle import worst_oracle
from tests.helpers import setup_oracle
from topoptspline3d_gb300 import workloads


def end_face(nx, ny, nz):
    """Vertex ids of the x = nx face and their outward normal +x."""
    vid = np.array([nx + (nx + 1) * (y + (ny + 1) * z) for z in range(nz + 1) for y in range(ny + 1)])
    return vid, np.tile([1.0, 0.0, 0.0], (len(vid), 1))


@pytest.mark.parametrize("free", [False, True])
def test_modified_pm_reaches_largest_eigenvalue(oracle_mod, free):
    # a 16x10x6 cantilever: two multigrid levels (the method's V-cycle needs a
    # coarse level to converge), a rectangular section so the leading load is
    # unique (a square section gives two equal bending modes)
    wl = workloads.cantilever(16, 10, 6, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    o.update_operators()
    vid, nrm = end_face(16, 10, 6)
    lam, vec, w = worst_oracle.dense_worst(o, vid, nrm, free)
    assert w[1] < 0.95 * lam
    assert lam > 0 and w[0] == lam
    c, x, its = worst_oracle.modified_pm(o, vid, nrm, seed=3, free_direction=free)
    assert its < 500
    assert abs(c - lam) <= 1e-3 * lam, (c, lam)
    assert abs(abs(np.dot(x, vec)) - 1.0) <= 1e-3


def test_dense_worst_is_a_maximum(oracle_mod):
    """No admissible unit load does better than the eigenvector (seeded probes)."""
    wl = workloads.cantilever(8, 4, 4, lattice=(5, 4, 4))
    o = setup_oracle(wl)
    o.update_operators()
    vid, nrm = end_face(8, 4, 4)
    lam, vec, _ = worst_oracle.dense_worst(o, vid, nrm, False)
    rng = np.random.default_rng(0)
    for _ in range(5):
        x = vec + 0.3 * rng.standard_normal(vec.size)
        x /= np.linalg.norm(x)
        f = worst_oracle.scatter(o, vid, nrm, x, False)
        o.put("f", f)
        o.put("u", np.zeros_like(f))
        o.pcg(2, 2, 1e-11, 500, 0)
        assert np.dot(f, o.get("u")) <= lam * (1 + 1e-9)
