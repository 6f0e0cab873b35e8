"""The oracle (and the library's host-side spline tables) against golden vectors
computed by the reference's own code: its knot series (grid/Grid.cpp:3253-3337),
Cox-de Boor basis (grid/Grid.cu:384-466), coeff2density (grid/Grid.cu:3325-3436),
spline-adjoint scatter (grid/Grid.cu:3643-3724) and sensitivity filter
(grid/Grid.cu:4130-4246), built as host code by oracle/ref_build.py and run by
tests/golden/make_ref_golden.py.  The reference works in FP32, the oracle in
FP64 from the same FP32 knots, so values agree to FP32 rounding and the knots
bit for bit."""
import numpy as np
import pytest

from tests import golden
from tests.helpers import rel
from topoptspline3d_gb300 import capi

G = golden.load()
N = int(G["cube"])


def _cube_oracle(oracle_mod, mask, order, part):
    o = oracle_mod.Oracle(N, N, N, eactive=mask)
    o.set_spline(order, part, (0.0, 0.0, 0.0), (float(N),) * 3)
    return o


@pytest.mark.parametrize("i", range(int(G["n_knots"])))
def test_knots_bit_exact(oracle_mod, i):
    order, part, box = int(G[f"knots_{i}_order"]), G[f"knots_{i}_part"], G[f"knots_{i}_box"]
    ref = G[f"knots_{i}_knots"]
    o = oracle_mod.Oracle(4, 4, 4)
    o.set_spline(order, [int(p) for p in part], box[:3], box[3:])
    off = 0
    for a in range(3):
        n = 2 * order + int(part[a])
        ko = o.knots(a, order, int(part[a]))
        assert np.array_equal(ko.astype(np.float32), ref[off:off + n]), (a, ko, ref[off:off + n])
        kl, _, _ = capi.spline_axis(order, int(part[a]), box[a], box[3 + a], 1, 1.0)
        assert np.array_equal(np.asarray(kl).astype(np.float32), ref[off:off + n])
        off += n


@pytest.mark.parametrize("i", range(int(G["n_knots"])))
def test_basis(oracle_mod, i):
    order, part, box = int(G[f"knots_{i}_order"]), G[f"knots_{i}_part"], G[f"knots_{i}_box"]
    o = oracle_mod.Oracle(4, 4, 4)
    o.set_spline(order, [int(p) for p in part], box[:3], box[3:])
    xs, Nref = G[f"basis_{i}_x"], G[f"basis_{i}_N"]
    for k in range(xs.shape[0]):
        for a in range(3):
            i0, nb = o.basis(a, float(xs[k, a]), order)
            assert i0 >= 0
            assert np.abs(nb - Nref[k, a]).max() <= 2e-6, (k, a, nb, Nref[k, a])
            assert abs(nb.sum() - 1.0) <= 1e-12


@pytest.mark.parametrize("i", range(int(G["n_dens"])))
def test_density_and_adjoint(oracle_mod, i):
    order, part = int(G[f"dens_{i}_order"]), [int(p) for p in G[f"dens_{i}_part"]]
    mask = golden.words_to_mask(G[f"dens_{i}_words"], N)
    o = _cube_oracle(oracle_mod, mask, order, part)
    o.put("coeff", G[f"dens_{i}_coeff"].astype(np.float64))
    o.coeff_to_density()
    rho = o.get("rho")[mask.astype(bool)]
    assert np.abs(rho - G[f"dens_{i}_rho"]).max() <= 2e-6
    sens = np.zeros(N ** 3)
    sens[mask.astype(bool)] = G[f"adj_{i}_sens"]
    o.put("sens", sens)
    o.spline_adjoint()
    assert rel(o.get("csens"), G[f"adj_{i}_csens"]) <= 1e-5


@pytest.mark.parametrize("i", range(int(G["n_filt"])))
def test_filter(oracle_mod, i):
    mask = golden.words_to_mask(G[f"filt_{i}_words"], N)
    o = _cube_oracle(oracle_mod, mask, 3, [3, 3, 3])
    sens = np.zeros(N ** 3)
    sens[mask.astype(bool)] = G[f"filt_{i}_sens"]
    o.put("sens", sens)
    o.filter(float(G[f"filt_{i}_radius"]))
    out = o.get("sens")[mask.astype(bool)]
    assert rel(out, G[f"filt_{i}_out"]) <= 1e-6
