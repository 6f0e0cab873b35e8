"""Learned preconditioner end to end on the GPU: harvest residual -> error pairs
from the mixed solver on seeded random densities, train the U-Net with the
library's own kernels, and compare the solve with and without the network
(the ablation).  The FP64 residual judges every solve.

What is asserted is what holds: the training loss falls on the training crops
and the fit carries over to crops of a density never trained on; the solve
with the network converges to the same tolerance with every V-cycle
corrected.  The network does not cut iterations at these sizes (measured:
33 against 32 here, 38 against 34 at 256x128x128), so the iteration bound is
a cap on the damage the energy-optimal blend can do, not a claimed gain."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

NX, NY, NZ = 64, 32, 32


def _problem():
    wl = workloads.half_mbb(NX, NY, NZ, lattice=(17, 9, 9))
    p = capi.Problem(NX, NY, NZ)
    p.set_bc(wl.fixed, wl.loads)
    p.set_operator_precision(2)
    return p


def _solve(p, rho, update=True, **kw):
    if update:
        p.put("rho", rho)
        p.update_operators()
    p.put("u", np.zeros(3 * p.nv))
    opts = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, pre=2, post=2, rtol=1e-6, max_iter=200,
                inner_max=1)
    opts.update(kw)
    return p.solve(**opts)


def test_learned_requires_enable_and_valid_options():
    p = _problem()
    rho = workloads.random_density(NX, NY, NZ, 3000)
    with pytest.raises(capi.TopoError) as e:
        _solve(p, rho, learned=1)
    assert e.value.code == capi.TOPO_E_STATE
    p.unet_enable(1)
    with pytest.raises(capi.TopoError) as e:
        _solve(p, rho, learned=2, inner_max=4)
    assert e.value.code == capi.TOPO_E_BAD_INPUT
    # untrained network: zero last layer, same iterates as without it (same
    # operators and spectral bounds for both solves)
    a = _solve(p, rho, learned=0)
    ua = p.get("u")
    b = _solve(p, rho, update=False, learned=1)
    assert b["learned_applied"] == b["vcycles"] and a["iterations"] == b["iterations"]
    assert np.array_equal(ua, p.get("u"))


@pytest.mark.parametrize("kernel", [capi.CONV_TCGEN05, capi.CONV_MMA_SYNC], ids=["tcgen05", "mma_sync"])
def test_harvest_train_ablation(kernel):
    p = _problem()
    p.unet_enable(11)
    p.unet_set_conv_kernel(kernel)
    p.unet_dataset_reserve(1024, crop=32, crops_per_iterate=16)
    for i in range(8):
        s = _solve(p, workloads.random_density(NX, NY, NZ, 3000 + i), learned=2, rtol=1e-8, max_iter=400,
                   check=False)
        assert s["relres"] <= 2e-8
    n = p.unet_dataset_size()
    assert n >= 256
    split = int(0.85 * n)
    # held-out crops come from the last harvested density (unseen in training)
    before = p.unet_train(20, batch=8, lo=split, hi=n, update=False, seed=5)
    fit0 = p.unet_train(20, batch=8, lo=0, hi=split, update=False, seed=7)
    assert abs(before - 1.0) < 1e-12 and abs(fit0 - 1.0) < 1e-12  # zero last layer: prediction 0
    p.unet_train(400, batch=8, lr=1e-3, lo=0, hi=split, seed=6)
    fit = p.unet_train(20, batch=8, lo=0, hi=split, update=False, seed=7)
    after = p.unet_train(20, batch=8, lo=split, hi=n, update=False, seed=5)
    print(f"relative loss: training crops {fit0:.4f} -> {fit:.4f}; held-out density {before:.4f} -> {after:.4f}")
    assert fit < 0.9 * fit0
    assert after < 0.9 * before  # generalises to an unseen density
    # ablation on an unseen density: same solver with and without the network;
    # the positivity guard and stagnation fallback keep the learned solve sound
    rho = workloads.random_density(NX, NY, NZ, 3999)
    plain = _solve(p, rho, learned=0)
    learned = _solve(p, rho, update=False, learned=1)
    print(f"ablation: V-cycle {plain['iterations']} its {plain['ms']:.2f} ms; "
          f"V-cycle + U-Net {learned['iterations']} its {learned['ms']:.2f} ms "
          f"(applied {learned['learned_applied']}, fallback {learned['learned_fallback']})")
    for s in (plain, learned):
        assert s["relres"] <= 1e-6
    assert learned["learned_applied"] == learned["vcycles"] and not learned["learned_fallback"]
    assert learned["iterations"] <= 1.25 * plain["iterations"] + 1
