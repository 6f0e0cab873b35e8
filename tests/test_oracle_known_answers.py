"""Pins the CPU oracle with known-answer tests derived from the mathematics.

The reference ships no golden vectors or numeric assertions for this path, so
the oracle is checked against identities every correct restatement satisfies:
the element matrix's rigid-body null space (element/templateMatrix.cpp:104-123),
B-spline partition of unity, the filter weight's endpoints, the Galerkin product
against an explicit sparse P^T A P, V-cycle contraction and the OC volume target.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from topoptspline3d_gb300 import workloads
from tests.helpers import setup_oracle, random_masked_u


def test_ke_symmetric_rigid_modes(oracle_mod):
    Ke = oracle_mod.ke_template(1e6, 0.4, 1.0)
    assert np.abs(Ke - Ke.T).max() < 1e-9 * np.abs(Ke).max()
    # rigid body modes: 3 translations + 3 rotations
    RE = np.zeros((24, 6))
    for a in range(8):
        p = np.array([a % 2, a // 2 % 2, a // 4], float)
        RE[3 * a:3 * a + 3, :3] = np.eye(3)
        RE[3 * a:3 * a + 3, 3:] = np.array([[0, -p[2], p[1]], [p[2], 0, -p[0]], [-p[1], p[0], 0]])
    assert np.abs(Ke @ RE).max() < 1e-9 * np.abs(Ke).max()
    w = np.linalg.eigvalsh(Ke)
    assert (np.abs(w[:6]) < 1e-9 * w[-1]).all() and (w[6:] > 1e-6 * w[-1]).all()


def test_ke_scaling_and_patch(oracle_mod):
    # Ke scales linearly with E and h (3-D elasticity: K ~ E h)
    K1 = oracle_mod.ke_template(1.0, 0.3, 1.0)
    K2 = oracle_mod.ke_template(2.0, 0.3, 0.5)
    assert np.allclose(K2, K1 * 2.0 * 0.5, rtol=1e-12, atol=1e-14)
    # uniform strain: internal nodal forces of a linear field sum to zero per element
    u = np.zeros(24)
    for a in range(8):
        p = np.array([a % 2, a // 2 % 2, a // 4], float)
        u[3 * a:3 * a + 3] = np.array([[0.1, 0.02, 0], [0.02, -0.05, 0.01], [0, 0.01, 0.03]]) @ p
    f = K1 @ u
    assert np.abs(f.reshape(8, 3).sum(0)).max() < 1e-12


def test_patch_test_interior_zero(oracle_mod):
    # a linear displacement field produces zero force at interior vertices
    o = oracle_mod.Oracle(6, 5, 4)
    nv = 7 * 6 * 5
    zz, yy, xx = np.meshgrid(np.arange(5), np.arange(6), np.arange(7), indexing="ij")
    G = np.array([[0.1, 0.02, -0.03], [0.04, -0.05, 0.01], [0.02, 0.01, 0.03]])
    pos = np.stack([xx.ravel(), yy.ravel(), zz.ravel()])
    u = (G @ pos).ravel()
    o.set_bc(np.zeros(nv, np.uint8), np.zeros(3 * nv))
    y = o.apply_fine(u).reshape(3, 5, 6, 7)
    assert np.abs(y[:, 1:-1, 1:-1, 1:-1]).max() < 1e-8 * np.abs(y).max()


def test_spline_partition_of_unity(oracle_mod):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    o.put("coeff", np.full(o.num_coeffs(), 0.37))
    o.coeff_to_density()
    rho = o.get("rho")
    assert np.abs(rho - 0.37).max() < 1e-12


def test_knots_reference_rule(oracle_mod):
    o = oracle_mod.Oracle(48, 24, 24)
    o.set_spline(3, (10, 4, 4), (0, 0, 0), (48, 24, 24))
    k = o.knots(0, 3, 10)
    # order copies of each end; p interior knots with constant step (float arithmetic)
    assert k.size == 16 and (k[:3] == k[0]).all() and (k[-3:] == k[-1]).all()
    step = np.diff(k[2:-2])
    assert np.allclose(step, step[0], rtol=1e-5)
    delta = 48.0
    assert abs(k[0] - (0 - 2 * delta / 11)) < 1e-4 and abs(k[-1] - (48 + 2 * delta / 11)) < 1e-4


def test_filter_constant_and_weight(oracle_mod):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    o.put("sens", np.full(16 * 8 * 8, -2.5))
    o.filter(2.0)
    assert np.abs(o.get("sens") + 2.5).max() < 1e-12
    fr = lambda s: 1 - 6 * s * s + 8 * s ** 3 - 3 * s ** 4  # noqa: E731
    assert fr(1.0) == 0.0 and fr(0.0) == 1.0


def _prolongation(fine_dims, coarse_dims, f):
    fx, fy, fz = (d + 1 for d in fine_dims)
    cx, cy, cz = (d + 1 for d in coarse_dims)
    rows, cols, vals = [], [], []
    for z in range(fz):
        for y in range(fy):
            for x in range(fx):
                v = x + fx * (y + fy * z)
                bx, by, bz = x // f, y // f, z // f
                rx, ry, rz = x % f, y % f, z % f
                for k in range(8):
                    ox, oy, oz = k & 1, (k >> 1) & 1, k >> 2
                    w = ((rx if ox else f - rx) * (ry if oy else f - ry) * (rz if oz else f - rz)) / f ** 3
                    if w == 0:
                        continue
                    cv = (bx + ox) + cx * ((by + oy) + cy * (bz + oz))
                    for c in range(3):
                        rows.append(c * fx * fy * fz + v)
                        cols.append(c * cx * cy * cz + cv)
                        vals.append(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(3 * fx * fy * fz, 3 * cx * cy * cz))


def _assembled_fine(o, wl, Ke, rhop, penalty=1e6):
    nx, ny, nz = wl.nx, wl.ny, wl.nz
    vx, vy = nx + 1, ny + 1
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    free = np.ones(3 * nv, bool)
    fixed = wl.fixed
    for c in range(3):
        free[c * nv:(c + 1) * nv] = ((fixed >> c) & 1) == 0
    rows, cols, vals = [], [], []
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                e = x + nx * (y + ny * z)
                dof = []
                for a in range(8):
                    v = (x + a % 2) + vx * ((y + a // 2 % 2) + vy * (z + a // 4))
                    dof += [c * nv + v for c in range(3)]
                dof = np.array(dof)
                K = rhop[e] * Ke.copy()
                fr = free[dof]
                for r in range(24):
                    for s in range(24):
                        k = K[r, s]
                        if not fr[r] or not fr[s]:
                            k = penalty if r == s else 0.0
                        if k != 0.0:
                            rows.append(dof[r]); cols.append(dof[s]); vals.append(k)
    return sp.csr_matrix((vals, (rows, cols)), shape=(3 * nv, 3 * nv))


def _stencil_to_matrix(st, dims):
    vx, vy, vz = (d + 1 for d in dims)
    nv = vx * vy * vz
    st = st.reshape(27, 3, 3, nv)
    rows, cols, vals = [], [], []
    for v in range(nv):
        x, y, z = v % vx, v // vx % vy, v // (vx * vy)
        for d in range(27):
            nx_, ny_, nz_ = x + d % 3 - 1, y + d // 3 % 3 - 1, z + d // 9 - 1
            if not (0 <= nx_ < vx and 0 <= ny_ < vy and 0 <= nz_ < vz):
                continue
            n = nx_ + vx * (ny_ + vy * nz_)
            for i in range(3):
                for j in range(3):
                    if st[d, i, j, v] != 0:
                        rows.append(i * nv + v); cols.append(j * nv + n); vals.append(st[d, i, j, v])
    return sp.csr_matrix((vals, (rows, cols)), shape=(3 * nv, 3 * nv))


def test_galerkin_matches_explicit_product(oracle_mod):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    rng = np.random.default_rng(3)
    o = setup_oracle(wl, coeff=rng.uniform(0.1, 0.9, 7 * 5 * 5))
    o.update_operators()
    Ke = o.get("ke").reshape(24, 24)
    rhop = o.get("rhop")
    A0 = _assembled_fine(o, wl, Ke, rhop)
    dims = [o.level_dims(l) for l in range(o.num_levels())]
    prev = A0
    for l in range(1, o.num_levels()):
        Pm = _prolongation(dims[l - 1], dims[l], o.level_factor(l))
        Ac = (Pm.T @ prev @ Pm).tocsr()
        As = _stencil_to_matrix(o.get("stencil", l), dims[l])
        err = abs(Ac - As).max() / abs(Ac).max()
        assert err < 1e-12, (l, err)
        prev = As


def test_vcycle_contracts_and_pcg_converges(oracle_mod):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    o.update_operators()
    rr = [o.vcycle(5, 5) for _ in range(4)]
    assert rr[1] < 0.5 * rr[0] and rr[3] < 0.5 * rr[2]
    o.put("u", np.zeros(3 * wl.nv))
    it, r = o.pcg(2, 2, 1e-8, 100, 0)
    assert r <= 1e-8 and it < 40
    c = o.compliance()
    # energy identity: u^T K u = f^T u
    u = o.get("u")
    assert abs(u @ o.apply_fine(u) - c) < 1e-6 * abs(c)


def test_chebyshev_pcg_same_solution(oracle_mod):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    o.update_operators()
    o.put("u", np.zeros(3 * wl.nv))
    o.pcg(2, 2, 1e-10, 200, 0)
    c0, u0 = o.compliance(), o.get("u")
    o.put("u", np.zeros(3 * wl.nv))
    it, r = o.pcg(2, 2, 1e-10, 200, 1)
    assert r <= 1e-10
    assert abs(o.compliance() - c0) < 1e-9 * abs(c0)
    assert np.linalg.norm(o.get("u") - u0) < 1e-7 * np.linalg.norm(u0)


def test_operator_symmetric_spd(oracle_mod):
    wl = workloads.half_mbb(8, 4, 4, lattice=(5, 5, 5))
    o = setup_oracle(wl)
    vm = o.get("vmask")
    a, b = random_masked_u(wl.nv, vm, 1), random_masked_u(wl.nv, vm, 2)
    ya, yb = o.apply_fine(a), o.apply_fine(b)
    assert abs(a @ yb - b @ ya) < 1e-10 * abs(a @ yb)
    assert a @ ya > 0


def test_oc_hits_volume(oracle_mod):
    wl = workloads.cantilever(16, 8, 8, lattice=(7, 5, 5))
    o = setup_oracle(wl)
    o.update_operators()
    o.put("u", np.zeros(3 * wl.nv))
    o.pcg(2, 2, 1e-6, 100, 0)
    o.sensitivity()
    s = o.get("sens")
    assert (s <= 0).all()
    o.filter(2.0)
    o.spline_adjoint()
    trials, lam = o.oc_update(0.3)
    assert abs(o.volume() - 0.3) <= 1e-4 or trials == 31


def test_sensitivity_matches_finite_difference(oracle_mod):
    # d c / d rho_e at fixed u equals -u^T dK/drho_e u = the sensitivity formula
    wl = workloads.cantilever(6, 4, 4, lattice=(5, 5, 5))
    o = setup_oracle(wl)
    o.update_operators()
    o.put("u", np.zeros(3 * wl.nv))
    o.pcg(2, 2, 1e-12, 200, 0)
    o.sensitivity()
    s = o.get("sens")
    rho = o.get("rho")
    u = o.get("u")
    e = 17
    eps = 1e-6
    r2 = rho.copy(); r2[e] += eps
    o.put("rho", r2); o.update_penalised()
    ku_p = u @ o.apply_fine(u)
    r2[e] -= 2 * eps
    o.put("rho", r2); o.update_penalised()
    ku_m = u @ o.apply_fine(u)
    fd = -(ku_p - ku_m) / (2 * eps)
    assert abs(fd - s[e]) < 1e-5 * abs(s[e])


def test_gs_maps_reference_ordering(oracle_mod):
    # colour-major with Round<32> padding, lexicographic within a colour
    o = oracle_mod.Oracle(5, 3, 2)
    vid, eid, gsn, ngv, nge = o.gs_maps(0)
    nv = 6 * 4 * 3
    cols = [(v % 6) % 2 + 2 * ((v // 6 % 4) % 2) + 4 * ((v // 24) % 2) for v in range(nv)]
    counts = [cols.count(c) for c in range(8)]
    assert list(gsn) == [(n + 31) // 32 * 32 for n in counts]
    assert ngv == sum(gsn)
    offs = np.concatenate([[0], np.cumsum(gsn)[:-1]])
    seen = [0] * 8
    for v in range(nv):
        c = cols[v]
        assert vid[v] == offs[c] + seen[c]
        seen[c] += 1
    assert len(set(eid.tolist())) == 30 and nge == sum((n + 31) // 32 * 32 for n in
                                                        np.bincount([(e % 5) % 2 + 2 * ((e // 5 % 3) % 2) + 4 * (e // 15 % 2) for e in range(30)], minlength=8))
