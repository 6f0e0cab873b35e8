"""Shared set-up of identical problems on the CUDA library and the CPU oracle."""
from __future__ import annotations

import numpy as np

from topoptspline3d_gb300 import workloads


def setup_oracle(wl: workloads.Workload, coeff=None, E=1e6, nu=0.4, penal=3.0, rho_min=1e-3):
    from oracle.oracle import Oracle
    o = Oracle(wl.nx, wl.ny, wl.nz, 1.0, E, nu, penal, rho_min, eactive=wl.eactive)
    o.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    o.set_spline(wl.order, wl.partition, bmin, bmax)
    nc = o.num_coeffs()
    o.put("coeff", np.full(nc, wl.coeff0) if coeff is None else coeff)
    o.coeff_to_density()
    return o


def setup_gpu(wl: workloads.Workload, coeff=None, E=1e6, nu=0.4, penal=3.0, rho_min=1e-3):
    from topoptspline3d_gb300 import Problem
    p = Problem(wl.nx, wl.ny, wl.nz, 1.0, E, nu, penal, rho_min, eactive=wl.eactive)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    nc = p.num_coeffs()
    p.put("coeff", np.full(nc, wl.coeff0) if coeff is None else coeff)
    p.coeff_to_density()
    return p


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.linalg.norm(b), 1e-300)
    return float(np.linalg.norm(a - b) / den)


def random_masked_u(nv, vmask, seed=0):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((3, nv))
    for c in range(3):
        u[c] *= ((vmask >> c) & 1) & ((vmask >> 3) & 1)
    return u.ravel()


def random_coeff(n, seed=1, lo=0.05, hi=0.95):
    return np.random.default_rng(seed).uniform(lo, hi, n)
