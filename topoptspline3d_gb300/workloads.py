"""Synthetic workloads: grids, boundary conditions and loads of the benchmark cases.

All arrays use the library layout (vertex v = x + (nx+1)*(y + (ny+1)*z), loads SoA
[3][nv]).  Nothing here is random unless a seed is given.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nz: int
    fixed: np.ndarray            # uint8[nv], bit c = DOF c fixed
    loads: np.ndarray            # float64[3*nv]
    partition: tuple             # spline partitions per axis (n_basis = order + partition)
    order: int = 3
    coeff0: float = 0.4          # initial spline coefficient value
    vgoal: float = 0.4
    filter_radius: float = 2.0
    eactive: np.ndarray | None = None
    notes: dict = field(default_factory=dict)

    @property
    def nv(self):
        return (self.nx + 1) * (self.ny + 1) * (self.nz + 1)

    def spline_box(self):
        return (0.0, 0.0, 0.0), (float(self.nx), float(self.ny), float(self.nz))


def _grid(nx, ny, nz):
    vx, vy, vz = nx + 1, ny + 1, nz + 1
    fixed = np.zeros((vz, vy, vx), np.uint8)
    loads = np.zeros((3, vz, vy, vx))
    return fixed, loads


def cantilever(nx=48, ny=24, nz=24, lattice=(13, 7, 7), order=3) -> Workload:
    """Cantilever: x = 0 face fully fixed; total force 1 downward (-z) spread
    uniformly over the nodes of the bottom edge (x = nx, z = 0)."""
    fixed, loads = _grid(nx, ny, nz)
    fixed[:, :, 0] = 7
    loads[2, 0, :, nx] = -1.0 / (ny + 1)
    part = tuple(n - order for n in lattice)
    return Workload(f"cantilever {nx}x{ny}x{nz}", nx, ny, nz, fixed.ravel(), loads.ravel(), part, order)


def half_mbb(nx=256, ny=128, nz=128, lattice=(65, 33, 33), order=3) -> Workload:
    """Half-MBB beam: symmetry rollers u_x = 0 on the x = 0 face; roller support
    u_z = 0 on the bottom edge at x = nx (nodes (nx, y, 0)); u_y = 0 on that edge
    as well, which removes the y-translation null mode; unit downward line load
    along the top edge at x = 0 (nodes (0, y, nz))."""
    fixed, loads = _grid(nx, ny, nz)
    fixed[:, :, 0] |= 1
    fixed[0, :, nx] |= 4 | 2
    loads[2, nz, :, 0] = -1.0 / (ny + 1)
    part = tuple(n - order for n in lattice)
    return Workload(f"half-MBB {nx}x{ny}x{nz}", nx, ny, nz, fixed.ravel(), loads.ravel(), part, order,
                    notes={"extra_constraint": "u_y = 0 on the roller edge (x=nx, z=0)"})


def small_cases():
    """Parity-test cases the oracle finishes in seconds."""
    return {
        "cantilever48": cantilever(),
        "cantilever16": cantilever(16, 8, 8, lattice=(7, 5, 5)),
        "mbb32": half_mbb(32, 16, 16, lattice=(11, 7, 7)),
    }


def perforated(nx, ny, nz, holes=6, radius=(2.0, 4.0), seed=7) -> np.ndarray:
    """Active-element mask: the box minus seeded spherical holes that stay clear
    of the x = 0 and x = nx faces (the domain stays connected and supported)."""
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.meshgrid(np.arange(nz) + 0.5, np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    m = np.ones((nz, ny, nx), bool)
    for _ in range(holes):
        r = rng.uniform(*radius)
        c = rng.uniform((r + 1, 0, 0), (nx - r - 1, ny, nz))
        m &= (xx - c[0]) ** 2 + (yy - c[1]) ** 2 + (zz - c[2]) ** 2 > r * r
    return m.astype(np.uint8).ravel()


def ellipsoid_union(nx, ny, nz, n=12, seed=4000, fill=(0.43, 0.47), axes=(20, 120)) -> np.ndarray:
    """Active-element mask: union of seeded random ellipsoids, rescaled until the
    fill fraction falls in ``fill``."""
    rng = np.random.default_rng(seed)
    c = rng.uniform((0, 0, 0), (nx, ny, nz), size=(n, 3))
    ax = rng.uniform(axes[0], axes[1], size=(n, 3))
    rot = []
    for _ in range(n):
        q, _r = np.linalg.qr(rng.standard_normal((3, 3)))
        rot.append(q)
    zz, yy, xx = np.meshgrid(np.arange(nz) + 0.5, np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    pts = np.stack([xx, yy, zz], -1).reshape(-1, 3)
    scale = 1.0
    for _ in range(40):
        m = np.zeros(pts.shape[0], bool)
        for k in range(n):
            d = (pts - c[k]) @ rot[k]
            m |= ((d / (ax[k] * scale)) ** 2).sum(1) <= 1.0
        f = m.mean()
        if fill[0] <= f <= fill[1]:
            break
        scale *= (0.45 / max(f, 1e-3)) ** (1 / 3)
    return m.astype(np.uint8)


def random_density(nx, ny, nz, seed, sigma=None, lo=1e-3) -> np.ndarray:
    """Seeded Gaussian-smoothed white noise, affinely mapped to mean 0.5 and
    spread 0.35 and clipped to [lo, 1] (the learned preconditioner's training
    densities).  sigma defaults to a seeded draw in [3, 6] voxels."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    if sigma is None:
        sigma = rng.uniform(3.0, 6.0)
    g = gaussian_filter(rng.standard_normal((nz, ny, nx)), sigma, mode="wrap")
    g = (g - g.mean()) / max(g.std(), 1e-12)
    return np.clip(0.5 + 0.35 * g, lo, 1.0).ravel()


def patch_loads(nx, ny, nz, nrhs, seed0=1000, patch=8) -> np.ndarray:
    """Load cases of the batched worst-case study: for k = 0..nrhs-1, with
    rng = default_rng(seed0 + k), a patch origin uniform over the valid
    patch x patch voxel positions of the x = nx face ((patch+1)^2 nodes), a
    direction rng.standard_normal(3) normalised, per-node force dir/(patch+1)^2.
    Returns [nrhs][3*nv]."""
    vx, vy, vz = nx + 1, ny + 1, nz + 1
    nv = vx * vy * vz
    out = np.zeros((nrhs, 3 * nv))
    for k in range(nrhs):
        rng = np.random.default_rng(seed0 + k)
        y0 = int(rng.integers(0, ny - patch + 1))
        z0 = int(rng.integers(0, nz - patch + 1))
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        npn = (patch + 1) ** 2
        for z in range(z0, z0 + patch + 1):
            for y in range(y0, y0 + patch + 1):
                v = nx + vx * (y + vy * z)
                for c in range(3):
                    out[k, c * nv + v] = d[c] / npn
    return out
