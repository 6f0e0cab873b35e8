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
    """Active-element mask: union of seeded random ellipsoids (centres uniform in
    the box, semi-axes uniform in ``axes``, random rotations), rescaled until the
    fill fraction falls in ``fill``.  The rescale search runs on a subsampled
    grid; the mask is then evaluated once at full resolution, slab by slab."""
    rng = np.random.default_rng(seed)
    c = rng.uniform((0, 0, 0), (nx, ny, nz), size=(n, 3))
    ax = rng.uniform(axes[0], axes[1], size=(n, 3))
    rot = []
    for _ in range(n):
        q, _r = np.linalg.qr(rng.standard_normal((3, 3)))
        rot.append(q)

    def inside(pts, scale):
        m = np.zeros(pts.shape[0], bool)
        for k in range(n):
            d = (pts - c[k]) @ rot[k]
            m |= ((d / (ax[k] * scale)) ** 2).sum(1) <= 1.0
        return m

    step = max(1, min(nx, ny, nz) // 32)
    zz, yy, xx = np.meshgrid(np.arange(0, nz, step) + 0.5, np.arange(0, ny, step) + 0.5,
                             np.arange(0, nx, step) + 0.5, indexing="ij")
    sub = np.stack([xx, yy, zz], -1).reshape(-1, 3)
    scale = 1.0
    for _ in range(60):
        f = inside(sub, scale).mean()
        if fill[0] <= f <= fill[1]:
            break
        scale *= (0.45 / max(f, 1e-3)) ** (1 / 3)
    out = np.zeros((nz, ny, nx), bool)
    yy2, xx2 = np.meshgrid(np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    for z in range(nz):
        pts = np.stack([xx2.ravel(), yy2.ravel(), np.full(xx2.size, z + 0.5)], -1)
        out[z] = inside(pts, scale).reshape(ny, nx)
    return out.astype(np.uint8).ravel()


def supported_components(eactive, nx, ny, nz, zmax=2) -> np.ndarray:
    """Keep the face-connected components of an element mask that reach the
    layer of elements below z = zmax (the supported ones)."""
    from scipy.ndimage import label
    m = np.asarray(eactive).reshape(nz, ny, nx) != 0
    lab, _ = label(m)
    keep = np.unique(lab[:zmax][lab[:zmax] > 0])
    return np.isin(lab, keep).astype(np.uint8).ravel()


def large_ellipsoids(nx=511, ny=256, nz=256, seed=4000, nloads=64, spacing=4, vgoal=0.3, order=3) -> Workload:
    """Large design: the supported part of a 12-ellipsoid union filling about
    45% of the box; every vertex with z <= 2 fixed; `nloads` unit point loads
    (direction -z) on top-surface vertices chosen with default_rng(seed + 1);
    spline control spacing `spacing` voxels; volume fraction `vgoal`."""
    ea = supported_components(ellipsoid_union(nx, ny, nz, seed=seed), nx, ny, nz)
    vx, vy, vz = nx + 1, ny + 1, nz + 1
    e3 = ea.reshape(nz, ny, nx).astype(bool)
    va = np.zeros((vz, vy, vx), bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                va[dz:dz + nz, dy:dy + ny, dx:dx + nx] |= e3
    fixed = np.zeros((vz, vy, vx), np.uint8)
    fixed[:3][va[:3]] = 7
    # top surface: the highest active vertex of each (x, y) column
    top = np.where(va.any(0), vz - 1 - np.argmax(va[::-1], axis=0), -1)
    cand = np.argwhere(top > 2)
    rng = np.random.default_rng(seed + 1)
    pick = cand[rng.choice(cand.shape[0], size=min(nloads, cand.shape[0]), replace=False)]
    loads = np.zeros((3, vz, vy, vx))
    for y, x in pick:
        loads[2, top[y, x], y, x] = -1.0
    lattice = (nx // spacing + 1, ny // spacing + 1, nz // spacing + 1)
    part = tuple(n - order for n in lattice)
    return Workload(f"ellipsoid union {nx}x{ny}x{nz}", nx, ny, nz, fixed.ravel(), loads.ravel(), part, order,
                    coeff0=vgoal, vgoal=vgoal, eactive=ea,
                    notes={"fill": float(ea.mean()), "loads": int(len(pick)), "lattice": lattice})


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


def batch_cantilevers(n=32, seed0=2000, nx_range=(32, 96), nyz_range=(32, 48), vf_range=(0.2, 0.5), spacing=4):
    """Independent cantilever designs of uneven sizes: for d = 0..n-1, with
    rng = default_rng(seed0 + d), nx uniform in nx_range, ny and nz uniform in
    nyz_range (integers, inclusive), volume fraction uniform in vf_range;
    cantilever boundary conditions; spline control spacing `spacing` voxels."""
    out = []
    for d in range(n):
        rng = np.random.default_rng(seed0 + d)
        nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
        ny = int(rng.integers(nyz_range[0], nyz_range[1] + 1))
        nz = int(rng.integers(nyz_range[0], nyz_range[1] + 1))
        vf = float(rng.uniform(*vf_range))
        wl = cantilever(nx, ny, nz, lattice=(nx // spacing + 1, ny // spacing + 1, nz // spacing + 1))
        wl.vgoal = vf
        wl.coeff0 = vf
        wl.name = f"cantilever {nx}x{ny}x{nz} vf {vf:.3f}"
        out.append(wl)
    return out
