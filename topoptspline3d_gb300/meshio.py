"""Triangle meshes for the mesh -> bit-mask voxeliser: a Wavefront OBJ reader
and writer (the reference reads its bench meshes with trimesh2) and seeded
closed test surfaces."""
from __future__ import annotations

import numpy as np


def read_obj(path):
    """(verts float32 [n][3], tris int32 [m][3]) of an OBJ file; polygons are
    split into fans, 'v/vt/vn' indices and negative (relative) indices are
    accepted, everything but 'v' and 'f' records is ignored."""
    verts, tris = [], []
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "v":
                verts.append([float(p[1]), float(p[2]), float(p[3])])
            elif p[0] == "f":
                ids = []
                for tok in p[1:]:
                    k = int(tok.split("/")[0])
                    ids.append(k - 1 if k > 0 else len(verts) + k)
                for j in range(1, len(ids) - 1):
                    tris.append([ids[0], ids[j], ids[j + 1]])
    return np.asarray(verts, dtype=np.float32).reshape(-1, 3), np.asarray(tris, dtype=np.int32).reshape(-1, 3)


def write_obj(path, verts, tris):
    with open(path, "w") as f:
        for v in np.asarray(verts).reshape(-1, 3):
            f.write(f"v {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}\n")
        for t in np.asarray(tris).reshape(-1, 3):
            f.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")


def uv_sphere(center=(0.0, 0.0, 0.0), radius=1.0, nu=24, nv=12):
    """Closed sphere: nv - 1 latitude rings of nu vertices plus the poles."""
    c = np.asarray(center, dtype=np.float64)
    verts = [c + [0, 0, radius]]
    for i in range(1, nv):
        th = np.pi * i / nv
        for j in range(nu):
            ph = 2 * np.pi * j / nu
            verts.append(c + radius * np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)]))
    verts.append(c + [0, 0, -radius])
    s = len(verts) - 1
    tris = []
    for j in range(nu):
        tris.append([0, 1 + j, 1 + (j + 1) % nu])
    for i in range(nv - 2):
        a, b = 1 + i * nu, 1 + (i + 1) * nu
        for j in range(nu):
            j1 = (j + 1) % nu
            tris.append([a + j, b + j, b + j1])
            tris.append([a + j, b + j1, a + j1])
    base = 1 + (nv - 2) * nu
    for j in range(nu):
        tris.append([base + j, s, base + (j + 1) % nu])
    return np.asarray(verts, dtype=np.float32), np.asarray(tris, dtype=np.int32)


def torus(center=(0.0, 0.0, 0.0), R=1.0, r=0.35, nu=32, nv=16):
    c = np.asarray(center, dtype=np.float64)
    verts, tris = [], []
    for i in range(nu):
        u = 2 * np.pi * i / nu
        for j in range(nv):
            v = 2 * np.pi * j / nv
            verts.append(c + [(R + r * np.cos(v)) * np.cos(u), (R + r * np.cos(v)) * np.sin(u), r * np.sin(v)])
    for i in range(nu):
        for j in range(nv):
            a, b = i * nv + j, ((i + 1) % nu) * nv + j
            a1, b1 = i * nv + (j + 1) % nv, ((i + 1) % nu) * nv + (j + 1) % nv
            tris.append([a, b, b1])
            tris.append([a, b1, a1])
    return np.asarray(verts, dtype=np.float32), np.asarray(tris, dtype=np.int32)


def box(lo, hi, rotation=None):
    """Closed box [lo, hi] (12 triangles), optionally rotated by a 3x3 matrix about its centre."""
    lo, hi = np.asarray(lo, dtype=np.float64), np.asarray(hi, dtype=np.float64)
    corners = np.array([[lo[0] if i & 1 == 0 else hi[0], lo[1] if i & 2 == 0 else hi[1], lo[2] if i & 4 == 0 else hi[2]]
                        for i in range(8)])
    if rotation is not None:
        ctr = 0.5 * (lo + hi)
        corners = (corners - ctr) @ np.asarray(rotation).T + ctr
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    tris = []
    for a, b, c, d in quads:
        tris += [[a, b, c], [a, c, d]]
    return corners.astype(np.float32), np.asarray(tris, dtype=np.int32)


def rotation(seed):
    """Seeded random rotation (QR of a Gaussian matrix, determinant +1)."""
    q, r = np.linalg.qr(np.random.default_rng(seed).standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def merge(*meshes):
    vs, ts, off = [], [], 0
    for v, t in meshes:
        vs.append(v)
        ts.append(t + off)
        off += len(v)
    return np.concatenate(vs).astype(np.float32), np.concatenate(ts).astype(np.int32)
