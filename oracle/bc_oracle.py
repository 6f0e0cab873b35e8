"""numpy restatement of the region-predicate boundary conditions (test
infrastructure only): the reference's region containment
(boundary/BoundaryCondition.h:38-173, 401-529), force fields (:555-700), surface
vertices (grid/Grid.cu:2781-2815) and the support-before-load assignment
(grid/Grid.cpp:2689-2721), written vectorised over all vertices."""
from __future__ import annotations

import numpy as np


def _contains(reg: dict, P: np.ndarray) -> np.ndarray:
    t = reg["type"]
    closed = bool(reg.get("closed", False))
    comp = bool(reg.get("complement", False))
    if t == "sphere":
        c = np.array(reg["center"], float)
        r2 = float(reg["radius"]) ** 2
        d2 = ((P - c) ** 2).sum(axis=1)
        m = (d2 < r2) | (closed & ((d2 - r2) < 1e-8))
    elif t == "box":
        p, q = np.array(reg["p"], float), np.array(reg["q"], float)
        lo, hi = np.minimum(p, q), np.maximum(p, q)
        strict = ((P > lo) & (P < hi)).all(axis=1)
        inc = ((P >= lo) & (P <= hi)).all(axis=1)
        m = strict | (closed & inc)
    elif t == "halfspace":
        a, b, c = (np.array(reg[k], float) for k in ("p1", "p2", "p3"))
        n = np.cross(b - a, c - a)
        s = (P - a) @ n
        m = (s > 0) | (closed & (s == 0))
    elif t == "cylinder":
        b0 = np.array(reg["bottomCenter"], float)
        hv = np.array(reg["heightVector"], float)
        hl = np.linalg.norm(hv)
        z = hv / hl
        w = P - b0
        proj = w @ z
        dev = np.linalg.norm(np.cross(w, z), axis=1)
        return (proj <= hl) & (proj >= 0) & (dev < float(reg["radius"]))
    else:
        raise ValueError(t)
    return ~m if comp else m


def _unit(v):
    n = np.linalg.norm(v, axis=-1, keepdims=True)
    return np.where(n > 0, v / np.where(n > 0, n, 1), 0.0)


def _field(f: dict, P: np.ndarray) -> np.ndarray:
    t = f["type"]
    amp = float(f.get("amplifier", 1.0))
    damp = float(f.get("dampRatio", 1.0))
    if t == "const":
        return float(f["norm"]) * np.broadcast_to(_unit(np.array(f["direction"], float)), P.shape)
    if t == "RadialNormConstDir":
        c = np.array(f["center"], float)
        nrm = amp * np.exp(-np.linalg.norm(c - P, axis=1) ** (2 * damp))
        return nrm[:, None] * _unit(np.array(f["direction"], float))[None, :]
    if t == "ConstNormRadialDir":
        c = np.array(f["center"], float)
        return float(f["norm"]) * _unit(c - P)
    if t == "RadialNormRadialDir":
        nc, dc = np.array(f["NormCenter"], float), np.array(f["DirCenter"], float)
        nrm = amp * np.exp(-np.linalg.norm(nc - P, axis=1) ** (2 * damp))
        return nrm[:, None] * _unit(dc - P)
    if t == "Twist":
        a, b = np.array(f["AxisStart"], float), np.array(f["AxisEnd"], float)
        nrm = np.linalg.norm(np.cross(P - a, _unit(b - a)), axis=1) * amp
        return nrm[:, None] * _unit(np.cross(P - a, b - a))
    raise ValueError(t)


def surface_vertices(nx, ny, nz, eactive=None) -> tuple[np.ndarray, np.ndarray]:
    """(active vertex mask, surface vertex mask), both [nv] lexicographic."""
    ea = np.ones((nz, ny, nx), bool) if eactive is None else np.asarray(eactive).reshape(nz, ny, nx) != 0
    pad = np.zeros((nz + 2, ny + 2, nx + 2), bool)
    pad[1:-1, 1:-1, 1:-1] = ea
    # s[l][j][i] = element (x-1+i, y-1+j, z-1+l) of vertex (x, y, z)
    s = [[[pad[l:l + nz + 1, j:j + ny + 1, i:i + nx + 1] for i in range(2)] for j in range(2)] for l in range(2)]
    active = np.zeros((nz + 1, ny + 1, nx + 1), bool)
    ax = [np.zeros_like(active) for _ in range(3)]
    for l in range(2):
        for j in range(2):
            for i in range(2):
                active |= s[l][j][i]
    for a in range(2):
        for b in range(2):
            ax[0] |= s[b][a][0] & s[b][a][1]
            ax[1] |= s[b][0][a] & s[b][1][a]
            ax[2] |= s[0][b][a] & s[1][b][a]
    surf = active & ~(ax[0] & ax[1] & ax[2])
    return active.ravel(), surf.ravel()


def plan(nx, ny, nz, doc: dict, origin=(0.0, 0.0, 0.0), spacing=1.0, eactive=None):
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    _, surf = surface_vertices(nx, ny, nz, eactive)
    z, y, x = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    P = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1) * float(spacing) + np.array(origin, float)
    fix = np.zeros(nv, bool)
    for r in doc.get("fixedarea", []):
        fix |= _contains(r, P)
    fix &= surf
    load = np.zeros(nv, bool)
    for r in doc.get("loadarea", []):
        load |= _contains(r, P)
    load &= surf & ~fix
    F = np.zeros((nv, 3))
    for f in doc.get("force", []):
        m = _contains(f["region"], P)
        F[m] += _field(f, P[m])
    F[~load] = 0.0
    fixed = np.where(fix, 7, 0).astype(np.uint8)
    return fixed, F.T.ravel().copy(), int(fix.sum()), int(load.sum())
