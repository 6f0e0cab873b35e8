"""Worst-case compliance on the CPU FP64 oracle (test infrastructure only).

Two restatements over the same load space (loads on a set of load vertices,
each along its normal or in any direction; no load on fixed DOFs):

dense_worst        the exact answer: M = S^T K^-1 S column by column from
                   oracle solves to 1e-11, then its largest eigenpair.  The
                   worst unit load is the eigenvector, its compliance the
                   eigenvalue.
modified_pm        the reference's modified power method
                   (optimization/optimization.cpp:213-351): random nodal force,
                   forceProject (optimization/projection.cpp:289-360: gather to
                   the load vertices, remove the tangential parts), unitise,
                   then repeat { one GS V(1,1) cycle on K u = f; f = project(u);
                   unitise; fch = |f_s - f_s,old| / |f_s,old| } until
                   fch <= 1e-4 and rel-res <= 1e-2 (at most 500 cycles);
                   compliance F . U.  The with-support modes only (the
                   no-support mode's rigid-body balancing needs a singular K).
"""
from __future__ import annotations

import numpy as np


def _masks(o, vid):
    vm = o.get("vmask")
    free = np.stack([((vm[vid] >> c) & 1).astype(np.float64) for c in range(3)], axis=1)  # [n][3]
    return free


def scatter(o, vid, normals, x, free_direction):
    """Nodal force SoA [3][nv] from load coordinates x (n or 3n)."""
    nv = o.nv
    f = np.zeros((3, nv))
    fr = _masks(o, vid)
    xs = x.reshape(-1, 3) if free_direction else x[:, None] * normals
    for c in range(3):
        f[c, vid] = xs[:, c] * fr[:, c]
    return f.ravel()


def gather(o, vid, normals, u, free_direction):
    """S^T u: load coordinates of a displacement SoA [3][nv]."""
    fr = _masks(o, vid)
    us = np.stack([u.reshape(3, -1)[c, vid] for c in range(3)], axis=1) * fr
    return us.ravel() if free_direction else (us * normals).sum(axis=1)


def dense_worst(o, vid, normals, free_direction=False, rtol=1e-11):
    """(largest eigenvalue, unit eigenvector, all eigenvalues) of M = S^T K^-1 S.
    The oracle's operators must be up to date (update_operators)."""
    vid = np.asarray(vid)
    normals = np.asarray(normals, dtype=np.float64).reshape(-1, 3)
    m = 3 * len(vid) if free_direction else len(vid)
    M = np.zeros((m, m))
    for j in range(m):
        e = np.zeros(m)
        e[j] = 1.0
        f = scatter(o, vid, normals, e, free_direction)
        if not f.any():
            continue
        o.put("f", f)
        o.put("u", np.zeros_like(f))
        o.pcg(2, 2, rtol, 500, 0)
        M[:, j] = gather(o, vid, normals, o.get("u"), free_direction)
    M = 0.5 * (M + M.T)
    w, V = np.linalg.eigh(M)
    return w[-1], V[:, -1], w[::-1]


def modified_pm(o, vid, normals, seed=1, max_itn=500, free_direction=False):
    """The reference's modified power method; returns (compliance, unit load
    coordinates, cycles)."""
    vid = np.asarray(vid)
    normals = np.asarray(normals, dtype=np.float64).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    nv = o.nv
    fr = _masks(o, vid)

    def project(v):  # gather onto the load vertices, keep the admissible part
        vs = np.stack([v.reshape(3, -1)[c, vid] for c in range(3)], axis=1) * fr
        if not free_direction:
            vs = (vs * normals).sum(axis=1, keepdims=True) * normals * fr
        f = np.zeros((3, nv))
        for c in range(3):
            f[c, vid] = vs[:, c]
        return f.ravel(), vs.ravel()

    f, fs = project(rng.uniform(-1.0, 1.0, 3 * nv))
    nr = np.linalg.norm(f)
    f, fs = f / nr, fs / nr
    o.put("f", f)
    o.put("u", np.zeros(3 * nv))
    fch, rel_res, itn = 1.0, 1.0, 0
    while itn < max_itn and (fch > 1e-4 or rel_res > 1e-2):
        itn += 1
        rel_res = o.vcycle(1, 1)
        u = o.get("u")
        f, fs_new = project(u)
        nr = np.linalg.norm(f)
        f, fs_new = f / nr, fs_new / nr
        fch = np.linalg.norm(fs_new - fs) / np.linalg.norm(fs)
        fs = fs_new
        o.put("f", f)
    c = float(np.dot(o.get("f"), o.get("u")))
    x = fs.reshape(-1, 3)
    coords = x.ravel() if free_direction else (x * normals).sum(axis=1)
    return c, coords, itn
