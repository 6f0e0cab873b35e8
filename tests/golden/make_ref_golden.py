"""Writes ref_spline_filter.npz: golden vectors from the reference's own code.

Runs in a container that holds the reference sources: oracle/ref_build.py cuts
the reference's knot series, Cox-de Boor basis, coeff2density, spline-adjoint
and sensitivity-filter code out of its sources and compiles it as host code;
this script calls it on seeded inputs and stores inputs and outputs.  The
fixture is committed, so the tests that read it need neither the reference
nor this script.

  python tests/golden/make_ref_golden.py

Cases (all in the reference's FP32):
  knots_*    set_spline_knot_series for config-0/config-1 lattices and odd boxes,
             orders 3 and 4
  basis_*    SplineBasisX/Y/Z at seeded coordinates inside the knot range
  dens_*     coeff2density on a 16^3 cube (full or a seeded mask), orders 3 and 4
  adj_*      ddensity2dcoeff_update's scatter on the same set-ups
  filt_*     filterSensitivity, radii 1.5, 2 and 3
Masks are stored as the reference's LSB-first uint32 bit words with x fastest
(bit b of word w is element x + n*(y + n*z) = 32*w + b).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_build  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_spline_filter.npz")
FP = C.POINTER(C.c_float)
IP = C.POINTER(C.c_int)
UP = C.POINTER(C.c_uint)


def _lib(m):
    lib = C.CDLL(ref_build.build()[0 if m == 3 else 1])
    lib.ref_m_im.restype = C.c_int
    lib.ref_set_spline.argtypes = [C.c_int, IP, FP, FP, FP, FP]
    lib.ref_basis.argtypes = [C.c_int, C.c_float, FP]
    lib.ref_coeff2density.argtypes = [C.c_int, C.c_int, UP, IP, FP, C.c_float, C.c_float, FP, C.c_int, FP]
    lib.ref_spline_adjoint.argtypes = [C.c_int, C.c_int, UP, IP, FP, C.c_float, FP, C.c_int, FP, C.c_int]
    lib.ref_filter.argtypes = [C.c_int, C.c_int, UP, IP, FP, C.c_double, C.c_int, FP]
    assert lib.ref_m_im() == m
    return lib


def _p(a, t):
    return a.ctypes.data_as(t)


def bitwords(mask):
    """uint8 mask [n^3] (x fastest) -> LSB-first uint32 words and their exclusive prefix counts."""
    bits = np.asarray(mask, dtype=np.uint8).ravel()
    assert bits.size % 32 == 0
    w = np.zeros(bits.size // 32, dtype=np.uint32)
    for b in range(32):
        w |= bits[b::32].astype(np.uint32) << np.uint32(b)
    cnt = np.array([bin(int(x)).count("1") for x in w], dtype=np.int32)
    sat = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int32)
    return w, sat


def set_spline(lib, order, part, box):
    part = np.asarray(part, dtype=np.int32)
    box = np.asarray(box, dtype=np.float32)
    knots = np.zeros(int(3 * 2 * order + part.sum()), dtype=np.float32)
    bmin = np.zeros(3, dtype=np.float32)
    step = np.zeros(3, dtype=np.float32)
    lib.ref_set_spline(order, _p(part, IP), _p(box, FP), _p(knots, FP), _p(bmin, FP), _p(step, FP))
    return knots, bmin, step


def main():
    libs = {3: _lib(3), 4: _lib(4)}
    g = {}
    # knot series
    knot_cases = [(3, (10, 4, 4), (0, 0, 0, 48, 24, 24)), (3, (62, 30, 30), (0, 0, 0, 256, 128, 128)),
                  (4, (9, 3, 3), (0, 0, 0, 48, 24, 24)), (4, (61, 29, 29), (0, 0, 0, 256, 128, 128)),
                  (3, (7, 2, 5), (-1.5, 0.25, 2.0, 30.7, 11.0, 9.5)), (4, (5, 6, 1), (0, 0, 0, 16, 16, 16))]
    for i, (order, part, box) in enumerate(knot_cases):
        knots, bmin, step = set_spline(libs[order], order, part, box)
        g[f"knots_{i}_order"] = np.int32(order)
        g[f"knots_{i}_part"] = np.asarray(part, dtype=np.int32)
        g[f"knots_{i}_box"] = np.asarray(box, dtype=np.float64)
        g[f"knots_{i}_knots"] = knots
        g[f"knots_{i}_bmin"] = bmin
        g[f"knots_{i}_step"] = step
        # basis at seeded coordinates inside the box (where element centres lie)
        rng = np.random.default_rng(100 + i)
        lo, hi = np.asarray(box[:3], dtype=np.float32), np.asarray(box[3:], dtype=np.float32)
        xs = (lo + (hi - lo) * rng.uniform(0.0, 1.0, (64, 3))).astype(np.float32)
        vals = np.zeros((64, 3, order + 1), dtype=np.float32)
        for k in range(64):
            for a in range(3):
                libs[order].ref_basis(a, float(xs[k, a]), _p(vals[k, a], FP))
        g[f"basis_{i}_x"] = xs
        g[f"basis_{i}_N"] = vals[:, :, :order]
    # density and adjoint on a 16^3 cube
    n = 16
    cube = (0, 0, 0, n, n, n)
    masks = {"full": np.ones(n ** 3, dtype=np.uint8),
             "masked": (np.random.default_rng(7).uniform(size=n ** 3) < 0.7).astype(np.uint8)}
    dens_cases = [(3, (5, 3, 4), "full"), (3, (6, 5, 3), "masked"), (4, (5, 4, 3), "masked")]
    for i, (order, part, mk) in enumerate(dens_cases):
        lib = libs[order]
        set_spline(lib, order, part, cube)
        w, sat = bitwords(masks[mk])
        na = int(masks[mk].sum())
        nc = int(np.prod([order + p for p in part]))
        rng = np.random.default_rng(200 + i)
        coeff = rng.uniform(0.0, 1.0, nc).astype(np.float32)
        origin = np.zeros(3, dtype=np.float32)
        rho = np.zeros(na, dtype=np.float32)
        lib.ref_coeff2density(n, w.size, _p(w, UP), _p(sat, IP), _p(origin, FP), 1.0, 1e-3, _p(coeff, FP), na,
                              _p(rho, FP))
        g[f"dens_{i}_order"] = np.int32(order)
        g[f"dens_{i}_part"] = np.asarray(part, dtype=np.int32)
        g[f"dens_{i}_words"] = w
        g[f"dens_{i}_coeff"] = coeff
        g[f"dens_{i}_rho"] = rho
        gsen = rng.standard_normal(na).astype(np.float32)
        cs = np.zeros(nc, dtype=np.float32)
        lib.ref_spline_adjoint(n, w.size, _p(w, UP), _p(sat, IP), _p(origin, FP), 1.0, _p(gsen, FP), na,
                               _p(cs, FP), nc)
        g[f"adj_{i}_sens"] = gsen
        g[f"adj_{i}_csens"] = cs
    # sensitivity filter
    filt_cases = [(2.0, "masked"), (1.5, "full"), (3.0, "masked")]
    for i, (R, mk) in enumerate(filt_cases):
        w, sat = bitwords(masks[mk])
        na = int(masks[mk].sum())
        sens = np.random.default_rng(300 + i).standard_normal(na).astype(np.float32)
        out = np.zeros(na, dtype=np.float32)
        libs[3].ref_filter(n, w.size, _p(w, UP), _p(sat, IP), _p(sens, FP), R, na, _p(out, FP))
        g[f"filt_{i}_radius"] = np.float64(R)
        g[f"filt_{i}_words"] = w
        g[f"filt_{i}_sens"] = sens
        g[f"filt_{i}_out"] = out
    g["cube"] = np.int32(n)
    g["n_knots"] = np.int32(len(knot_cases))
    g["n_dens"] = np.int32(len(dens_cases))
    g["n_filt"] = np.int32(len(filt_cases))
    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
