"""Writes ref_ops.npz: golden vectors of the reference's fine-level elasticity
kernels, run as host code.

Runs in a container that holds the reference sources: oracle/ref_build.py cuts
applyK_OTFA_kernel, update_residual_OTFA_WS_kernel and gs_relax_OTFA_WS_kernel
(grid/Grid.cu:1698-1842, 2277-2333, 4278-4356) out of the reference and compiles
them with oracle/ref_ops_harness.cpp; this script calls them on seeded inputs
and stores inputs and outputs.  The fixture is committed, so the tests that
read it need neither the reference nor this script.

  python tests/golden/make_ref_ops_golden.py

Cases: a 14x10x8 box with seeded spherical holes and a full 12x8x6 box, the
x = 0 face's vertices supported (the reference fixes whole nodes), rho = k/16
(k seeded in 1..16, so the reference's FP32 rho and powf(rho, 3) are exact and
equal the FP64 values), E = 1e6, nu = 0.4, h = 1.  The element matrix is the
FP64 oracle's restatement of the reference's template (element/templateMatrix.cpp),
the one input these kernels take from outside grid/Grid.cu.  Per case: K u,
f - K u, and two forward Gauss-Seidel sweeps from u on f.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_build  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402
from topoptspline3d_gb300 import workloads  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_ops.npz")
U8 = C.POINTER(C.c_uint8)
FP = C.POINTER(C.c_float)
DP = C.POINTER(C.c_double)


def _lib():
    lib = C.CDLL(ref_build.build()[3])
    lib.ref_apply_k.argtypes = [C.c_int, C.c_int, C.c_int, U8, U8, FP, DP, C.c_double, DP, DP]
    lib.ref_residual.argtypes = [C.c_int, C.c_int, C.c_int, U8, U8, FP, DP, C.c_double, DP, DP, DP]
    lib.ref_gs_sweeps.argtypes = [C.c_int, C.c_int, C.c_int, U8, U8, FP, DP, C.c_double, DP, DP, C.c_int]
    return lib


def _p(a, t):
    return a.ctypes.data_as(t)


def vertex_active(ea, nx, ny, nz):
    e3 = ea.reshape(nz, ny, nx).astype(bool)
    va = np.zeros((nz + 1, ny + 1, nx + 1), bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                va[dz:dz + nz, dy:dy + ny, dx:dx + nx] |= e3
    return va.ravel()


def case(lib, name, nx, ny, nz, ea, seed, out):
    rng = np.random.default_rng(seed)
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    va = vertex_active(ea, nx, ny, nz)
    sup = np.zeros((nz + 1, ny + 1, nx + 1), np.uint8)
    sup[:, :, 0] = 1
    sup = (sup.ravel() & va).astype(np.uint8)
    free = (va & (sup == 0)).astype(np.float64)
    rho = (rng.integers(1, 17, size=nx * ny * nz) / 16.0).astype(np.float32)
    rho[ea == 0] = 0.0
    u = (rng.standard_normal((3, nv)) * free).ravel()
    f = (rng.standard_normal((3, nv)) * free).ravel()
    o = Oracle(nx, ny, nz, 1.0, 1e6, 0.4, 3.0, 1e-3, eactive=ea)
    ke = np.ascontiguousarray(o.get("ke"), dtype=np.float64)
    ku, r, ug = np.zeros(3 * nv), np.zeros(3 * nv), u.copy()
    args = (nx, ny, nz, _p(ea, U8), _p(sup, U8), _p(rho, FP), _p(ke, DP), 3.0)
    lib.ref_apply_k(*args, _p(u, DP), _p(ku, DP))
    lib.ref_residual(*args, _p(u, DP), _p(f, DP), _p(r, DP))
    lib.ref_gs_sweeps(*args, _p(ug, DP), _p(f, DP), 2)
    out.update({f"{name}_dims": np.array([nx, ny, nz]), f"{name}_eactive": ea, f"{name}_support": sup,
                f"{name}_rho": rho, f"{name}_u": u, f"{name}_f": f, f"{name}_ke": ke,
                f"{name}_Ku": ku, f"{name}_r": r, f"{name}_gs2": ug})


def main():
    lib = _lib()
    out = {}
    ea = workloads.perforated(14, 10, 8, holes=3, radius=(1.5, 2.5), seed=21).astype(np.uint8)
    case(lib, "holes", 14, 10, 8, ea, 31, out)
    case(lib, "box", 12, 8, 6, np.ones(12 * 8 * 6, np.uint8), 32, out)
    out["cases"] = np.array(["holes", "box"])
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
