"""ctypes front end of the CPU FP64 oracle (test infrastructure only).

The shared library is compiled from ``topo_oracle.cpp`` with g++ (OpenMP, no
architecture-specific flags, FP contraction off) into ``oracle/_build``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libtopo_oracle.so")

RHO, RHOP, COEFF, SENS, CSENS, U, F, R, STENCIL, KELEM, VMASK, EACTIVE, KE, DIAG = range(14)
_NAMES = {
    "rho": RHO, "rhop": RHOP, "coeff": COEFF, "sens": SENS, "csens": CSENS, "u": U, "f": F,
    "r": R, "stencil": STENCIL, "kelem": KELEM, "vmask": VMASK, "eactive": EACTIVE, "ke": KE,
}


ORACLE_SOURCES = ("topo_oracle.cpp", "mma_oracle.cpp")


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in ORACLE_SOURCES] + [os.path.join(HERE, "topo_oracle.h")]
    if not force and os.path.exists(ORACLE_LIB) and all(
            os.path.getmtime(ORACLE_LIB) >= os.path.getmtime(s) for s in srcs):
        return ORACLE_LIB
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    tmp = ORACLE_LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                           "-std=c++17", "-o", tmp] + srcs[:-1])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


_lib = None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build_oracle()
    lib = C.CDLL(ORACLE_LIB)
    vp, dp, ip, i64 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int64
    sig = {
        "orc_ke_template": (None, [C.c_double, C.c_double, C.c_double, dp]),
        "orc_create": (vp, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                            C.c_double, C.c_double, vp]),
        "orc_destroy": (None, [vp]),
        "orc_num_levels": (C.c_int, [vp]),
        "orc_level_dims": (None, [vp, C.c_int, ip]),
        "orc_level_factor": (C.c_int, [vp, C.c_int]),
        "orc_set_bc": (None, [vp, vp, vp]),
        "orc_set_spline": (None, [vp, C.c_int, ip, dp, dp]),
        "orc_num_coeffs": (C.c_int, [vp]),
        "orc_get_knots": (None, [vp, C.c_int, dp]),
        "orc_put": (None, [vp, C.c_int, C.c_int, vp]),
        "orc_get": (None, [vp, C.c_int, C.c_int, vp]),
        "orc_size": (i64, [vp, C.c_int, C.c_int]),
        "orc_spline_basis": (C.c_int, [vp, C.c_int, C.c_double, dp]),
        "orc_coeff_to_density": (None, [vp]),
        "orc_update_penalised": (None, [vp]),
        "orc_update_operators": (None, [vp]),
        "orc_apply_fine": (None, [vp, vp, vp]),
        "orc_residual": (None, [vp, C.c_int]),
        "orc_smooth": (None, [vp, C.c_int, C.c_int, C.c_int]),
        "orc_restrict": (None, [vp, C.c_int]),
        "orc_prolong": (None, [vp, C.c_int]),
        "orc_coarsest_solve": (None, [vp]),
        "orc_vcycle": (C.c_double, [vp, C.c_int, C.c_int]),
        "orc_pcg": (C.c_int, [vp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, dp]),
        "orc_compliance": (C.c_double, [vp]),
        "orc_volume": (C.c_double, [vp, C.c_int]),
        "orc_sensitivity": (None, [vp]),
        "orc_filter": (None, [vp, C.c_double]),
        "orc_spline_adjoint": (None, [vp]),
        "orc_oc_update": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_int, C.c_int, dp]),
        "orc_gs_maps": (C.c_int, [vp, C.c_int, vp, vp, vp, vp]),
        "orc_set_chebyshev": (None, [vp, C.c_int, C.c_double, C.c_double]),
        "orc_mma_create": (vp, [C.c_int, C.c_int]),
        "orc_mma_destroy": (None, [vp]),
        "orc_mma_set_constraint_amplifier": (None, [vp, C.c_double, C.c_double]),
        "orc_mma_init": (None, [vp, dp, dp]),
        "orc_mma_update": (C.c_int, [vp, dp, dp, dp]),
        "orc_mma_get_x": (None, [vp, dp]),
        "orc_mma_set_x": (None, [vp, dp]),
        "orc_mma_get_stats": (None, [vp, dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ke_template(E: float, nu: float, h: float) -> np.ndarray:
    lib = _load()
    out = np.zeros(576)
    lib.orc_ke_template(E, nu, h, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(24, 24)


class Oracle:
    """One problem instance: grid, hierarchy, BCs, spline and solver state."""

    def __init__(self, nx, ny, nz, h=1.0, E=1e6, nu=0.4, penal=3.0, rho_min=1e-3, eactive=None):
        self.lib = _load()
        self.dims = (nx, ny, nz)
        self.nv = (nx + 1) * (ny + 1) * (nz + 1)
        self.ne = nx * ny * nz
        self.penal = penal
        mask = None
        if eactive is not None:
            self._mask = np.ascontiguousarray(eactive, dtype=np.uint8).ravel()
            mask = self._mask.ctypes.data
        self.h = self.lib.orc_create(nx, ny, nz, h, E, nu, penal, rho_min, mask)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    # --- hierarchy
    def num_levels(self) -> int:
        return self.lib.orc_num_levels(self.h)

    def level_dims(self, level: int):
        d = (C.c_int * 3)()
        self.lib.orc_level_dims(self.h, level, d)
        return tuple(d)

    def level_factor(self, level: int) -> int:
        return self.lib.orc_level_factor(self.h, level)

    # --- set-up
    def set_bc(self, fixed: np.ndarray, loads: np.ndarray):
        fixed = np.ascontiguousarray(fixed, dtype=np.uint8).ravel()
        loads = np.ascontiguousarray(loads, dtype=np.float64).ravel()
        self.lib.orc_set_bc(self.h, fixed.ctypes.data, loads.ctypes.data)

    def set_spline(self, order, partition, bmin, bmax):
        p = (C.c_int * 3)(*partition)
        a = (C.c_double * 3)(*bmin)
        b = (C.c_double * 3)(*bmax)
        self.lib.orc_set_spline(self.h, order, p, a, b)

    def num_coeffs(self) -> int:
        return self.lib.orc_num_coeffs(self.h)

    def knots(self, axis: int, order: int, partition: int) -> np.ndarray:
        out = np.zeros(2 * order + partition)
        self.lib.orc_get_knots(self.h, axis, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def basis(self, axis: int, x: float, order: int):
        """(first basis index or -1, the order basis values) at coordinate x."""
        out = np.zeros(8)
        i0 = self.lib.orc_spline_basis(self.h, axis, float(x), out.ctypes.data_as(C.POINTER(C.c_double)))
        return i0, out[:order]

    # --- arrays
    def get(self, name: str, level: int = 0) -> np.ndarray:
        which = _NAMES[name]
        n = self.lib.orc_size(self.h, which, level)
        dt = np.uint8 if which in (VMASK, EACTIVE) else np.float64
        out = np.zeros(n, dtype=dt)
        self.lib.orc_get(self.h, which, level, out.ctypes.data)
        return out

    def put(self, name: str, arr, level: int = 0):
        which = _NAMES[name]
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        n = self.lib.orc_size(self.h, which, level)
        assert a.size == n, (name, a.size, n)
        self.lib.orc_put(self.h, which, level, a.ctypes.data)

    # --- pipeline
    def coeff_to_density(self):
        self.lib.orc_coeff_to_density(self.h)

    def update_penalised(self):
        self.lib.orc_update_penalised(self.h)

    def update_operators(self):
        self.lib.orc_update_operators(self.h)

    def apply_fine(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        y = np.zeros_like(u)
        self.lib.orc_apply_fine(self.h, u.ctypes.data, y.ctypes.data)
        return y

    def residual(self, level=0):
        self.lib.orc_residual(self.h, level)

    def smooth(self, level, sweeps, reverse=False):
        self.lib.orc_smooth(self.h, level, sweeps, int(reverse))

    def restrict(self, coarse_level):
        self.lib.orc_restrict(self.h, coarse_level)

    def prolong(self, fine_level):
        self.lib.orc_prolong(self.h, fine_level)

    def coarsest_solve(self):
        self.lib.orc_coarsest_solve(self.h)

    def vcycle(self, pre=5, post=5) -> float:
        return self.lib.orc_vcycle(self.h, pre, post)

    def pcg(self, pre=2, post=2, rtol=1e-6, maxit=200, smoother=0):
        rr = C.c_double(0)
        it = self.lib.orc_pcg(self.h, pre, post, rtol, maxit, smoother, C.byref(rr))
        return it, rr.value

    def compliance(self) -> float:
        return self.lib.orc_compliance(self.h)

    def volume(self, reference_denominator=True) -> float:
        return self.lib.orc_volume(self.h, int(reference_denominator))

    def sensitivity(self):
        self.lib.orc_sensitivity(self.h)

    def filter(self, radius):
        self.lib.orc_filter(self.h, radius)

    def spline_adjoint(self):
        self.lib.orc_spline_adjoint(self.h)

    def oc_update(self, vgoal, damp=0.5, step=0.03, cmin=0.0, cmax=1.0, apply_twice=False,
                  reference_denominator=True):
        lam = C.c_double(0)
        t = self.lib.orc_oc_update(self.h, vgoal, damp, step, cmin, cmax, int(apply_twice),
                                   int(reference_denominator), C.byref(lam))
        return t, lam.value

    def gs_maps(self, level=0):
        nva = int((self.get("vmask", level) & 8).astype(bool).sum())
        nea = int(self.get("eactive", level).astype(bool).sum())
        vid = np.zeros(max(nva, 1), dtype=np.int32)
        eid = np.zeros(max(nea, 1), dtype=np.int32)
        gsn = np.zeros(8, dtype=np.int32)
        nge = C.c_int(0)
        ngv = self.lib.orc_gs_maps(self.h, level, vid.ctypes.data, eid.ctypes.data, gsn.ctypes.data,
                                   C.byref(nge))
        return vid[:nva], eid[:nea], gsn, ngv, nge.value

    def set_chebyshev(self, degree=2, lo=0.3, hi=1.1):
        self.lib.orc_set_chebyshev(self.h, degree, lo, hi)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleMMA:
    """CPU restatement of the reference MMA (optimization/mma_t.*): n variables,
    m constraints g_i(x) <= 0, update(df, dg, g) -> converged."""

    def __init__(self, n, m, lb=0.0, ub=1.0):
        self.lib = _load()
        self.n, self.m = n, m
        self.h = self.lib.orc_mma_create(n, m)
        if not self.h:
            raise ValueError("bad MMA size")
        self.init(lb, ub)

    def init(self, lb, ub):
        lb = np.ascontiguousarray(np.broadcast_to(np.asarray(lb, dtype=np.float64), (self.n,)))
        ub = np.ascontiguousarray(np.broadcast_to(np.asarray(ub, dtype=np.float64), (self.n,)))
        self.lib.orc_mma_init(self.h, _dp(lb), _dp(ub))

    def set_constraint_amplifier(self, c, d):
        self.lib.orc_mma_set_constraint_amplifier(self.h, c, d)

    def update(self, df, dg, g) -> bool:
        df = np.ascontiguousarray(df, dtype=np.float64)
        dg = np.ascontiguousarray(np.asarray(dg, dtype=np.float64).reshape(self.m, self.n))
        g = np.ascontiguousarray(np.asarray(g, dtype=np.float64).reshape(self.m))
        return bool(self.lib.orc_mma_update(self.h, _dp(df), _dp(dg), _dp(g)))

    @property
    def x(self) -> np.ndarray:
        out = np.zeros(self.n)
        self.lib.orc_mma_get_x(self.h, _dp(out))
        return out

    @x.setter
    def x(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.lib.orc_mma_set_x(self.h, _dp(v))

    def stats(self) -> dict:
        s = np.zeros(5)
        self.lib.orc_mma_get_stats(self.h, _dp(s))
        return {"subiterations": int(s[0]), "kkt_err": s[1], "step": s[2], "dx_norm": s[3],
                "overflow": bool(s[4])}

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_mma_destroy(self.h)
                self.h = None
        except Exception:
            pass
