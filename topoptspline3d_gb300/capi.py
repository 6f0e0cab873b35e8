"""ctypes binding of the C ABI declared in include/topo_gb300.h.

``Problem`` wraps one ``topo_handle``.  The library is loaded from the in-tree
build (``_lib/libtopo_gb300.so``); there is no fallback: if the CUDA library
cannot be built or loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

TOPO_OK, TOPO_E_CUDA, TOPO_E_BAD_INPUT, TOPO_E_STATE, TOPO_E_NOT_CONVERGED, TOPO_E_SINGULAR, \
    TOPO_E_NOMEM, TOPO_E_NONFINITE, TOPO_E_TIMEOUT = range(9)
STATUS_NAMES = {0: "TOPO_OK", 1: "TOPO_E_CUDA", 2: "TOPO_E_BAD_INPUT", 3: "TOPO_E_STATE",
                4: "TOPO_E_NOT_CONVERGED", 5: "TOPO_E_SINGULAR", 6: "TOPO_E_NOMEM", 7: "TOPO_E_NONFINITE",
                8: "TOPO_E_TIMEOUT"}

ARRAYS = {"rho": 0, "rhop": 1, "coeff": 2, "sens": 3, "csens": 4, "u": 5, "f": 6, "r": 7,
          "stencil": 8, "kelem": 9, "vmask": 10, "eactive": 11, "ke": 12, "work": 13, "volcsens": 14, "multi_f": 15,
          "multi_u": 16, "sscsens": 17, "dripcsens": 18, "rho_init": 19, "surf_points": 20, "surf_normals": 21}
BYTE_ARRAYS = {"vmask", "eactive"}

SOLVE_VCYCLE, SOLVE_PCG64, SOLVE_MIXED = 0, 1, 2
CONV_MMA_SYNC, CONV_TCGEN05 = 0, 1
UNET_IN = 8  # network input channels: r xyz, z xyz (local units), log-density, 0
SMOOTH_GS, SMOOTH_CHEBYSHEV = 0, 1
K_FINE_APPLY64, K_FINE_APPLY32, K_FINE_SMOOTH64, K_FINE_SMOOTH32 = 0, 1, 2, 3

# Every symbol the header declares (checked by the CPU test suite).
EXPORTED = [
    "topo_create", "topo_destroy", "topo_last_error", "topo_num_levels", "topo_level_dims", "topo_sync",
    "topo_set_bc", "topo_set_spline", "topo_num_coeffs", "topo_get_knots", "topo_array_size",
    "topo_put_array", "topo_get_array", "topo_device_ptr", "topo_coeff_to_density",
    "topo_update_operators", "topo_apply_fine", "topo_residual", "topo_smooth", "topo_restrict",
    "topo_prolong", "topo_coarsest_solve", "topo_vcycle", "topo_solve", "topo_compliance",
    "topo_volume", "topo_sensitivity", "topo_filter", "topo_spline_adjoint", "topo_oc_update",
    "topo_gs_maps", "topo_profile_enable", "topo_profile_read", "topo_launch_count",
    "topo_set_operator_precision", "topo_set_reference_precision", "topo_host_alloc", "topo_host_free", "topo_design_iteration",
    "topo_element_template", "topo_plan_levels", "topo_spline_axis", "topo_plan_gs_maps",
    "topo_timer_start", "topo_timer_stop", "topo_spline_adjoint_noalloc", "topo_volume_csens",
    "topo_mma_create", "topo_mma_create_for", "topo_mma_destroy", "topo_mma_last_error", "topo_mma_size",
    "topo_mma_set_constraint_amplifier", "topo_mma_init", "topo_mma_init_uniform", "topo_mma_update",
    "topo_mma_get_x", "topo_mma_read_x", "topo_mma_write_x", "topo_set_bc_regions", "topo_plan_bc_regions",
    "topo_unet_enable", "topo_unet_set_conv_kernel", "topo_unet_num_params", "topo_unet_get_params", "topo_unet_set_params", "topo_unet_forward",
    "topo_unet_loss_grad", "topo_unet_dataset_reserve", "topo_unet_dataset_size", "topo_unet_train",
    "topo_unet_dataset_get", "topo_multi_reserve", "topo_solve_multi", "topo_set_fine_arithmetic", "topo_set_fine_tensor_cores", "topo_apply_level", "topo_set_fine_tile_rows",
    "topo_autotune", "topo_set_graphs", "topo_graph_state", "topo_set_coarse_refresh", "topo_design_batch", "topo_set_tiles", "topo_profiler_range",
    "topo_set_load_region", "topo_worst_compliance", "topo_bitmask_to_eactive", "topo_eactive_to_bitmask",
    "topo_create_bitmask", "topo_write_array", "topo_read_array", "topo_write_active_records",
    "topo_checkpoint_save", "topo_checkpoint_load", "topo_mma_checkpoint_save", "topo_mma_checkpoint_load",
    "topo_voxel_frame", "topo_voxelize_mesh", "topo_heaviside_project", "topo_heaviside_sensitivity",
    "topo_heaviside_volume_csens", "topo_support_constraints",
]


class TopoConfig(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double),
                ("youngs_modulus", C.c_double), ("poisson_ratio", C.c_double),
                ("power_penalty", C.c_double), ("min_density", C.c_double),
                ("max_coarse_elements", C.c_int), ("device", C.c_int)]


class SolveOpts(C.Structure):
    _fields_ = [("mode", C.c_int), ("smoother", C.c_int), ("pre", C.c_int), ("post", C.c_int),
                ("rtol", C.c_double), ("max_iter", C.c_int), ("inner_rtol", C.c_double),
                ("cheb_degree", C.c_int), ("cheb_lo", C.c_double), ("cheb_hi", C.c_double),
                ("inner_max", C.c_int), ("learned", C.c_int), ("learned_stall", C.c_double)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("vcycles", C.c_int), ("relres", C.c_double), ("ms", C.c_double),
                ("learned_applied", C.c_int), ("learned_fallback", C.c_int)]


class OcOpts(C.Structure):
    _fields_ = [("vgoal", C.c_double), ("damp", C.c_double), ("step", C.c_double), ("cmin", C.c_double),
                ("cmax", C.c_double), ("apply_twice", C.c_int), ("reference_volume", C.c_int)]


class OcStats(C.Structure):
    _fields_ = [("trials", C.c_int), ("lambda_", C.c_double), ("volume", C.c_double)]


class IterOpts(C.Structure):
    _fields_ = [("solve", SolveOpts), ("oc", OcOpts), ("filter_radius", C.c_double)]


class IterStats(C.Structure):
    _fields_ = [("compliance", C.c_double), ("volume", C.c_double), ("solve", SolveStats),
                ("oc_trials", C.c_int), ("ms", C.c_double)]


class BatchStats(C.Structure):
    _fields_ = [("wall_ms", C.c_double), ("sum_ms", C.c_double), ("max_ms", C.c_double), ("failures", C.c_int)]


class TuneReport(C.Structure):
    _fields_ = [("tz32", C.c_int), ("tz64", C.c_int), ("cheb_ms", C.c_double * 4), ("apply_ms", C.c_double * 4),
                ("candidates", C.c_int), ("base_ms", C.c_double), ("best_ms", C.c_double), ("tune_ms", C.c_double),
                ("tc", C.c_int), ("cheb_tc_ms", C.c_double * 4), ("rows32", C.c_int),
                ("cheb_rows_ms", (C.c_double * 4) * 2)]


class MultiStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("vcycles", C.c_int), ("max_relres", C.c_double), ("ms", C.c_double)]


class WorstOpts(C.Structure):
    _fields_ = [("solve", SolveOpts), ("free_direction", C.c_int), ("block", C.c_int), ("max_iter", C.c_int),
                ("tol", C.c_double), ("seed", C.c_ulonglong)]


class WorstStats(C.Structure):
    _fields_ = [("compliance", C.c_double), ("second", C.c_double), ("change", C.c_double), ("relres", C.c_double),
                ("iterations", C.c_int), ("solve_iterations", C.c_int), ("ms", C.c_double)]


class SupportOpts(C.Structure):
    _fields_ = [("lattice", C.c_int), ("max_points", C.c_int), ("print_angle", C.c_double), ("ss_mode", C.c_int),
                ("drip_mode", C.c_int), ("beta", C.c_double), ("p_norm", C.c_double), ("hfunction_c", C.c_double),
                ("sigmoid_c", C.c_double), ("drip_beta", C.c_double), ("drip_mu", C.c_double),
                ("drip_angle", C.c_double), ("drip_alpha", C.c_double), ("drip_beta_scale", C.c_double),
                ("drip_version", C.c_int), ("reference_quirks", C.c_int)]


class SupportStats(C.Structure):
    _fields_ = [("candidates", C.c_int), ("points", C.c_int), ("overhang_points", C.c_int), ("flipped", C.c_int),
                ("ss_value", C.c_double), ("drip_value", C.c_double)]


SUPPORT_DEFAULTS = dict(lattice=64, max_points=200000, print_angle=0.75, ss_mode=4, drip_mode=4, beta=4.0,
                        p_norm=0.0, hfunction_c=0.0, sigmoid_c=0.0, drip_beta=0.0, drip_mu=0.0, drip_angle=0.0,
                        drip_alpha=0.0, drip_beta_scale=0.0, drip_version=0, reference_quirks=0)


class MmaStats(C.Structure):
    _fields_ = [("subiterations", C.c_int), ("kkt_err", C.c_double), ("step", C.c_double),
                ("dx_norm", C.c_double), ("overflow", C.c_int), ("converged", C.c_int)]


class TopoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build: bool = True):
    """Load (building first if needed) the CUDA library; raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"libtopo_gb300 not built at {path}")
    lib = C.CDLL(path)
    vp, i, d, ip, dp, sz = C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_size_t
    sigs = {
        "topo_create": (i, [C.POINTER(TopoConfig), vp, C.POINTER(vp)]),
        "topo_destroy": (None, [vp]),
        "topo_last_error": (C.c_char_p, [vp]),
        "topo_num_levels": (i, [vp, ip]),
        "topo_level_dims": (i, [vp, i, ip, ip]),
        "topo_sync": (i, [vp]),
        "topo_set_bc": (i, [vp, vp, vp]),
        "topo_set_spline": (i, [vp, i, ip, dp, dp]),
        "topo_num_coeffs": (i, [vp, ip]),
        "topo_get_knots": (i, [vp, i, dp, sz]),
        "topo_array_size": (i, [vp, i, i, C.POINTER(sz)]),
        "topo_put_array": (i, [vp, i, i, vp, sz]),
        "topo_get_array": (i, [vp, i, i, vp, sz]),
        "topo_device_ptr": (i, [vp, i, i, C.POINTER(vp)]),
        "topo_coeff_to_density": (i, [vp]),
        "topo_set_operator_precision": (i, [vp, i]),
        "topo_set_reference_precision": (i, [vp, i]),
        "topo_update_operators": (i, [vp]),
        "topo_apply_fine": (i, [vp, i]),
        "topo_residual": (i, [vp, i]),
        "topo_smooth": (i, [vp, i, i, i]),
        "topo_restrict": (i, [vp, i]),
        "topo_prolong": (i, [vp, i]),
        "topo_coarsest_solve": (i, [vp]),
        "topo_vcycle": (i, [vp, i, i, dp]),
        "topo_solve": (i, [vp, C.POINTER(SolveOpts), C.POINTER(SolveStats)]),
        "topo_compliance": (i, [vp, dp]),
        "topo_volume": (i, [vp, i, dp]),
        "topo_sensitivity": (i, [vp]),
        "topo_filter": (i, [vp, d]),
        "topo_spline_adjoint": (i, [vp]),
        "topo_oc_update": (i, [vp, C.POINTER(OcOpts), C.POINTER(OcStats)]),
        "topo_gs_maps": (i, [vp, i, vp, sz, vp, sz, vp, ip, ip]),
        "topo_profile_enable": (i, [vp, i]),
        "topo_profile_read": (i, [vp, i, ip, dp]),
        "topo_launch_count": (i, [vp, C.POINTER(C.c_longlong)]),
        "topo_host_alloc": (i, [sz, C.POINTER(vp)]),
        "topo_host_free": (i, [vp]),
        "topo_design_iteration": (i, [vp, C.POINTER(IterOpts), C.POINTER(IterStats)]),
        "topo_element_template": (i, [d, d, d, dp]),
        "topo_plan_levels": (i, [i, i, i, vp, i, i, ip, ip, ip]),
        "topo_spline_axis": (i, [i, i, d, d, i, d, dp, ip, dp]),
        "topo_plan_gs_maps": (i, [i, i, i, vp, i, i, vp, sz, vp, sz, vp, ip, ip]),
        "topo_timer_start": (i, [vp]),
        "topo_timer_stop": (i, [vp, dp]),
        "topo_spline_adjoint_noalloc": (i, [vp, vp, vp]),
        "topo_volume_csens": (i, [vp, i, d, vp]),
        "topo_unet_enable": (i, [vp, C.c_ulonglong]),
        "topo_unet_set_conv_kernel": (i, [vp, i]),
        "topo_multi_reserve": (i, [vp, i]),
        "topo_set_fine_arithmetic": (i, [vp, i]),
        "topo_set_fine_tensor_cores": (i, [vp, i]),
        "topo_apply_level": (i, [vp, i, i]),
        "topo_set_fine_tile_rows": (i, [vp, i]),
        "topo_set_graphs": (i, [vp, i]),
        "topo_graph_state": (i, [vp, ip]),
        "topo_set_coarse_refresh": (i, [vp, i]),
        "topo_set_tiles": (i, [vp, i, i]),
        "topo_profiler_range": (i, [i]),
        "topo_design_batch": (i, [C.POINTER(vp), i, C.POINTER(IterOpts), i, i, i, C.POINTER(IterStats),
                                  C.POINTER(BatchStats)]),
        "topo_autotune": (i, [vp, C.POINTER(SolveOpts), C.POINTER(SolveOpts), C.POINTER(TuneReport)]),
        "topo_solve_multi": (i, [vp, i, C.POINTER(SolveOpts), C.POINTER(MultiStats), dp]),
        "topo_unet_num_params": (i, [C.POINTER(sz)]),
        "topo_unet_get_params": (i, [vp, vp, sz]),
        "topo_unet_set_params": (i, [vp, vp, sz]),
        "topo_unet_forward": (i, [vp, i, i, i, i, vp, vp]),
        "topo_unet_loss_grad": (i, [vp, i, i, i, i, vp, vp, vp, dp, vp]),
        "topo_unet_dataset_reserve": (i, [vp, i, i, i]),
        "topo_unet_dataset_size": (i, [vp, ip]),
        "topo_unet_dataset_get": (i, [vp, i, vp, vp, vp, ip]),
        "topo_unet_train": (i, [vp, i, i, d, C.c_ulonglong, i, i, i, dp]),
        "topo_set_bc_regions": (i, [vp, vp, ip, ip]),
        "topo_plan_bc_regions": (i, [i, i, i, vp, vp, vp, vp, ip, ip]),
        "topo_set_load_region": (i, [vp, i, ip, dp]),
        "topo_worst_compliance": (i, [vp, C.POINTER(WorstOpts), C.POINTER(WorstStats)]),
        "topo_heaviside_project": (i, [vp, d]),
        "topo_heaviside_sensitivity": (i, [vp, d]),
        "topo_heaviside_volume_csens": (i, [vp, d, i, d, d, vp]),
        "topo_support_constraints": (i, [vp, C.POINTER(SupportOpts), C.POINTER(SupportStats)]),
        "topo_voxel_frame": (i, [vp, i, i, ip, vp]),
        "topo_voxelize_mesh": (i, [i, vp, i, vp, i, i, ip, vp, vp, sz]),
        "topo_bitmask_to_eactive": (i, [ip, vp, i, i, i, vp]),
        "topo_eactive_to_bitmask": (i, [i, i, i, vp, ip, vp]),
        "topo_create_bitmask": (i, [C.POINTER(TopoConfig), ip, vp, C.POINTER(vp)]),
        "topo_write_array": (i, [vp, i, i, C.c_char_p, i]),
        "topo_read_array": (i, [vp, i, i, C.c_char_p, i]),
        "topo_write_active_records": (i, [vp, i, C.c_char_p, C.POINTER(C.c_int64)]),
        "topo_checkpoint_save": (i, [vp, C.c_char_p, vp, sz]),
        "topo_checkpoint_load": (i, [vp, C.c_char_p, vp, sz, C.POINTER(sz)]),
        "topo_mma_checkpoint_save": (i, [vp, C.c_char_p]),
        "topo_mma_checkpoint_load": (i, [vp, C.c_char_p]),
        "topo_mma_create": (i, [i, i, i, C.POINTER(vp)]),
        "topo_mma_create_for": (i, [vp, i, C.POINTER(vp)]),
        "topo_mma_destroy": (None, [vp]),
        "topo_mma_last_error": (C.c_char_p, [vp]),
        "topo_mma_size": (i, [vp, ip, ip]),
        "topo_mma_set_constraint_amplifier": (i, [vp, d, d]),
        "topo_mma_init": (i, [vp, dp, dp]),
        "topo_mma_init_uniform": (i, [vp, d, d]),
        "topo_mma_update": (i, [vp, vp, C.POINTER(vp), dp, C.POINTER(MmaStats)]),
        "topo_mma_get_x": (i, [vp, vp]),
        "topo_mma_read_x": (i, [vp, dp]),
        "topo_mma_write_x": (i, [vp, dp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ck_free(rc, what):
    if rc != TOPO_OK:
        raise TopoError(rc, what)


def profiler_range(start: bool) -> None:
    """Open or close the profiler's capture range (cudaProfilerStart/Stop)."""
    _ck_free(load(build=False).topo_profiler_range(int(bool(start))), "topo_profiler_range")


def element_template(E, nu, h) -> np.ndarray:
    """Host-only: the library's 24x24 element template."""
    lib = load()
    out = np.zeros(576)
    _ck_free(lib.topo_element_template(E, nu, h, out.ctypes.data_as(C.POINTER(C.c_double))), "element_template")
    return out.reshape(24, 24)


def plan_levels(nx, ny, nz, eactive=None, max_coarse=400):
    """Host-only: element dims and coarsening factors of the multigrid levels."""
    lib = load()
    dims = np.zeros(3 * 16, dtype=np.int32)
    fac = np.zeros(16, dtype=np.int32)
    n = C.c_int()
    m = None
    if eactive is not None:
        ea = np.ascontiguousarray(eactive, dtype=np.uint8).ravel()
        m = ea.ctypes.data
    _ck_free(lib.topo_plan_levels(nx, ny, nz, m, max_coarse, 16, C.byref(n), dims.ctypes.data_as(C.POINTER(C.c_int)),
                                  fac.ctypes.data_as(C.POINTER(C.c_int))), "plan_levels")
    return [tuple(dims[3 * l:3 * l + 3]) for l in range(n.value)], list(fac[:n.value])


def spline_axis(order, partition, bmin, bmax, nelem, h=1.0):
    """Host-only: knots, first basis index per element slice and basis values."""
    lib = load()
    knots = np.zeros(2 * order + partition)
    i0 = np.zeros(nelem, dtype=np.int32)
    N = np.zeros(nelem * order)
    _ck_free(lib.topo_spline_axis(order, partition, bmin, bmax, nelem, h, knots.ctypes.data_as(C.POINTER(C.c_double)),
                                  i0.ctypes.data_as(C.POINTER(C.c_int)), N.ctypes.data_as(C.POINTER(C.c_double))),
             "spline_axis")
    return knots, i0, N.reshape(nelem, order)


def plan_gs_maps(nx, ny, nz, level=0, eactive=None, max_coarse=400):
    """Host-only: the reference's GS-coloured ordering of one level."""
    lib = load()
    m, ea = None, None
    if eactive is not None:
        ea = np.ascontiguousarray(eactive, dtype=np.uint8).ravel()
        m = ea.ctypes.data
    gsn = np.zeros(8, dtype=np.int32)
    ngv, nge = C.c_int(), C.c_int()
    _ck_free(lib.topo_plan_gs_maps(nx, ny, nz, m, max_coarse, level, None, 0, None, 0, gsn.ctypes.data,
                                   C.byref(ngv), C.byref(nge)), "plan_gs_maps")
    # active counts: padded colour sizes bound them; ask with exact sizes by counting actives
    dims, facs = plan_levels(nx, ny, nz, eactive, max_coarse)
    ex, ey, ez = (int(v) for v in dims[level])
    eact = _plan_eactive(nx, ny, nz, ea, dims, facs, level)
    vact = np.zeros((ez + 1, ey + 1, ex + 1), bool)
    e3 = eact.reshape(ez, ey, ex)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                vact[dz:dz + ez, dy:dy + ey, dx:dx + ex] |= e3
    nva, nea = int(vact.sum()), int(eact.sum())
    vid = np.zeros(max(nva, 1), dtype=np.int32)
    eid = np.zeros(max(nea, 1), dtype=np.int32)
    _ck_free(lib.topo_plan_gs_maps(nx, ny, nz, m, max_coarse, level, vid.ctypes.data, nva, eid.ctypes.data, nea,
                                   gsn.ctypes.data, C.byref(ngv), C.byref(nge)), "plan_gs_maps")
    return vid[:nva], eid[:nea], gsn, ngv.value, nge.value


def _plan_eactive(nx, ny, nz, ea, dims, facs, level):
    """Active-element mask of a planned level (child-OR of the fine mask)."""
    cur = np.ones((nz, ny, nx), bool) if ea is None else ea.reshape(nz, ny, nx).astype(bool)
    for l in range(1, level + 1):
        cx, cy, cz = (int(v) for v in dims[l])
        f = int(facs[l])
        pad = np.zeros((cz * f, cy * f, cx * f), bool)
        pad[:cur.shape[0], :cur.shape[1], :cur.shape[2]] = cur
        cur = pad.reshape(cz, f, cy, f, cx, f).any(axis=(1, 3, 5))
    return cur.ravel()


class PinnedBuffer:
    """Page-locked host buffer from topo_host_alloc, viewed as a numpy array."""

    def __init__(self, n, dtype=np.float64):
        self.lib = load()
        self.nbytes = int(n) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        _ck_free(self.lib.topo_host_alloc(self.nbytes, C.byref(p)), "topo_host_alloc")
        self.ptr = p.value
        self.array = np.frombuffer((C.c_char * self.nbytes).from_address(self.ptr), dtype=dtype)

    def close(self):
        if self.ptr:
            self.array = None
            self.lib.topo_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bitmask_to_eactive(reso, words, nx, ny, nz) -> np.ndarray:
    """Host-only: the reference's LSB-first uint32 domain bit mask over a reso
    frame -> element mask of the nx x ny x nz box at its origin."""
    lib = load()
    r = (C.c_int * 3)(*reso)
    w = np.ascontiguousarray(words, dtype=np.uint32)
    out = np.zeros(nx * ny * nz, dtype=np.uint8)
    _ck_free(lib.topo_bitmask_to_eactive(r, w.ctypes.data, nx, ny, nz, out.ctypes.data), "bitmask_to_eactive")
    return out


def eactive_to_bitmask(nx, ny, nz, eactive, reso) -> np.ndarray:
    """Host-only: element mask -> LSB-first uint32 words over the reso frame."""
    lib = load()
    r = (C.c_int * 3)(*reso)
    ea = None if eactive is None else np.ascontiguousarray(eactive, dtype=np.uint8).ravel()
    out = np.zeros((int(np.prod(reso)) + 31) // 32, dtype=np.uint32)
    _ck_free(lib.topo_eactive_to_bitmask(nx, ny, nz, None if ea is None else ea.ctypes.data, r, out.ctypes.data),
             "eactive_to_bitmask")
    return out


def voxel_frame(verts, preferred_resolution):
    """Host-only: (resolution, box[6]) of the voxelisation frame of a mesh."""
    lib = load()
    v = np.ascontiguousarray(verts, dtype=np.float32).ravel()
    r = C.c_int()
    box = np.zeros(6, dtype=np.float32)
    _ck_free(lib.topo_voxel_frame(v.ctypes.data, v.size // 3, int(preferred_resolution), C.byref(r), box.ctypes.data),
             "voxel_frame")
    return r.value, box


def voxelize_mesh(verts, tris, preferred_resolution, device=0):
    """Solid voxelisation on the GPU: (resolution, box[6], LSB-first uint32 words)."""
    lib = load()
    v = np.ascontiguousarray(verts, dtype=np.float32).ravel()
    t = np.ascontiguousarray(tris, dtype=np.int32).ravel()
    reso, box = voxel_frame(v, preferred_resolution)
    words = np.zeros((reso ** 3 + 31) // 32, dtype=np.uint32)
    r = C.c_int()
    _ck_free(lib.topo_voxelize_mesh(device, v.ctypes.data, v.size // 3, t.ctypes.data, t.size // 3,
                                    int(preferred_resolution), C.byref(r), box.ctypes.data, words.ctypes.data,
                                    words.size), "voxelize_mesh")
    return r.value, box, words


class Problem:
    """One topology-optimisation problem on one GPU (wraps ``topo_handle``)."""

    def __init__(self, nx, ny, nz, h=1.0, E=1e6, nu=0.4, penal=3.0, rho_min=1e-3, eactive=None,
                 max_coarse_elements=400, device=0, bitmask=None):
        """bitmask = (reso[3], uint32 words): the reference's domain input
        (topo_create_bitmask) instead of eactive."""
        self.lib = load()
        self.dims = (nx, ny, nz)
        self.nv = (nx + 1) * (ny + 1) * (nz + 1)
        self.ne = nx * ny * nz
        cfg = TopoConfig(nx, ny, nz, h, E, nu, penal, rho_min, max_coarse_elements, device)
        hp = C.c_void_p()
        if bitmask is not None:
            reso, words = bitmask
            self._words = np.ascontiguousarray(words, dtype=np.uint32)
            rc = self.lib.topo_create_bitmask(C.byref(cfg), (C.c_int * 3)(*reso), self._words.ctypes.data,
                                              C.byref(hp))
        else:
            mask = None
            if eactive is not None:
                self._mask = np.ascontiguousarray(eactive, dtype=np.uint8).ravel()
                assert self._mask.size == self.ne
                mask = self._mask.ctypes.data
            rc = self.lib.topo_create(C.byref(cfg), mask, C.byref(hp))
        if rc != TOPO_OK:
            raise TopoError(rc, "topo_create failed")
        self.h = hp

    def close(self):
        if getattr(self, "h", None):
            self.lib.topo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != TOPO_OK:
            raise TopoError(rc, self.lib.topo_last_error(self.h).decode())
        return rc

    def last_error(self) -> str:
        """The handle's last recorded message (errors, and fallbacks such as a graph not captured)."""
        return self.lib.topo_last_error(self.h).decode()

    # --- hierarchy
    def num_levels(self) -> int:
        n = C.c_int()
        self._ck(self.lib.topo_num_levels(self.h, C.byref(n)))
        return n.value

    def level_dims(self, level):
        d = (C.c_int * 3)()
        f = C.c_int()
        self._ck(self.lib.topo_level_dims(self.h, level, d, C.byref(f)))
        return tuple(d), f.value

    # --- set-up
    def set_bc(self, fixed, loads):
        fixed = np.ascontiguousarray(fixed, dtype=np.uint8).ravel()
        loads = np.ascontiguousarray(loads, dtype=np.float64).ravel()
        assert fixed.size == self.nv and loads.size == 3 * self.nv
        self._ck(self.lib.topo_set_bc(self.h, fixed.ctypes.data, loads.ctypes.data))

    def set_bc_regions(self, spec):
        """Boundary conditions from a parsed region spec (bc_regions.parse):
        returns (support vertices, load vertices)."""
        nf, nl = C.c_int(), C.c_int()
        self._ck(self.lib.topo_set_bc_regions(self.h, C.byref(spec.c), C.byref(nf), C.byref(nl)))
        return nf.value, nl.value

    def set_spline(self, order, partition, bmin, bmax):
        p = (C.c_int * 3)(*partition)
        a = (C.c_double * 3)(*bmin)
        b = (C.c_double * 3)(*bmax)
        self._ck(self.lib.topo_set_spline(self.h, order, p, a, b))

    def num_coeffs(self) -> int:
        n = C.c_int()
        self._ck(self.lib.topo_num_coeffs(self.h, C.byref(n)))
        return n.value

    def knots(self, axis, count):
        out = np.zeros(count)
        self._ck(self.lib.topo_get_knots(self.h, axis, out.ctypes.data_as(C.POINTER(C.c_double)), count))
        return out

    # --- arrays
    def size(self, name, level=0) -> int:
        n = C.c_size_t()
        self._ck(self.lib.topo_array_size(self.h, ARRAYS[name], level, C.byref(n)))
        return n.value

    def get(self, name, level=0) -> np.ndarray:
        n = self.size(name, level)
        out = np.zeros(n, dtype=np.uint8 if name in BYTE_ARRAYS else np.float64)
        self._ck(self.lib.topo_get_array(self.h, ARRAYS[name], level, out.ctypes.data, n))
        return out

    def put(self, name, arr, level=0):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        self._ck(self.lib.topo_put_array(self.h, ARRAYS[name], level, a.ctypes.data, a.size))

    def device_ptr(self, name, level=0) -> int:
        p = C.c_void_p()
        self._ck(self.lib.topo_device_ptr(self.h, ARRAYS[name], level, C.byref(p)))
        return p.value

    # --- hot path
    def coeff_to_density(self):
        self._ck(self.lib.topo_coeff_to_density(self.h))

    def set_tiles(self, tz32, tz64):
        self._ck(self.lib.topo_set_tiles(self.h, tz32, tz64))

    def set_graphs(self, enable):
        self._ck(self.lib.topo_set_graphs(self.h, int(enable)))

    def set_coarse_refresh(self, every):
        """Recompute the coarsest inverse at every `every`-th operator update (1: each)."""
        self._ck(self.lib.topo_set_coarse_refresh(self.h, int(every)))

    def graph_state(self):
        """The graphs the handle holds: {"vcycle", "inner", "solve", "nested_inner", "oc",
        "iteration"} -> bool."""
        st = C.c_int()
        self._ck(self.lib.topo_graph_state(self.h, C.byref(st)))
        names = ("vcycle", "inner", "solve", "nested_inner", "oc", "iteration")
        return {n: bool(st.value >> k & 1) for k, n in enumerate(names)}

    def set_fine_arithmetic(self, arith):
        """0: native FP64 fine operator, 1: double-float (default)."""
        self._ck(self.lib.topo_set_fine_arithmetic(self.h, arith))

    def set_fine_tile_rows(self, rows):
        """Element rows (4, 8, 16) of the FP32 modal fine kernels' CTA tile."""
        self._ck(self.lib.topo_set_fine_tile_rows(self.h, rows))

    def set_fine_tensor_cores(self, on):
        """FP32 fine element products on the tcgen05 tensor cores (three-term TF32)."""
        self._ck(self.lib.topo_set_fine_tensor_cores(self.h, int(bool(on))))

    def set_operator_precision(self, mask):
        self._ck(self.lib.topo_set_operator_precision(self.h, mask))

    def set_reference_precision(self, enable):
        """1: rho, coefficients and sensitivities kept at FP32 values, rho^p by powf (the reference's storage)."""
        self._ck(self.lib.topo_set_reference_precision(self.h, int(enable)))

    def update_operators(self):
        self._ck(self.lib.topo_update_operators(self.h))

    def apply_fine(self, u, precision=0) -> np.ndarray:
        self.put("work", u)
        self._ck(self.lib.topo_apply_fine(self.h, precision))
        return self.get("r")

    def apply_level(self, level, u, precision=0) -> np.ndarray:
        """A_level u on a coarse level (>= 1): precision 0 FP64 operator, 1 FP32."""
        self.put("u", u, level)
        self._ck(self.lib.topo_apply_level(self.h, level, precision))
        return self.get("r", level)

    def residual(self, level=0):
        self._ck(self.lib.topo_residual(self.h, level))

    def smooth(self, level, sweeps, reverse=False):
        self._ck(self.lib.topo_smooth(self.h, level, sweeps, int(reverse)))

    def restrict(self, coarse_level):
        self._ck(self.lib.topo_restrict(self.h, coarse_level))

    def prolong(self, fine_level):
        self._ck(self.lib.topo_prolong(self.h, fine_level))

    def coarsest_solve(self):
        self._ck(self.lib.topo_coarsest_solve(self.h))

    def vcycle(self, pre=5, post=5) -> float:
        rr = C.c_double()
        self._ck(self.lib.topo_vcycle(self.h, pre, post, C.byref(rr)))
        return rr.value

    def solve(self, mode=SOLVE_PCG64, smoother=SMOOTH_GS, pre=2, post=2, rtol=1e-6, max_iter=200,
              inner_rtol=1e-1, cheb_degree=2, cheb_lo=0.3, cheb_hi=1.1, inner_max=1, learned=0,
              learned_stall=0.0, check=True):
        o = SolveOpts(mode, smoother, pre, post, rtol, max_iter, inner_rtol, cheb_degree, cheb_lo, cheb_hi,
                      inner_max, learned, learned_stall)
        s = SolveStats()
        rc = self.lib.topo_solve(self.h, C.byref(o), C.byref(s))
        if check:
            self._ck(rc)
        return {"iterations": s.iterations, "vcycles": s.vcycles, "relres": s.relres, "ms": s.ms, "rc": rc,
                "learned_applied": s.learned_applied, "learned_fallback": bool(s.learned_fallback)}

    # --- autotuner

    def autotune(self, base=None):
        """Tile (z-march depth) and solver-schedule tuning on the current state.
        Returns (best solve-options dict, report dict)."""
        b = dict(mode=SOLVE_MIXED, smoother=SMOOTH_CHEBYSHEV, pre=2, post=2, rtol=1e-6, max_iter=300,
                 inner_rtol=0.1, cheb_degree=2, cheb_lo=0.3, cheb_hi=1.1, inner_max=4, learned=0,
                 learned_stall=0.0)
        b.update(base or {})
        keys = [f[0] for f in SolveOpts._fields_]
        o = SolveOpts(*[b[k] for k in keys])
        best = SolveOpts()
        r = TuneReport()
        self._ck(self.lib.topo_autotune(self.h, C.byref(o), C.byref(best), C.byref(r)))
        bd = {k: getattr(best, k) for k in keys}
        rep = {"tz32": r.tz32, "tz64": r.tz64, "cheb_ms": list(r.cheb_ms), "apply_ms": list(r.apply_ms),
               "candidates": r.candidates, "base_ms": r.base_ms, "best_ms": r.best_ms, "tune_ms": r.tune_ms,
               "tc": r.tc, "cheb_tc_ms": list(r.cheb_tc_ms), "rows32": r.rows32,
               "cheb_rows_ms": {4: list(r.cheb_rows_ms[0]), 16: list(r.cheb_rows_ms[1])}}
        return bd, rep

    # --- many load cases

    def multi_reserve(self, capacity):
        self._ck(self.lib.topo_multi_reserve(self.h, capacity))
        self._multi_cap = capacity

    def solve_multi(self, F, U0=None, pre=2, post=2, rtol=1e-6, max_iter=200, cheb_degree=2, cheb_lo=0.3,
                    cheb_hi=1.1, inner_max=1, inner_rtol=0.1, check=True):
        """F [nrhs][3*nv] host right-hand sides -> (U [nrhs][3*nv], stats, relres[nrhs]).
        inner_max > 1: each outer step runs that many batched FP32 CG iterations
        (to inner_rtol per right-hand side) preconditioned by the V-cycle."""
        F = np.ascontiguousarray(F, dtype=np.float64)
        nrhs = F.shape[0]
        cap = self._multi_cap
        full = np.zeros((cap, 3 * self.nv))
        full[:nrhs] = F
        self.put("multi_f", full.ravel())
        u = np.zeros((cap, 3 * self.nv))
        if U0 is not None:
            u[:nrhs] = U0
        self.put("multi_u", u.ravel())
        o = SolveOpts(SOLVE_MIXED, SMOOTH_CHEBYSHEV, pre, post, rtol, max_iter, inner_rtol, cheb_degree, cheb_lo,
                      cheb_hi, inner_max, 0, 0.0)
        st = MultiStats()
        rel = np.zeros(nrhs)
        rc = self.lib.topo_solve_multi(self.h, nrhs, C.byref(o), C.byref(st), rel.ctypes.data_as(C.POINTER(C.c_double)))
        if check:
            self._ck(rc)
        U = self.get("multi_u").reshape(cap, 3 * self.nv)[:nrhs].copy()
        return U, {"iterations": st.iterations, "vcycles": st.vcycles, "max_relres": st.max_relres, "ms": st.ms,
                   "rc": rc}, rel

    # --- learned preconditioner

    def unet_enable(self, seed=1):
        self._ck(self.lib.topo_unet_enable(self.h, seed))

    def unet_set_conv_kernel(self, kind):
        """CONV_MMA_SYNC (default) or CONV_TCGEN05 for the network's convolutions."""
        self._ck(self.lib.topo_unet_set_conv_kernel(self.h, kind))

    @staticmethod
    def unet_num_params() -> int:
        n = C.c_size_t()
        _ck_free(load().topo_unet_num_params(C.byref(n)), "topo_unet_num_params")
        return n.value

    def unet_params(self) -> np.ndarray:
        n = self.unet_num_params()
        out = np.zeros(n, dtype=np.float32)
        self._ck(self.lib.topo_unet_get_params(self.h, out.ctypes.data, n))
        return out

    def unet_set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._ck(self.lib.topo_unet_set_params(self.h, p.ctypes.data, p.size))

    def unet_forward(self, x):
        """x [nb, Z, Y, X, 8] float32 (r xyz, z xyz, log-density, 0) -> [nb, Z, Y, X, 3]."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        nb, Z, Y, X, _ = x.shape
        y = np.zeros((nb, Z, Y, X, 3), dtype=np.float32)
        self._ck(self.lib.topo_unet_forward(self.h, X, Y, Z, nb, x.ctypes.data, y.ctypes.data))
        return y

    def unet_loss_grad(self, x, t, m):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        m = np.ascontiguousarray(m, dtype=np.uint8)
        nb, Z, Y, X, _ = x.shape
        g = np.zeros(self.unet_num_params(), dtype=np.float32)
        loss = C.c_double()
        self._ck(self.lib.topo_unet_loss_grad(self.h, X, Y, Z, nb, x.ctypes.data, t.ctypes.data, m.ctypes.data,
                                              C.byref(loss), g.ctypes.data))
        return loss.value, g

    def unet_dataset_reserve(self, capacity, crop=32, crops_per_iterate=64):
        self._ck(self.lib.topo_unet_dataset_reserve(self.h, capacity, crop, crops_per_iterate))

    def unet_dataset_size(self) -> int:
        n = C.c_int()
        self._ck(self.lib.topo_unet_dataset_size(self.h, C.byref(n)))
        return n.value

    def unet_dataset_get(self, slot, crop=32):
        per = crop ** 3
        x = np.zeros((per, UNET_IN), dtype=np.float32)
        t = np.zeros((per, 3), dtype=np.float32)
        m = np.zeros(per, dtype=np.uint8)
        side = C.c_int()
        self._ck(self.lib.topo_unet_dataset_get(self.h, slot, x.ctypes.data, t.ctypes.data, m.ctypes.data,
                                                C.byref(side)))
        assert side.value == crop
        s3 = (crop, crop, crop)
        return x.reshape(s3 + (UNET_IN,)), t.reshape(s3 + (3,)), m.reshape(s3)

    def unet_train(self, steps, batch=8, lr=1e-3, seed=1, lo=0, hi=0, update=True) -> float:
        loss = C.c_double()
        self._ck(self.lib.topo_unet_train(self.h, steps, batch, lr, seed, lo, hi, int(update), C.byref(loss)))
        return loss.value

    def set_load_region(self, vertices, normals=None):
        """Load region of the worst-case compliance: level-0 vertex ids and (for
        loads along the normal) their outward normals [n][3]."""
        v = np.ascontiguousarray(vertices, dtype=np.int32).ravel()
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float64).ravel()
        self._ck(self.lib.topo_set_load_region(self.h, int(v.size), v.ctypes.data_as(C.POINTER(C.c_int)),
                                               None if nrm is None else nrm.ctypes.data_as(C.POINTER(C.c_double))))

    def worst_compliance(self, block=8, free_direction=False, max_iter=100, tol=1e-4, seed=1, check=True, **solve):
        """Worst-case compliance over unit loads on the load region; leaves the
        worst load in F and its displacement in U."""
        so = dict(mode=SOLVE_MIXED, smoother=SMOOTH_CHEBYSHEV, pre=1, post=1, rtol=1e-6, max_iter=300,
                  inner_rtol=0.1, cheb_degree=2, cheb_lo=0.3, cheb_hi=1.1, inner_max=1, learned=0, learned_stall=0.0)
        so.update(solve)
        o = WorstOpts(SolveOpts(*[so[f[0]] for f in SolveOpts._fields_]), int(bool(free_direction)), int(block),
                      int(max_iter), float(tol), int(seed))
        st = WorstStats()
        rc = self.lib.topo_worst_compliance(self.h, C.byref(o), C.byref(st))
        if check or rc not in (TOPO_OK, TOPO_E_NOT_CONVERGED):
            self._ck(rc)
        return {"compliance": st.compliance, "second": st.second, "change": st.change, "relres": st.relres,
                "iterations": st.iterations, "solve_iterations": st.solve_iterations, "ms": st.ms, "rc": rc}

    # --- Heaviside projection and manufacturing constraints
    def heaviside_project(self, beta):
        self._ck(self.lib.topo_heaviside_project(self.h, float(beta)))

    def heaviside_sensitivity(self, beta):
        self._ck(self.lib.topo_heaviside_sensitivity(self.h, float(beta)))

    def heaviside_volume_csens(self, beta, filter_radius=2.0, scale=1.0, reference_denominator=True, dst_ptr=None):
        self._ck(self.lib.topo_heaviside_volume_csens(self.h, float(beta), int(bool(reference_denominator)),
                                                      float(filter_radius), float(scale), dst_ptr))

    def support_constraints(self, **opts):
        """Self-support and drip constraint values; gradients in "sscsens" / "dripcsens",
        points and normals in "surf_points" / "surf_normals"."""
        o = dict(SUPPORT_DEFAULTS)
        o.update(opts)
        so = SupportOpts(*[o[f[0]] for f in SupportOpts._fields_])
        st = SupportStats()
        self._ck(self.lib.topo_support_constraints(self.h, C.byref(so), C.byref(st)))
        return {f[0]: getattr(st, f[0]) for f in SupportStats._fields_}

    # --- files and checkpoints
    def write_array(self, name, path, fp32=False, level=0):
        """Raw record of an array (bio::write_vector); fp32 as the reference's writeCoeff."""
        self._ck(self.lib.topo_write_array(self.h, ARRAYS[name], level, os.fsencode(path), int(bool(fp32))))

    def read_array(self, name, path, fp32=False, level=0):
        self._ck(self.lib.topo_read_array(self.h, ARRAYS[name], level, os.fsencode(path), int(bool(fp32))))

    def write_active_records(self, name, path) -> int:
        """(x, y, z, value) FP32 records of the active elements (density or sensitivity)."""
        n = C.c_int64()
        self._ck(self.lib.topo_write_active_records(self.h, ARRAYS[name], os.fsencode(path), C.byref(n)))
        return n.value

    def checkpoint_save(self, path, user=b""):
        buf = C.create_string_buffer(bytes(user), max(len(user), 1))
        self._ck(self.lib.topo_checkpoint_save(self.h, os.fsencode(path), buf, len(user)))

    def checkpoint_load(self, path, user_cap=4096) -> bytes:
        buf = C.create_string_buffer(max(user_cap, 1))
        n = C.c_size_t()
        self._ck(self.lib.topo_checkpoint_load(self.h, os.fsencode(path), buf, user_cap, C.byref(n)))
        return buf.raw[:min(n.value, user_cap)]

    def compliance(self) -> float:
        c = C.c_double()
        self._ck(self.lib.topo_compliance(self.h, C.byref(c)))
        return c.value

    def volume(self, reference_denominator=True) -> float:
        v = C.c_double()
        self._ck(self.lib.topo_volume(self.h, int(reference_denominator), C.byref(v)))
        return v.value

    def sensitivity(self):
        self._ck(self.lib.topo_sensitivity(self.h))

    def filter(self, radius):
        self._ck(self.lib.topo_filter(self.h, radius))

    def spline_adjoint(self):
        self._ck(self.lib.topo_spline_adjoint(self.h))

    def volume_csens(self, dst_ptr=None, scale=1.0, reference_denominator=True):
        """scale * d volume / d coefficient into the device buffer at dst_ptr
        (None: the handle's "volcsens" array)."""
        self._ck(self.lib.topo_volume_csens(self.h, int(reference_denominator), scale,
                                            C.c_void_p(dst_ptr) if dst_ptr else None))

    def oc_update(self, vgoal, damp=0.5, step=0.03, cmin=0.0, cmax=1.0, apply_twice=False,
                  reference_denominator=True):
        o = OcOpts(vgoal, damp, step, cmin, cmax, int(apply_twice), int(reference_denominator))
        s = OcStats()
        self._ck(self.lib.topo_oc_update(self.h, C.byref(o), C.byref(s)))
        return s.trials, s.lambda_

    def gs_maps(self, level=0):
        vm = self.get("vmask", level)
        nva = int(((vm & 8) != 0).sum())
        nea = int((self.get("eactive", level) != 0).sum())
        vid = np.zeros(max(nva, 1), dtype=np.int32)
        eid = np.zeros(max(nea, 1), dtype=np.int32)
        gsn = np.zeros(8, dtype=np.int32)
        ngv, nge = C.c_int(), C.c_int()
        self._ck(self.lib.topo_gs_maps(self.h, level, vid.ctypes.data, nva, eid.ctypes.data, nea,
                                       gsn.ctypes.data, C.byref(ngv), C.byref(nge)))
        return vid[:nva], eid[:nea], gsn, ngv.value, nge.value

    def profile_enable(self, on=True):
        self._ck(self.lib.topo_profile_enable(self.h, int(on)))

    def profile_read(self, family):
        n, ms = C.c_int(), C.c_double()
        self._ck(self.lib.topo_profile_read(self.h, family, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def launch_count(self) -> int:
        n = C.c_longlong()
        self._ck(self.lib.topo_launch_count(self.h, C.byref(n)))
        return n.value

    def sync(self):
        self._ck(self.lib.topo_sync(self.h))

    def timer_start(self):
        self._ck(self.lib.topo_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._ck(self.lib.topo_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def put_from(self, name, host_ptr, count, level=0):
        """Copy ``count`` elements from a raw host pointer (e.g. pinned memory)."""
        self._ck(self.lib.topo_put_array(self.h, ARRAYS[name], level, host_ptr, count))

    def get_into(self, name, host_ptr, count, level=0):
        self._ck(self.lib.topo_get_array(self.h, ARRAYS[name], level, host_ptr, count))

    @staticmethod
    def iter_opts(solve=None, oc=None, filter_radius=2.0):
        s = dict(mode=SOLVE_MIXED, smoother=SMOOTH_GS, pre=2, post=2, rtol=1e-6, max_iter=200,
                 inner_rtol=1e-1, cheb_degree=2, cheb_lo=0.3, cheb_hi=1.1, inner_max=1, learned=0,
                 learned_stall=0.0)
        s.update(solve or {})
        c = dict(vgoal=0.4, damp=0.5, step=0.03, cmin=0.0, cmax=1.0, apply_twice=0, reference_volume=1)
        c.update(oc or {})
        keys = [f[0] for f in SolveOpts._fields_]
        return IterOpts(SolveOpts(*[s[k] for k in keys]),
                        OcOpts(c["vgoal"], c["damp"], c["step"], c["cmin"], c["cmax"], int(c["apply_twice"]),
                               int(c["reference_volume"])), filter_radius)

    def design_iteration(self, solve=None, oc=None, filter_radius=2.0):
        s = dict(mode=SOLVE_MIXED, smoother=SMOOTH_GS, pre=2, post=2, rtol=1e-6, max_iter=200,
                 inner_rtol=1e-1, cheb_degree=2, cheb_lo=0.3, cheb_hi=1.1, inner_max=1, learned=0,
                 learned_stall=0.0)
        s.update(solve or {})
        c = dict(vgoal=0.4, damp=0.5, step=0.03, cmin=0.0, cmax=1.0, apply_twice=0, reference_volume=1)
        c.update(oc or {})
        o = IterOpts(SolveOpts(s["mode"], s["smoother"], s["pre"], s["post"], s["rtol"], s["max_iter"],
                               s["inner_rtol"], s["cheb_degree"], s["cheb_lo"], s["cheb_hi"], s["inner_max"],
                               s["learned"], s["learned_stall"]),
                     OcOpts(c["vgoal"], c["damp"], c["step"], c["cmin"], c["cmax"], int(c["apply_twice"]),
                            int(c["reference_volume"])), filter_radius)
        st = IterStats()
        rc = self.lib.topo_design_iteration(self.h, C.byref(o), C.byref(st))
        if rc not in (TOPO_OK, TOPO_E_NOT_CONVERGED):
            self._ck(rc)
        return {"compliance": st.compliance, "volume": st.volume, "iterations": st.solve.iterations,
                "vcycles": st.solve.vcycles, "relres": st.solve.relres, "solve_ms": st.solve.ms,
                "oc_trials": st.oc_trials, "ms": st.ms, "rc": rc,
                "learned_applied": st.solve.learned_applied, "learned_fallback": bool(st.solve.learned_fallback)}


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class MMA:
    """Method of Moving Asymptotes on the GPU (wraps ``topo_mma``; reference
    ``MMA::mma_t``, optimization/mma_t.h).  ``MMA(n, m)`` is standalone with its own
    stream; ``MMA.for_problem(p, m)`` optimises ``p``'s spline coefficients on its
    stream.  ``update(df_ptr, [dg_ptr...], g)`` takes device pointers for the
    gradients and host values for the constraints."""

    def __init__(self, n=None, m=1, device=0, lb=None, ub=None, _handle=None):
        self.lib = load()
        self.problem = None
        hp = C.c_void_p()
        if _handle is not None:
            rc = self.lib.topo_mma_create_for(_handle.h, m, C.byref(hp))
            if rc != TOPO_OK:
                raise TopoError(rc, self.lib.topo_last_error(_handle.h).decode())
            self.problem = _handle
        else:
            rc = self.lib.topo_mma_create(int(n), int(m), int(device), C.byref(hp))
            if rc != TOPO_OK:
                raise TopoError(rc, "topo_mma_create failed")
        self.h = hp
        nn, mm = C.c_int(), C.c_int()
        self._ck(self.lib.topo_mma_size(self.h, C.byref(nn), C.byref(mm)))
        self.n, self.m = nn.value, mm.value
        if lb is not None and ub is not None:
            self.init(lb, ub)

    @classmethod
    def for_problem(cls, problem, m=1, lb=None, ub=None):
        return cls(m=m, lb=lb, ub=ub, _handle=problem)

    def _ck(self, rc):
        if rc != TOPO_OK:
            raise TopoError(rc, self.lib.topo_mma_last_error(self.h).decode())

    def init(self, lb, ub):
        if np.ndim(lb) == 0 and np.ndim(ub) == 0:
            self._ck(self.lib.topo_mma_init_uniform(self.h, float(lb), float(ub)))
        else:
            lbv = np.ascontiguousarray(np.broadcast_to(np.asarray(lb, dtype=np.float64), (self.n,)))
            ubv = np.ascontiguousarray(np.broadcast_to(np.asarray(ub, dtype=np.float64), (self.n,)))
            self._ck(self.lib.topo_mma_init(self.h, _dp(lbv), _dp(ubv)))

    def set_constraint_amplifier(self, c, d):
        self._ck(self.lib.topo_mma_set_constraint_amplifier(self.h, c, d))

    def update(self, df_ptr, dg_ptrs, g) -> dict:
        dg = (C.c_void_p * self.m)(*[C.c_void_p(int(q)) for q in dg_ptrs])
        gv = np.ascontiguousarray(np.asarray(g, dtype=np.float64).reshape(self.m))
        st = MmaStats()
        self._ck(self.lib.topo_mma_update(self.h, C.c_void_p(int(df_ptr)), dg, _dp(gv), C.byref(st)))
        return {"subiterations": st.subiterations, "kkt_err": st.kkt_err, "step": st.step,
                "dx_norm": st.dx_norm, "overflow": bool(st.overflow), "converged": bool(st.converged)}

    def checkpoint_save(self, path):
        self._ck(self.lib.topo_mma_checkpoint_save(self.h, os.fsencode(path)))

    def checkpoint_load(self, path):
        self._ck(self.lib.topo_mma_checkpoint_load(self.h, os.fsencode(path)))

    def get_x(self, dst_ptr):
        self._ck(self.lib.topo_mma_get_x(self.h, C.c_void_p(int(dst_ptr))))

    @property
    def x(self) -> np.ndarray:
        out = np.zeros(self.n)
        self._ck(self.lib.topo_mma_read_x(self.h, _dp(out)))
        return out

    @x.setter
    def x(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        assert v.size == self.n
        self._ck(self.lib.topo_mma_write_x(self.h, _dp(v)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.topo_mma_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mma_design_iteration(p, mma, vfrac, dvol_ptr=None, solve=None, filter_radius=2.0, vol_scale=1e3,
                         reference_volume=True):
    """One MMA design iteration of the spline coefficients (the loop body of the
    reference's testOrdinarySplineTopoptMMA, utils/test_utils.cpp:1047-1186):
    coefficients from MMA, density, operators, solve, compliance, sensitivity,
    filter, spline adjoint, then ``mma.update`` with the volume constraint
    ``vol_scale * (vol - vfrac) <= 0``.  ``dvol_ptr`` holds ``vol_scale * dvol/dc``
    (default: the handle's "volcsens" array, filled by ``Problem.volume_csens``).
    Returns compliance, volume and MMA stats."""
    if dvol_ptr is None:
        dvol_ptr = p.device_ptr("volcsens")
    mma.get_x(p.device_ptr("coeff"))
    p.coeff_to_density()
    vol = p.volume(reference_volume)
    p.update_operators()
    s = dict(mode=SOLVE_PCG64, smoother=SMOOTH_GS, pre=2, post=2, rtol=1e-6, max_iter=300)
    s.update(solve or {})
    r = p.solve(**s)
    c = p.compliance()
    p.sensitivity()
    p.filter(filter_radius)
    p.spline_adjoint()
    st = mma.update(p.device_ptr("csens"), [dvol_ptr], [vol_scale * (vol - vfrac)])
    st.update({"compliance": c, "volume": vol, "iterations": r["iterations"], "relres": r["relres"]})
    return st


def design_batch(problems, iterations, threads=None, solve=None, ocs=None, filter_radius=2.0):
    """topo_design_batch: `iterations` design iterations on every problem, from
    `threads` host threads (default: one per problem).  solve: one solve-options
    dict for all, or a list with one per problem; ocs: one OC dict per problem
    (or None).  Returns (per-problem last-iteration stats, batch stats)."""
    lib = load()
    n = len(problems)
    hs = (C.c_void_p * n)(*[p.h for p in problems])
    solves = list(solve) if isinstance(solve, (list, tuple)) else [solve] * n
    opts = (IterOpts * n)(*[Problem.iter_opts(solves[k], (ocs[k] if ocs else None), filter_radius)
                            for k in range(n)])
    last = (IterStats * n)()
    bs = BatchStats()
    rc = lib.topo_design_batch(hs, n, opts, n, iterations, threads or n, last, C.byref(bs))
    if rc not in (TOPO_OK, TOPO_E_NOT_CONVERGED):
        raise TopoError(rc, "topo_design_batch")
    out = [{"compliance": s.compliance, "volume": s.volume, "iterations": s.solve.iterations, "ms": s.ms}
           for s in last]
    return out, {"wall_ms": bs.wall_ms, "sum_ms": bs.sum_ms, "max_ms": bs.max_ms, "failures": bs.failures}
