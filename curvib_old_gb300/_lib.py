"""ctypes view of libcvb.so (include/cvb.h).

There is no fallback: if the CUDA library has not been built, or no GPU is
present when a context is created, the call raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libcvb.so"
_lib = None

CVB_OK, CVB_NOT_CONVERGED, CVB_NAN_DETECTED, CVB_OOM, CVB_BAD_INPUT, CVB_TIMEOUT, CVB_CUDA_ERROR, \
    CVB_NOT_SETUP = range(8)
STATUS_NAMES = {0: "OK", 1: "NOT_CONVERGED", 2: "NAN_DETECTED", 3: "OOM", 4: "BAD_INPUT", 5: "TIMEOUT",
                6: "CUDA_ERROR", 7: "NOT_SETUP"}
FP64, MIXED = 0, 1
JACOBI, ZEBRA = 0, 1

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int


class Options(ctypes.Structure):
    _fields_ = [("device", _I), ("stream", _P)]


class LevelDesc(ctypes.Structure):
    _fields_ = ([(n, _I) for n in ("mx", "my", "mz", "gxs", "gys", "gzs", "gxm", "gym", "gzm")]
                + [("bctype", _I * 6), ("isc", _I), ("jsc", _I), ("ksc", _I)]
                + [(n, _P) for n in ("icsi", "ieta", "izet", "jcsi", "jeta", "jzet", "kcsi", "keta", "kzet",
                                     "iaj", "jaj", "kaj", "aj", "csi", "eta", "zet")])


class SolveOpts(ctypes.Structure):
    _fields_ = [("precision", _I), ("rtol", _D), ("atol", _D), ("max_it", _I), ("restart", _I),
                ("pre_sweeps", _I), ("post_sweeps", _I), ("omega", _D), ("project_rhs", _I),
                ("warm_start", _I), ("coarse_dense_max", _I), ("cgs_refine", _I), ("smoother", _I)]


class SolveStats(ctypes.Structure):
    _fields_ = [("status", _I), ("iterations", _I), ("restarts", _I), ("rel_residual", _D),
                ("abs_residual", _D), ("rhs_norm", _D), ("rhs_projected", _D), ("device_ms", _D)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        d["status_name"] = STATUS_NAMES.get(self.status, str(self.status))
        return d


class ImpRKOpts(ctypes.Structure):
    _fields_ = [("ren", _D), ("dt", _D), ("st", _D), ("cfl", _D), ("ti", _I), ("tistart", _I), ("central", _I),
                ("imp_atol", _D), ("imp_rtol", _D), ("imp_max_it", _I), ("inletprofile", _I),
                ("flux_intp_sum", _D)]


def imp_rk_opts(**kw):
    """cvb_imp_rk_opts with the reference's defaults, overridden by keywords."""
    o = ImpRKOpts()
    lib().cvb_imp_rk_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(k)
        setattr(o, k, v)
    return o


class ImpRKStats(ctypes.Structure):
    _fields_ = [("pseudo_iterations", _I), ("rejected", _I), ("norm_du", _D), ("rel_du", _D), ("norm_f", _D),
                ("rel_f", _D), ("lambda_", _D), ("flux_in_sum", _D)]

    def as_dict(self):
        return {f.rstrip("_"): getattr(self, f) for f, _ in self._fields_}


EXPORTS = {
    "cvb_solve_opts_default": ([_P], _I),
    "cvb_init": ([_P, _P], _I),
    "cvb_destroy": ([_P], None),
    "cvb_last_error": ([_P], ctypes.c_char_p),
    "cvb_setup_hierarchy": ([_P, _I, _P, _P], _I),
    "cvb_set_nvert": ([_P, _P], _I),
    "cvb_get_nvert": ([_P, _I, _P, _P], _I),
    "cvb_level_dims": ([_P, _I, _P, _P, _P], _I),
    "cvb_volume_flux_rev": ([_P, _P, _D, _I, _P, _P], _I),
    "cvb_poisson_rhs": ([_P, _P, _D, _D, _P, _P], _I),
    "cvb_poisson_solve": ([_P, _P, _P, _P, _P], _I),
    "cvb_poisson_solver_mg": ([_P, _P, _D, _I, _D, _D, _P, _P, _P], _I),
    "cvb_update_pressure": ([_P, _P, _P], _I),
    "cvb_projection": ([_P, _P, _D, _D, _P], _I),
    "cvb_contra2cart": ([_P, _P, _P], _I),
    "cvb_ghost_node_velocity": ([_P, _P, _P], _I),
    "cvb_projection_cart": ([_P, _P, _D, _D, _P, _P, _P], _I),
    "cvb_ibm_search": ([_P, _P, _I, _P, _I, _P, _P, _I, _I, _P, _P], _I),
    "cvb_ibm_ray_offsets": ([_I, _P], _I),
    "cvb_divergence": ([_P, _P, _P, _P], _I),
    "cvb_metrics_divergence": ([_P, _P, _P], _I),
    "cvb_convection": ([_P, _P, _P, _I, _P], _I),
    "cvb_petsc_vec_write": ([ctypes.c_char_p, _P, ctypes.c_longlong, _I], _I),
    "cvb_petsc_vec_size": ([ctypes.c_char_p, _P], _I),
    "cvb_petsc_vec_read": ([ctypes.c_char_p, _P, ctypes.c_longlong], _I),
    "cvb_restart_write": ([ctypes.c_char_p, _I, _I, ctypes.c_longlong, _P, _P, _P, _P], _I),
    "cvb_restart_read": ([ctypes.c_char_p, _I, _I, ctypes.c_longlong, _P, _P, _P], _I),
    "cvb_grid_dat_read": ([ctypes.c_char_p, _I, _I, _D, _D, _P, _P, _P, _P, ctypes.c_longlong], _I),
    "cvb_device_rhs": ([_P], _P),
    "cvb_device_phi": ([_P], _P),
    "cvb_solve_resident": ([_P, _P, _P], _I),
    "cvb_stream": ([_P], _P),
    "cvb_apply_operator": ([_P, _I, _P, _P], _I),
    "cvb_apply_operator_f32": ([_P, _I, _P, _P], _I),
    "cvb_get_weights": ([_P, _I, _P], _I),
    "cvb_level_cross": ([_P, _I, _P, _P], _I),
    "cvb_restrict": ([_P, _I, _P, _P], _I),
    "cvb_interpolate": ([_P, _I, _P, _P], _I),
    "cvb_nullspace": ([_P, _I, _P], _I),
    "cvb_kernel_launches": ([], ctypes.c_longlong),
    "cvb_time_kernel": ([_P, _I, _I, _I, _P, _P], _I),
    "cvb_tuning_report": ([_P, ctypes.c_char_p, _I], _I),
    "cvb_poisson_rhs_noalloc": ([_P, _P, _P, _I, _I, _I, _D, _D, _P, _P, _P], _I),
    "cvb_batch_create": ([_P, _P, _P], _I),
    "cvb_batch_destroy": ([_P], None),
    "cvb_batch_last_error": ([_P], ctypes.c_char_p),
    "cvb_batch_submit": ([_P, _P, _P, _D, _D, _I, _I, _I, _P], _I),
    "cvb_batch_step": ([_P, _P], _I),
    "cvb_batch_poll": ([_P, _P, _P], _I),
    "cvb_batch_read_phi": ([_P, _P, _P], _I),
    "cvb_batch_solve": ([_P, _I, _P, _P], _I),
    "cvb_batch_in_flight": ([_P], _I),
    "cvb_batch_set_round_limit": ([_P, ctypes.c_longlong], _I),
    "cvb_batch_set_graphs": ([_P, _I], _I),
    "cvb_setup_times": ([_P, _P], _I),
    "cvb_batch_graph_stats": ([_P, _P, _P, _P], _I),
    "cvb_zebra_half_f32": ([_P, _I, _I, _I, ctypes.c_float, _P, _P], _I),
    "cvb_viscous": ([_P, _P, _D, _P], _I),
    "cvb_form_function1": ([_P, _P, _P, _P, _D, _I, _P], _I),
    "cvb_calc_rhs": ([_P, _P, _P, _P, _P, _P, _D, _D, _I, _I, _I, _P], _I),
    "cvb_inflow_flux": ([_P, _P, _P, _I, _P], _I),
    "cvb_bcs_dat_read": ([ctypes.c_char_p, _I, _P, _P], _I),
    "cvb_set_cell_centres": ([_P, _P], _I),
    "cvb_set_plate_velocity": ([_P, _D], _I),
    "cvb_set_inlet_nodes": ([_P, _P, _D, _D, _D], _I),
    "cvb_set_inlet_flux": ([_P, _D, _I], _I),
    "cvb_inlet_flux_in": ([_P], _D),
    "cvb_set_inlet_table": ([_P, _P], _I),
    "cvb_form_bcs": ([_P, _P, _P, _P, _P, _D, _D], _I),
    "cvb_imp_rk_opts_default": ([_P], None),
    "cvb_imp_rk": ([_P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "cvb_device_bytes": ([_P, _P], _I),
    "cvb_set_device_limit": ([_P, ctypes.c_ulonglong], _I),
    "cvb_solve_opts_from_file": ([ctypes.c_char_p, _P, ctypes.c_char_p, _I], _I),
    "cvb_solve_opts_from_args": ([_I, _P, _P, ctypes.c_char_p, _I], _I),
    "cvb_geometry_bytes": ([_P, _P, _P], _I),
    "cvb_setup_like": ([_P, _P, _P], _I),
    "cvb_setup_geometry": ([_P, _I, _P], _I),
    "cvb_set_rhs": ([_P, _P], _I),
    "cvb_set_phi": ([_P, _P], _I),
    "cvb_get_phi": ([_P, _P], _I),
}
KERNELS = {"line_sweep_f32": 0, "line_sweep_f64": 1, "residual_f32": 2, "residual_f64": 3, "zebra_f32": 4,
           "zebra_f64": 5, "vcycle_f32": 6, "vcycle_f64": 7, "contra2cart": 8, "ghost_nodes": 9,
           "convection": 10, "viscous": 11, "momentum_rhs": 12}


def lib_path() -> Path:
    return _LIB_PATH


def lib():
    """The loaded libcvb.so with argument types set; raises if it was not built."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise ImportError(f"{_LIB_PATH} is missing: run curvib_old_gb300.build.build() (nvcc, sm_103a)")
        L = ctypes.CDLL(str(_LIB_PATH))
        for name, (args, res) in EXPORTS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class CvbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def opts_from_control(path, args=(), **kw) -> SolveOpts:
    """Solve options from a control.dat file, then argv-style overrides, then kw."""
    o = SolveOpts()
    lib().cvb_solve_opts_default(ctypes.byref(o))
    bad = ctypes.create_string_buffer(256)
    if path is not None:
        rc = lib().cvb_solve_opts_from_file(str(path).encode(), ctypes.byref(o), bad, len(bad))
        if rc:
            raise CvbError(rc, f"control file: {bad.value.decode()}")
    if args:
        arr = (ctypes.c_char_p * len(args))(*[a.encode() for a in args])
        rc = lib().cvb_solve_opts_from_args(len(args), arr, ctypes.byref(o), bad, len(bad))
        if rc:
            raise CvbError(rc, f"option: {bad.value.decode()}")
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def default_opts(**kw) -> SolveOpts:
    o = SolveOpts()
    lib().cvb_solve_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o
