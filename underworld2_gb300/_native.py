"""ctypes binding of libuwg (the C ABI declared in include/uwg.h).

The library is built in-tree (``underworld2_gb300/_build/libuwg.so``) by
``underworld2_gb300.build.build()``.  There is no CPU fallback: if the library
is missing or no GPU is visible every call raises.
"""
import ctypes
import os

from . import build as _build

_lib = None

UWG_OK = 0
ERRORS = {
    -1: "invalid argument", -2: "CUDA error", -3: "call out of order", -4: "empty element",
    -5: "element holds too many particles", -6: "not converged", -7: "non-finite value",
    -8: "particles left the domain",
}


class UwgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libuwg error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


class MeshDesc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("order", ctypes.c_int), ("porder", ctypes.c_int),
                ("res", ctypes.c_int * 3), ("minc", ctypes.c_double * 3), ("maxc", ctypes.c_double * 3)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("mixed", ctypes.c_int), ("rtol", ctypes.c_double), ("inner_rtol", ctypes.c_double),
                ("outer_rtol", ctypes.c_double), ("max_inner", ctypes.c_int), ("max_outer", ctypes.c_int),
                ("mg_levels", ctypes.c_int), ("smooth_steps", ctypes.c_int), ("restart", ctypes.c_int),
                ("zero_guess", ctypes.c_int), ("schur_pc", ctypes.c_int), ("schur_pc_rtol", ctypes.c_double),
                ("relax_inner", ctypes.c_int), ("schur_pc_smooth", ctypes.c_int), ("p_dir", ctypes.c_void_p),
                ("null_space", ctypes.c_int), ("schur_pc_its", ctypes.c_int), ("coarse_agg", ctypes.c_int),
                ("coarse_rtol", ctypes.c_double)]


class FnOp(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("dst", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32),
                ("imm", ctypes.c_double)]


class FnInput(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("count", ctypes.c_int32),
                ("by_particle", ctypes.c_int32), ("pad", ctypes.c_int32)]


class SolveStats(ctypes.Structure):
    _fields_ = [("pressure_its", ctypes.c_int), ("velocity_presolve_its", ctypes.c_int),
                ("velocity_pressuresolve_its", ctypes.c_int), ("velocity_backsolve_its", ctypes.c_int),
                ("velocity_total_its", ctypes.c_int), ("refinement_steps", ctypes.c_int),
                ("setup_time", ctypes.c_double), ("presolve_time", ctypes.c_double),
                ("pressure_time", ctypes.c_double), ("backsolve_time", ctypes.c_double),
                ("total_time", ctypes.c_double), ("residual", ctypes.c_double),
                ("vmin", ctypes.c_double), ("vmax", ctypes.c_double), ("pmin", ctypes.c_double),
                ("pmax", ctypes.c_double), ("fhat_reason", ctypes.c_int), ("outer_reason", ctypes.c_int),
                ("backsolve_reason", ctypes.c_int), ("schur_pc_its", ctypes.c_int),
                ("schur_pc_time", ctypes.c_double), ("schur_op_time", ctypes.c_double),
                ("schur_pc_used", ctypes.c_int), ("coarse_dim", ctypes.c_int), ("coarse_setup_time", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
_CTX = ctypes.c_void_p

SIGNATURES = {
    "uwg_ctx_create": (_I, [ctypes.POINTER(MeshDesc), ctypes.POINTER(_CTX)]),
    "uwg_ctx_destroy": (None, [_CTX]),
    "uwg_last_error": (ctypes.c_char_p, [_CTX]),
    "uwg_set_stream": (_I, [_CTX, _P]),
    "uwg_sync": (_I, [_CTX]),
    "uwg_mesh_sizes": (_I, [_CTX, _P]),
    "uwg_mesh_axis": (_I, [_CTX, _I, _P]),
    "uwg_layout_random": (_I, [_CTX, _I, ctypes.POINTER(_I64), _P, _P, _P, _P]),
    "uwg_locate": (_I, [_CTX, _I64, _P, _P]),
    "uwg_gauss_nearest": (_I, [_CTX, _I, _P, _P, _P, _P, _P]),
    "uwg_update_owners": (_I, [_CTX, _I64, _P, _P, _P, _P, ctypes.POINTER(_I64)]),
    "uwg_update_owners_f32": (_I, [_CTX, _I64, _P, _P, _P, _P, ctypes.POINTER(_I64)]),
    "uwg_pic_map": (_I, [_CTX, _I64, _P, _P, _P, _P]),
    "uwg_dvc_weights": (_I, [_CTX, _I, _P, _P, _P]),
    "uwg_dvc_weights_noalloc": (_I, [_I, _I, _I64, _P, _P, _P, _P]),
    "uwg_set_bcs": (_I, [_CTX, _P, _P]),
    "uwg_assemble": (_I, [_CTX, _I64, _P, _P, _P, _P, _P, _P, _P]),
    "uwg_element_matrices": (_I, [_CTX, _I64, _P, _P, _P, _P]),
    "uwg_add_force": (_I, [_CTX, _P]),
    "uwg_add_source": (_I, [_CTX, _P, _P, _P, _P, _P]),
    "uwg_fn_eval": (_I, [_CTX, _I, _P, _I, _P, _I64, _P, _I, _I, _P, ctypes.POINTER(ctypes.c_int32)]),
    "uwg_solve_opts_default": (None, [ctypes.POINTER(SolveOpts)]),
    "uwg_stokes_solve": (_I, [_CTX, ctypes.POINTER(SolveOpts), _P, _P, ctypes.POINTER(SolveStats)]),
    "uwg_stokes_residuals": (_I, [_CTX, _P, _P, _P]),
    "uwg_apply_K64": (_I, [_CTX, _I, _P, _P]),
    "uwg_apply_K_refine": (_I, [_CTX, _P, _P]),
    "uwg_apply_K32": (_I, [_CTX, _I, _P, _P]),
    "uwg_apply_G": (_I, [_CTX, _P, _P]),
    "uwg_apply_Gt": (_I, [_CTX, _P, _P]),
    "uwg_rk2_advect": (_I, [_CTX, _I64, _D, _P, _P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "uwg_rk2_advect_f32": (_I, [_CTX, _I64, _D, _P, _P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "uwg_interpolate": (_I, [_CTX, _I64, _P, _P, _P]),
    "uwg_max_dt": (_I, [_CTX, _P, ctypes.POINTER(_D)]),
    "uwg_advdiff_step": (_I, [_CTX, _D, _P, _P, _P, _P, _P, _P, _P, _P, _I, _D, _P]),
    "uwg_advdiff_max_dt": (_I, [_CTX, _P, _P, _D, ctypes.POINTER(_D)]),
    "uwg_slcn_phistar": (_I, [_CTX, _D, _P, _P, _P]),
    "uwg_interpolate_field": (_I, [_CTX, ctypes.c_int64, _P, _P, _I, _P, _P]),
    "uwg_pop_plan_escaped": (_I, [_CTX, _I64, _P, _P, _P, ctypes.POINTER(_I64)]),
    "uwg_pop_plan_pcdvc": (_I, [_CTX, _I64, _P, _P, _P, _P, _D, _D, _I, _I, ctypes.POINTER(_I64),
                                ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "uwg_pop_apply": (_I, [_CTX, _P, _P, _P, _P, _P, _P, _P]),
    "uwg_cnn_gemm": (_I, [_CTX, _I, _I, _I, _P, _I64, _I, _P, _I64, _I, _P, _P, _I64, _P, _I, _I]),
    "uwg_cnn_set_path": (_I, [_CTX, _I]),
    "uwg_cnn_check": (_I, [_CTX]),
    "uwg_cnn_im2col": (_I, [_CTX, _I, _I, _I, _I, _P, _P]),
    "uwg_cnn_col2im": (_I, [_CTX, _I, _I, _I, _I, _P, _P]),
    "uwg_cnn_elementwise": (_I, [_CTX, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P]),
    "uwg_cnn_bias_grad": (_I, [_CTX, _I64, _I, _P, _P]),
    "uwg_cnn_mse": (_I, [_CTX, _I64, _I, _I, _P, _P, _P, _P]),
    "uwg_cnn_adam": (_I, [_CTX, _I64, _P, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, _I]),
    "uwg_slcn_solve": (_I, [_CTX, _D, _P, _P, _P, _P, _P, _D, _I, ctypes.POINTER(_I), ctypes.POINTER(_D), _P]),
}


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libuwg.so (building it first when absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libuwg.so is not built (run underworld2_gb300.build.build())")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(ctx, rc):
    if rc != UWG_OK:
        msg = load().uwg_last_error(ctx)
        raise UwgError(rc, msg.decode() if msg else "")
    return rc
