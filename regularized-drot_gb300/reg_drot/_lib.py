"""ctypes binding of libdrot_gb300.so (the C ABI in include/drot_gb300.h).

The library is built in tree by ``regularized-drot_gb300/build.py``.  There is
no fallback: if the shared library is missing or fails to load, every solver
call raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdrot_gb300.so")

# Symbols declared in include/drot_gb300.h, with ctypes signatures.
_c_int, _c_float, _c_double, _c_size = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_size_t
_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_fp = ctypes.POINTER(ctypes.c_float)


class DrotResult(ctypes.Structure):
    _fields_ = [
        ("n_iter", ctypes.c_int),
        ("iters_run", ctypes.c_int),
        ("converged", ctypes.c_int),
        ("status", ctypes.c_int),
        ("objective_valid", ctypes.c_int),
        ("objective", ctypes.c_float),
        ("objective_f64", ctypes.c_double),
        ("residual", ctypes.c_double),
        ("phase_ms", ctypes.c_double * 4),
    ]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["phase_ms"] = list(self.phase_ms)
        return d


_RP = ctypes.POINTER(DrotResult)


class DrotBatchInstance(ctypes.Structure):
    _fields_ = [
        ("n_rows", ctypes.c_int), ("n_cols", ctypes.c_int), ("ld", ctypes.c_int),
        ("pad", ctypes.c_int),
        ("c_offset", ctypes.c_longlong), ("x_offset", ctypes.c_longlong),
        ("p_offset", ctypes.c_longlong), ("q_offset", ctypes.c_longlong),
        ("rho", ctypes.c_float), ("r_weight", ctypes.c_float), ("eps", ctypes.c_float),
        ("pad2", ctypes.c_float),
    ]


class DrotBatchResult(ctypes.Structure):
    _fields_ = [
        ("n_iter", ctypes.c_int), ("iters_run", ctypes.c_int), ("converged", ctypes.c_int),
        ("objective_valid", ctypes.c_int), ("objective", ctypes.c_double),
        ("residual", ctypes.c_double),
    ]


class DrotAdjointInstance(ctypes.Structure):
    _fields_ = [
        ("n_rows", ctypes.c_int), ("n_cols", ctypes.c_int), ("ld", ctypes.c_int),
        ("pad", ctypes.c_int), ("c_offset", ctypes.c_longlong), ("v_offset", ctypes.c_longlong),
        ("phi1_offset", ctypes.c_longlong), ("phi2_offset", ctypes.c_longlong),
        ("step_size", ctypes.c_float), ("lambda_", ctypes.c_float),
    ]


_AIP = ctypes.POINTER(DrotAdjointInstance)


class DrotLaunchChoice(ctypes.Structure):
    _fields_ = [("vectors_per_lane", ctypes.c_int), ("warps_per_cta", ctypes.c_int),
                ("data_path", ctypes.c_int), ("ctas_per_sm", ctypes.c_int)]


class DrotCostInstance(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int), ("n", ctypes.c_int), ("ld", ctypes.c_int), ("pad", ctypes.c_int),
        ("x_offset", ctypes.c_longlong), ("y_offset", ctypes.c_longlong),
        ("c_offset", ctypes.c_longlong),
    ]


_CIP = ctypes.POINTER(DrotCostInstance)
_BIP = ctypes.POINTER(DrotBatchInstance)


class DrotGlBatchInstance(ctypes.Structure):
    _fields_ = [
        ("n_rows", ctypes.c_int), ("n_cols", ctypes.c_int), ("ld", ctypes.c_int),
        ("n_groups", ctypes.c_int),
        ("c_offset", ctypes.c_longlong), ("x_offset", ctypes.c_longlong),
        ("p_offset", ctypes.c_longlong), ("q_offset", ctypes.c_longlong),
        ("rho", ctypes.c_float), ("lambda_", ctypes.c_float), ("eps", ctypes.c_float),
        ("pad", ctypes.c_float),
    ]


class DrotGlAdjointBatchInstance(ctypes.Structure):
    _fields_ = [
        ("n_rows", ctypes.c_int), ("n_cols", ctypes.c_int), ("ld", ctypes.c_int),
        ("n_groups", ctypes.c_int),
        ("x_offset", ctypes.c_longlong), ("c_offset", ctypes.c_longlong),
        ("row_offset", ctypes.c_longlong), ("col_offset", ctypes.c_longlong),
        ("step_size", ctypes.c_float), ("lambda_", ctypes.c_float),
    ]


class DrotBatchTuning(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("fine_cols", "finest_cols", "item_lines",
                                           "finest_item_lines", "level_quarters",
                                           "prefetch_distance", "tail_quarters")]


_BRP = ctypes.POINTER(DrotBatchResult)

SIGNATURES = {
    "drot_set_launch_choice": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_int,
                                        ctypes.POINTER(DrotLaunchChoice)]),
    "drot_clear_launch_choices": (_c_int, []),
    "drot_status_string": (ctypes.c_char_p, [_c_int]),
    "drot_last_status": (_c_int, []),
    "drot_q_get_work_size_update_x": (_c_int, [_c_int, _c_int]),
    "drot_gl_get_work_size_update_x": (_c_int, [_c_int, _c_int]),
    "drot_gl_group_bounds": (_c_int, [_c_int, _c_int, _ip]),
    "drot_init_state": (_c_int, [_c_int, _c_int, _c_float, _c_int, _vp, _vp, _vp, _vp, _vp,
                                 _vp, _vp, _vp, _vp]),
    "drot_qr_workspace_bytes": (_c_size, [_c_int, _c_int]),
    "drot_gl_workspace_bytes": (_c_size, [_c_int, _c_int, _c_int]),
    "drot_qr_solve": (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_float, _c_float, _c_int,
                               _c_float, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_size, _RP, _vp]),
    "drot_gl_solve": (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_int, _c_float, _c_float,
                               _c_int, _c_float, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_size,
                               _RP, _vp]),
    "drot_read_result": (_c_int, [_vp, _RP, _vp]),
    "drot_np_workspace_bytes": (_c_size, [_c_int, _c_int, _c_int, _c_int, _ip]),
    "drot_np_solve": (_c_int, [_c_int, _vp, _c_int, _vp, _vp, _c_int, _c_int, _c_int, _ip, _c_float,
                               _c_float, _c_int, _c_float, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                               _c_size, _RP, _vp]),
    "drot_qr_solve_ex": (_c_int, [_vp, _c_int, _vp, _vp, _c_int, _c_int, _c_float, _c_float,
                                  _c_int, _c_float, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_size,
                                  _RP, _vp]),
    "drot_gl_solve_ex": (_c_int, [_vp, _c_int, _vp, _vp, _c_int, _c_int, _c_int, _c_float,
                                  _c_float, _c_int, _c_float, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                  _c_size, _RP, _vp]),
    "drot_quadratic_drot_ex": (_c_int, [_vp, _c_int, _vp, _vp, _c_int, _c_int, _c_float,
                                        _c_float, _c_int, _c_float, _vp, _vp, _c_size, _RP,
                                        _vp]),
    "drot_group_lasso_drot_ex": (_c_int, [_vp, _c_int, _vp, _vp, _c_int, _c_int, _c_int,
                                          _c_float, _c_float, _c_int, _c_float, _vp, _vp,
                                          _c_size, _RP, _vp]),
    "drot_quadratic_drot_workspace_bytes": (_c_size, [_c_int, _c_int]),
    "drot_quadratic_drot": (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_float, _c_float, _c_int,
                                     _c_float, _vp, _vp, _c_size, _RP, _vp]),
    "drot_group_lasso_drot_workspace_bytes": (_c_size, [_c_int, _c_int, _c_int]),
    "drot_group_lasso_drot": (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_int, _c_float,
                                       _c_float, _c_int, _c_float, _vp, _vp, _c_size, _RP,
                                       _vp]),
    "drot_qr_wrapper": (_fp, [_vp, _vp, _vp, _c_int, _c_int, _c_float, _c_float, _c_int,
                              _c_float, _fp, _fp, _ip, _fp, _c_int, _c_int]),
    "drot_gl_wrapper": (_fp, [_vp, _vp, _vp, _c_int, _c_int, _c_int, _c_float, _c_float,
                              _c_int, _c_float, _fp, _fp, _ip, _fp, _c_int, _c_int]),
    "drot_free_host": (None, [_fp]),
    "drot_quadratic_drot_noalloc": (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_float, _c_float,
                                             _c_int, _c_float, _vp, _RP, _vp]),
    "drot_batch_plan_create": (_c_int, [_c_int, _BIP, _c_int, ctypes.POINTER(_vp)]),
    "drot_batch_plan_create_ex": (_c_int, [_c_int, _BIP, _c_int, _c_int, ctypes.POINTER(_vp)]),
    "drot_batch_state_ex": (_c_int, [_vp, _vp] + [ctypes.POINTER(_vp)] * 5),
    "drot_gl_batch_plan_create": (_c_int, [_c_int, ctypes.POINTER(DrotGlBatchInstance), _c_int,
                                           ctypes.POINTER(_vp)]),
    "drot_qr_batch_launch_points": (_c_int, [_vp, _vp, _vp, _c_int, _c_float, _vp, _vp, _vp, _c_int,
                                             _vp, _c_size, _vp]),
    "drot_batch_set_tuning": (_c_int, [ctypes.POINTER(DrotBatchTuning)]),
    "drot_batch_resume": (_c_int, [_vp, _vp, _c_int, _vp, _vp, _vp, _c_int, _vp, _c_size, _vp]),
    "drot_gl_adjoint_batch_plan_create": (_c_int, [_c_int,
                                                   ctypes.POINTER(DrotGlAdjointBatchInstance),
                                                   ctypes.POINTER(_vp)]),
    "drot_gl_adjoint_batch_plan_destroy": (None, [_vp]),
    "drot_gl_adjoint_batch_workspace_bytes": (_c_size, [_vp]),
    "drot_gl_adjoint_batch_setup": (_c_int, [_vp, ctypes.POINTER(DrotGlAdjointBatchInstance),
                                             _vp, _c_int] + [_vp] * 6 + [_c_size, _vp]),
    "drot_gl_adjoint_batch_step": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_size, _vp]),
    "drot_batch_plan_destroy": (None, [_vp]),
    "drot_batch_plan_workspace_bytes": (_c_size, [_vp]),
    "drot_batch_plan_tiles": (_c_int, [_vp]),
    "drot_batch_set_iteration_log": (_c_int, [_vp, _vp, _vp, _c_int]),
    "drot_batch_upload": (_c_int, [_vp, _vp, _c_size, _vp]),
    "drot_qr_batch_launch": (_c_int, [_vp, _vp, _c_int, _vp, _vp, _vp, _c_int, _vp, _c_size,
                                      _vp]),
    "drot_batch_results": (_c_int, [_vp, _vp, _BRP, _vp]),
    "drot_batch_state": (_c_int, [_vp, _vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "drot_qr_adjoint_workspace_bytes": (_c_size, [_c_int, _AIP]),
    "drot_qr_adjoint_prepare": (_c_int, [_c_int, _AIP, _vp, _c_int, _vp, _vp, _vp, _vp,
                                         _c_size, _vp]),
    "drot_qr_adjoint_solve": (_c_int, [_c_int, _AIP, _vp, _vp, ctypes.c_double, _c_int, _vp,
                                       _c_size, _ip, _vp]),
    "drot_qr_adjoint_grad": (_c_int, [_c_int, _AIP, _vp, _vp, _vp, _vp, _vp, _vp, _c_size, _vp]),
    "drot_qr_adjoint_residuals": (_c_int, [_c_int, _AIP, _vp, _c_size,
                                           ctypes.POINTER(ctypes.c_double), _vp]),
    "drot_gl_adjoint_workspace_bytes": (_c_size, [_c_int, _c_int, _c_int]),
    "drot_gl_adjoint_step": (_c_int, [_vp, _c_int, _c_int, _c_int, _c_int, _c_float, _c_float,
                                      _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_size, _vp]),
    "drot_gl_adjoint_segment": (_c_int, [_vp, _c_int, _vp, _vp, _c_int, _c_int, _c_int, _c_float,
                                         _c_float, _vp, _vp, _vp, _vp, _vp, _vp, _c_int, _vp,
                                         _vp, _c_size, _vp, _vp, _vp, _vp, _vp, _vp, _c_size,
                                         _vp]),
    "drot_sqeuclidean_cost": (_c_int, [_c_int, _CIP, _vp, _vp, _c_int, _c_float, _c_int, _vp,
                                       _vp]),
    "drot_sqeuclidean_cost_grad_workspace_bytes": (_c_size, [_c_int, _CIP, _c_int]),
    "drot_sqeuclidean_cost_grad": (_c_int, [_c_int, _CIP, _vp, _vp, _c_int, _c_float, _vp, _vp,
                                            _vp, _vp, _vp, _c_size, _vp]),
}

_lib = None


class DrotError(RuntimeError):
    """A solver entry point returned a non-zero drot_status."""

    def __init__(self, status, where=""):
        self.status = status
        msg = status_string(status) if _lib is not None else str(status)
        super().__init__(f"{where}: {msg} (drot_status {status})" if where else msg)


def lib():
    """Load libdrot_gb300.so (once) and attach the C signatures."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is not built; run `python regularized-drot_gb300/build.py` "
                "(or __graft_entry__.build()) first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(status):
    return lib().drot_status_string(int(status)).decode()


def check(status, where=""):
    if status != 0:
        raise DrotError(status, where)
