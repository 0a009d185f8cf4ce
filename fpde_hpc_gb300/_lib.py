"""ctypes binding of libfpde_gb300.so (declared in include/fpde_gb300.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfpde_gb300.so")

c_int, c_i64, c_dbl, c_vp = C.c_int, C.c_int64, C.c_double, C.c_void_p
P_dbl = C.POINTER(C.c_double)


class FpdeError(RuntimeError):
    def __init__(self, code, where, msg):
        super().__init__(f"{where} failed with status {code}: {msg}")
        self.code = code


class LineTuning(C.Structure):
    _fields_ = [("solve_sp", c_int), ("chunks", c_int), ("far_splits", c_int), ("gemv_splits", c_int),
                ("far_super", c_int), ("ms_per_step", c_dbl)]


class Richards(C.Structure):
    _fields_ = [("k_form", c_int), ("k_sat", c_dbl), ("sZ", c_vp), ("dL", c_vp * 3), ("evaporation", c_vp),
                ("evaporation_rows", c_int), ("salt_c0", c_vp), ("salt_nu", c_dbl), ("salt_sigma", c_dbl),
                ("salt_D", c_dbl)]


class LineDesc(C.Structure):
    _fields_ = [("N", c_i64), ("alpha", c_dbl), ("tau", c_dbl), ("Da", c_dbl),
                ("left_kind", c_int), ("left_value", c_dbl), ("right_kind", c_int),
                ("right_value", c_dbl), ("dLN", c_dbl), ("precision", c_int), ("block", c_int),
                ("max_steps", c_int), ("lag_weights", c_vp), ("theta", c_dbl), ("source", c_vp),
                ("source_rows", c_int), ("tuning", C.POINTER(LineTuning)), ("restrict_eps", c_dbl),
                ("richards", C.POINTER(Richards))]


class SpaceFrac(C.Structure):
    _fields_ = [("space_der", c_int), ("tol", c_dbl), ("max_iter", c_int), ("Tm", c_vp * 3), ("mc", c_vp * 3),
                ("iw", c_vp * 3), ("implicit3d", c_int), ("exact", c_int)]


class Sf3dSystem(C.Structure):
    _fields_ = [("sN", c_int), ("M", c_int), ("K", c_int), ("space_der", c_int), ("mat", c_vp), ("mc", c_vp),
                ("Tm", c_vp * 3), ("iw", c_vp), ("rs", c_vp)]


class Lod3dDesc(C.Structure):
    _fields_ = [("sN", c_int), ("M", c_int), ("K", c_int), ("alpha", c_dbl), ("tau", c_dbl), ("Da", c_dbl),
                ("left_kind", c_int * 3), ("right_kind", c_int * 3), ("dLN", c_dbl * 3), ("precision", c_int),
                ("max_steps", c_int), ("lag_weights", c_vp), ("source", c_vp), ("source_rows", c_int),
                ("bc", c_vp), ("bc_rows", c_int), ("restrict_eps", c_dbl), ("series_terms", c_int),
                ("richards", C.POINTER(Richards)), ("time_steps", c_vp), ("weight_rows", c_vp),
                ("kernel_power", c_dbl), ("space_frac", C.POINTER(SpaceFrac)), ("segments", c_int * 3)]


class ColumnDesc(C.Structure):
    _fields_ = [("N", c_i64), ("alpha", c_dbl), ("tau", c_dbl), ("Da", c_dbl), ("left_kind", c_int),
                ("left_value", c_dbl), ("right_kind", c_int), ("right_value", c_dbl), ("dLN", c_dbl),
                ("A", c_vp), ("B", c_vp), ("Rlap", c_vp), ("u0", c_vp), ("lag_weights", c_vp),
                ("restrict_eps", c_dbl)]


# name -> (restype, argtypes)
_SIGS = {
    "fpde_ctx_create": (c_int, [c_int, C.POINTER(c_vp)]),
    "fpde_ctx_destroy": (c_int, [c_vp]),
    "fpde_ctx_set_stream": (c_int, [c_vp, c_vp]),
    "fpde_ctx_synchronize": (c_int, [c_vp]),
    "fpde_ctx_sm_count": (c_int, [c_vp, C.POINTER(c_int)]),
    "fpde_last_error_string": (C.c_char_p, []),
    "fpde_kernel_launch_count": (c_i64, []),
    "fpde_weights_l1": (c_int, [c_dbl, c_vp, c_int, c_vp, P_dbl]),
    "fpde_weights_l1_lags": (c_int, [c_dbl, c_int, c_vp]),
    "fpde_gamma": (c_int, [c_dbl, P_dbl]),
    "fpde_do_weights": (c_int, [c_int, c_vp, c_vp, c_vp, c_dbl, c_int, c_vp]),
    "fpde_line_autotune": (c_int, [c_vp, C.POINTER(LineDesc), c_vp, c_vp, c_vp, c_vp, C.POINTER(LineTuning)]),
    "fpde_batch_create": (c_int, [c_vp, C.POINTER(ColumnDesc), c_int, c_int, c_int, C.POINTER(c_vp)]),
    "fpde_batch_destroy": (c_int, [c_vp]),
    "fpde_batch_run": (c_int, [c_vp, c_int]),
    "fpde_batch_get_state": (c_int, [c_vp, c_int, c_vp, c_int]),
    "fpde_batch_layout": (c_int, [c_vp, c_int, C.POINTER(c_i64), C.POINTER(c_i64), C.POINTER(c_i64)]),
    "fpde_batch_reset": (c_int, [c_vp, c_vp, c_int]),
    "fpde_batch_solve_host": (c_int, [c_vp, c_vp, c_int, c_vp]),
    "fpde_lod3d_create": (c_int, [c_vp, C.POINTER(Lod3dDesc), c_vp, c_vp, c_vp, c_vp, C.POINTER(c_vp)]),
    "fpde_lod3d_destroy": (c_int, [c_vp]),
    "fpde_lod3d_run": (c_int, [c_vp, c_int]),
    "fpde_lod3d_get_state": (c_int, [c_vp, c_vp, c_int]),
    "fpde_lod3d_reset": (c_int, [c_vp, c_vp, c_int]),
    "fpde_lod3d_solve_host": (c_int, [c_vp, c_vp, c_int, c_vp]),
    "fpde_lod3d_steps_done": (c_int, [c_vp, C.POINTER(c_i64)]),
    "fpde_lod3d_sf_iterations": (c_int, [c_vp, C.POINTER(c_i64)]),
    "fpde_lod3d_autotune": (c_int, [c_vp, C.POINTER(Lod3dDesc), c_vp, c_vp, c_vp, c_vp, c_int, c_int * 3,
                                    C.POINTER(c_dbl)]),
    "fpde_lod3d_get_concentration": (c_int, [c_vp, c_vp, c_int]),
    "fpde_sf_matvec": (c_int, [c_vp, c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_vp, c_vp, c_int]),
    "fpde_sf_solve": (c_int, [c_vp, c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_vp, c_vp, c_dbl, c_int,
                              c_vp, c_int]),
    "fpde_sf_toeplitz_row": (c_int, [c_dbl, c_vp, c_int, c_vp]),
    "fpde_sf3d_matvec": (c_int, [c_vp, C.POINTER(Sf3dSystem), c_vp, c_vp, c_int]),
    "fpde_sf3d_solve": (c_int, [c_vp, C.POINTER(Sf3dSystem), c_vp, c_vp, c_dbl, c_int, c_int, C.POINTER(c_int),
                                c_int]),
    "fpde_do_derivative": (c_int, [c_vp, c_vp, c_i64, c_i64, c_int, c_dbl, c_vp, c_int, c_int, c_int, c_vp, c_i64,
                                   c_int]),
    "fpde_history_create": (c_int, [c_vp, c_i64, c_i64, c_int, C.POINTER(c_vp)]),
    "fpde_history_destroy": (c_int, [c_vp]),
    "fpde_history_reset": (c_int, [c_vp]),
    "fpde_history_length": (c_int, [c_vp, C.POINTER(c_i64)]),
    "fpde_history_append": (c_int, [c_vp, c_vp, c_int]),
    "fpde_l1_sum": (c_int, [c_vp, c_vp, c_vp, c_dbl, c_vp, c_int]),
    "fpde_l1_sum_noalloc": (c_int, [c_vp, c_int, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "fpde_far_contract": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, c_i64, c_int, c_int, c_dbl,
                                  c_vp, c_int]),
    "fpde_far_contract3": (c_int, [c_vp, C.POINTER(c_vp), c_i64, c_i64, C.POINTER(c_vp), c_i64, c_int, c_vp, c_vp,
                                   c_i64, c_vp, c_int]),
    "fpde_sum_snapshots": (c_int, [c_vp, c_vp, c_vp, c_int, c_i64, c_i64, c_vp, c_vp, c_int]),
    "fpde_restricted_lags": (c_int, [c_vp, c_int, c_dbl, C.POINTER(c_int)]),
    "fpde_weights_g": (c_int, [c_vp, c_dbl, c_dbl, c_vp, c_int, c_int, c_vp, c_i64, c_int]),
    "fpde_sum": (c_int, [c_vp, c_int, c_int, c_i64, c_i64, c_vp, c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_dbl,
                         c_dbl, c_dbl, c_dbl, c_int, c_int]),
    "fpde_tridiag_solve": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64,
                                   c_int, c_vp, c_int, c_vp, c_dbl, c_int]),
    "fpde_line_create": (c_int, [c_vp, C.POINTER(LineDesc), c_vp, c_vp, c_vp, c_vp, C.POINTER(c_vp)]),
    "fpde_line_destroy": (c_int, [c_vp]),
    "fpde_line_reset": (c_int, [c_vp, c_vp, c_int]),
    "fpde_line_run": (c_int, [c_vp, c_int]),
    "fpde_line_get_state": (c_int, [c_vp, c_vp, c_int]),
    "fpde_line_state_ptr": (c_int, [c_vp, C.POINTER(c_vp)]),
    "fpde_line_solve_host": (c_int, [c_vp, c_vp, c_int, c_vp]),
    "fpde_line_steps_done": (c_int, [c_vp, C.POINTER(c_i64)]),
    "fpde_line_graph_stats": (c_int, [c_vp, C.POINTER(c_int), C.POINTER(c_i64)]),
    "fpde_step_block": (c_int, [c_vp, C.POINTER(c_int)]),
    "fpde_line_coefs": (c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "fpde_line_set_probe": (c_int, [c_vp, c_int]),
    "fpde_line_probe_stats": (c_int, [c_vp, c_int, P_dbl, P_dbl, P_dbl, C.POINTER(c_int)]),
}

_lib = None


def exported_symbols():
    return list(_SIGS)


def load(path=None):
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} not found: build it with fpde_hpc_gb300.build.build() "
                          "(nvcc, sm_103a); there is no CPU fallback")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, where):
    if rc != 0:
        msg = load().fpde_last_error_string().decode(errors="replace")
        raise FpdeError(rc, where, msg)
