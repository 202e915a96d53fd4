"""ctypes binding of libanneal_gb300.so (the C ABI in include/anneal_gb300.h).

The library is the only compute path: importing this module fails loudly when the
shared object is missing, and every call checks the returned status.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# ANL_DEBUG_LIB=1 loads the bounds-checked debug build (python -m anneal_gb300.build --debug)
DEBUG_LIB = os.environ.get("ANL_DEBUG_LIB", "0") not in ("", "0")
LIB_PATH = os.path.join(HERE, "_lib_debug" if DEBUG_LIB else "_lib", "libanneal_gb300.so")

ANL_OK = 0
ANL_ERR_MAXITER = 1
ANL_ERR_NONFINITE = 2
ANL_ERR_BREAKDOWN = 3
ANL_ERR_BADARG = 4
ANL_ERR_CUDA = 5
ANL_ERR_SINGULAR = 6
ANL_ERR_NOMEM = 7
ANL_ERR_STATE = 8
ANL_ERR_STAGNATION = 9
ANL_FLAG_FP64 = 1


def ANL_FLAG_RHS(n):
    """Right-hand-side slots of an FP32 context (1..255)."""
    return int(n) << 8


STATUS_NAMES = {0: "OK", 1: "MAXITER", 2: "NONFINITE", 3: "BREAKDOWN", 4: "BADARG", 5: "CUDA",
                6: "SINGULAR", 7: "NOMEM", 8: "STATE", 9: "STAGNATION"}

# Every symbol include/anneal_gb300.h declares; tests check the library exports them all.
EXPORTS = [
    "anl_version", "anl_last_error", "anl_ctx_create", "anl_ctx_destroy", "anl_set_domain",
    "anl_free_mask", "anl_apply_K", "anl_solve", "anl_dot", "anl_element_energy",
    "anl_sensitivity", "anl_stiffness_scale", "anl_filter_init", "anl_filter_fwd",
    "anl_filter_bwd", "anl_physical", "anl_oc_update", "anl_design_stats", "anl_profile_apply",
    "anl_launch_count", "anl_mg_info", "anl_dot_static",
    "anl_mc_create", "anl_mc_destroy", "anl_mc_extract", "anl_mc_smooth", "anl_mc_components", "anl_mc_copy",
    "anl_mc_table", "anl_nn_conv3d", "anl_nn_conv3d_bwd_data", "anl_nn_conv3d_bwd_weight", "anl_nn_gelu_bwd",
    "anl_nn_pool2", "anl_nn_up2", "anl_nn_mse", "anl_nn_adam", "anl_element_stress",
    "anl_vox_create", "anl_vox_destroy", "anl_voxel_fill", "anl_output_field", "anl_choose_level",
    "anl_label_above", "anl_edt", "anl_profile_pass", "anl_solve_status", "anl_debug_oob",
]


class NativeError(RuntimeError):
    """A non-zero status from the CUDA library."""

    def __init__(self, status, func, msg):
        super().__init__(f"{func} failed with {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None

P = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double
I64 = ctypes.c_int64

_SIGS = {
    "anl_version": (I, []),
    "anl_last_error": (ctypes.c_char_p, []),
    "anl_ctx_create": (I, [ctypes.POINTER(P), I, I, I, D, D, I]),
    "anl_ctx_destroy": (None, [P]),
    "anl_set_domain": (I, [P, P, P, ctypes.POINTER(I64), P]),
    "anl_free_mask": (I, [P, P, P]),
    "anl_apply_K": (I, [P, P, P, P, P]),
    "anl_solve": (I, [P, P, P, P, I, D, I, I, ctypes.POINTER(I), ctypes.POINTER(D), P]),
    "anl_solve_status": (I, [P, I]),
    "anl_dot": (I, [P, P, P, ctypes.POINTER(D), P]),
    "anl_element_energy": (I, [P, P, P, P]),
    "anl_sensitivity": (I, [P, P, I, ctypes.POINTER(D), P, P, P, D, D, D, P, P, P]),
    "anl_stiffness_scale": (I, [P, P, P, D, D, D, P, P]),
    "anl_filter_init": (I, [P, D, P]),
    "anl_filter_fwd": (I, [P, P, P, P]),
    "anl_filter_bwd": (I, [P, P, P, P]),
    "anl_physical": (I, [P, P, P, D, D, P, P, P]),
    "anl_oc_update": (I, [P, P, P, P, P, P, D, D, D, D, P, ctypes.POINTER(I), ctypes.POINTER(D), P]),
    "anl_design_stats": (I, [P, P, P, P, P, P, ctypes.POINTER(D), P]),
    "anl_profile_apply": (I, [P, P, P, I, ctypes.POINTER(D), P]),
    "anl_profile_pass": (I, [P, I, I, ctypes.POINTER(D), P]),
    "anl_launch_count": (I64, []),
    "anl_debug_oob": (I, [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "anl_mg_info": (I, [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(D)]),
    "anl_dot_static": (I, [P, P, I64, P, P]),
    "anl_mc_create": (I, [ctypes.POINTER(P)]),
    "anl_mc_destroy": (None, [P]),
    "anl_mc_extract": (I, [P, P, I, I, I, I, D, D, ctypes.POINTER(D), ctypes.POINTER(I64), ctypes.POINTER(I64), P]),
    "anl_mc_smooth": (I, [P, I, D, D, P]),
    "anl_mc_components": (I, [P, P, ctypes.POINTER(I), P]),
    "anl_mc_copy": (I, [P, P, P, P]),
    "anl_mc_table": (I, [P, P]),
    "anl_vox_create": (I, [ctypes.POINTER(P)]),
    "anl_vox_destroy": (None, [P]),
    "anl_voxel_fill": (I, [P, P, I64, I, I, I, D, ctypes.POINTER(D), I, P, ctypes.POINTER(I64), P]),
    "anl_output_field": (I, [P, P, P, P, P, P, I64, P, P]),
    "anl_choose_level": (I, [P, I64, D, D, D, I, P, P, ctypes.POINTER(D), P]),
    "anl_label_above": (I, [P, I, I, I, D, P, P]),
    "anl_edt": (I, [P, I, I, I, P, P, ctypes.c_size_t, P]),
    "anl_nn_conv3d": (I, [P, P, P, P, P, I, I, I, I, I, I, I, I, P]),
    "anl_nn_conv3d_bwd_data": (I, [P, P, P, P, I, I, I, I, I, I, I, P]),
    "anl_nn_conv3d_bwd_weight": (I, [P, P, P, I64, P, P, I, I, I, I, I, I, I, P]),
    "anl_nn_gelu_bwd": (I, [P, P, P, I64, P]),
    "anl_nn_pool2": (I, [P, P, I, I, I, I, I, I, P]),
    "anl_nn_up2": (I, [P, P, I, I, I, I, I, P]),
    "anl_nn_mse": (I, [P, P, P, P, I, I64, P, P, P, P]),
    "anl_nn_adam": (I, [P, P, P, P, I64, D, D, D, D, I, P]),
    "anl_element_stress": (I, [P, P, P, D, P, P, P]),
}


def lib_path():
    return LIB_PATH


def load():
    """Load the library (once). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build the CUDA library first "
                          f"(python -m anneal_gb300.build{' --debug' if DEBUG_LIB else ''})")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    return load().anl_last_error().decode(errors="replace")


def check(status, func):
    if status != ANL_OK:
        raise NativeError(status, func, last_error())
    return status


def call(name, *args):
    return check(getattr(load(), name)(*args), name)
