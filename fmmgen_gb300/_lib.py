"""ctypes binding of libfmmgen_gb300.so (include/fmmgen_gb300.h).

Loading never falls back: if the shared library is missing, or a call is made
without a CUDA device, the error propagates to the caller.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfmmgen_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "fmmgen_gb300.h")

OK, ERR_ARG, ERR_CUDA, ERR_DEPTH, ERR_RANGE, ERR_STATE = range(6)
PREC_FP64, PREC_MIXED, PREC_MIXED_SIMT = 0, 1, 2


class FMMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fmmgen_gb300 error {code}: {msg}")
        self.code = code


_lib = None

_vp, _dp, _lp = C.c_void_p, C.c_void_p, C.c_void_p
_SIGS = {
    "fmmgen_last_error": (C.c_char_p, []),
    "fmmgen_version": (C.c_char_p, []),
    "fmmgen_max_order": (C.c_int, []),
    "fmmgen_launch_count": (C.c_longlong, []),
    "fmmgen_nterms": (C.c_long, [C.c_int]),
    "fmmgen_msize": (C.c_long, [C.c_int, C.c_int]),
    "fmmgen_lsize": (C.c_long, [C.c_int, C.c_int]),
    "fmmgen_minorder": (C.c_int, [C.c_int, C.c_int]),
    "fmmgen_sourcesize": (C.c_int, [C.c_int]),
    "fmmgen_outputsize": (C.c_int, [C.c_int, C.c_int]),
    "fmmgen_gpu_P2M": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_M2M": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_M2L": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_L2L": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_L2P": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_P2P": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_M2P": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_P2M_f32": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_M2M_f32": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_M2L_f32": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_L2L_f32": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_L2P_f32": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_P2P_f32": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, _vp]),
    "fmmgen_gpu_M2P_f32": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    "fmmgen_configure": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int]),
    "P2M": (None, [C.c_double, C.c_double, C.c_double, C.c_double, _dp, C.c_int]),
    "M2M": (None, [C.c_double, C.c_double, C.c_double, _dp, _dp, C.c_int]),
    "M2L": (None, [C.c_double, C.c_double, C.c_double, _dp, _dp, C.c_int]),
    "L2L": (None, [C.c_double, C.c_double, C.c_double, _dp, _dp, C.c_int]),
    "L2P": (None, [C.c_double, C.c_double, C.c_double, _dp, _dp, C.c_int]),
    "M2P": (None, [C.c_double, C.c_double, C.c_double, _dp, _dp, C.c_int]),
    "P2P": (None, [C.c_double, C.c_double, C.c_double, _dp, _dp]),
    "P2Mf": (None, [C.c_float, C.c_float, C.c_float, C.c_float, _dp, C.c_int]),
    "M2Mf": (None, [C.c_float, C.c_float, C.c_float, _dp, _dp, C.c_int]),
    "M2Lf": (None, [C.c_float, C.c_float, C.c_float, _dp, _dp, C.c_int]),
    "L2Lf": (None, [C.c_float, C.c_float, C.c_float, _dp, _dp, C.c_int]),
    "L2Pf": (None, [C.c_float, C.c_float, C.c_float, _dp, _dp, C.c_int]),
    "M2Pf": (None, [C.c_float, C.c_float, C.c_float, _dp, _dp, C.c_int]),
    "P2Pf": (None, [C.c_float, C.c_float, C.c_float, _dp, _dp]),
    "fmmgen_tree_build": (C.c_int, [_dp, C.c_long, C.c_long, C.c_int, C.c_double, C.c_int, _vp,
                                    C.POINTER(C.c_void_p)]),
    "fmmgen_forest_build": (C.c_int, [_dp, _lp, C.c_int, C.c_long, C.c_int, C.c_double, C.c_int, _vp,
                                      C.POINTER(C.c_void_p)]),
    "fmmgen_tree_compute_field_fmm": (C.c_int, [_vp, _dp, _dp, C.c_int, C.c_int, C.c_int, _vp]),
    "fmmgen_tree_build_compute": (C.c_int, [_dp, _lp, C.c_int, C.c_long, C.c_long, C.c_int, C.c_double, C.c_int, _dp,
                                            _dp, C.c_int, C.c_int, C.c_int, _vp, C.POINTER(C.c_void_p)]),
    "fmmgen_gpu_direct": (C.c_int, [_dp, _dp, C.c_long, _lp, C.c_long, C.c_int, C.c_int, C.c_int, _dp, _vp]),
    "fmmgen_tree_compute_field_bh": (C.c_int, [_vp, _dp, _dp, C.c_int, C.c_int, _vp]),
    "fmmgen_tree_free": (C.c_int, [_vp]),
    "fmmgen_root_box_noalloc": (C.c_int, [_dp, C.c_long, _dp, _vp]),
    "fmmgen_tree_info": (C.c_int, [_vp, _lp]),
    "fmmgen_tree_counts": (C.c_int, [_vp, _lp]),
    "fmmgen_tree_root": (C.c_int, [_vp, _dp]),
    "fmmgen_tree_nsys": (C.c_int, [_vp]),
    "fmmgen_tree_set_graph": (C.c_int, [_vp, C.c_int]),
    "fmmgen_tree_export_systems": (C.c_int, [_vp, _dp, _vp]),
    "fmmgen_tree_export_cells": (C.c_int, [_vp, _lp, _lp, _dp, _lp, _lp]),
    "fmmgen_tree_export_lists": (C.c_int, [_vp, _lp, _lp]),
    "fmmgen_tree_export_expansions": (C.c_int, [_vp, _dp, _dp]),
    "fmmgen_tree_times": (C.c_int, [_vp, _vp, _vp]),
    "fmmgen_tree_kernel_ms": (C.c_int, [_vp, _vp]),
    "fmmgen_tree_m2l_work": (C.c_int, [_vp, _dp]),
    "fmmgen_tree_set_tune": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "fmmgen_tree_get_tune": (C.c_int, [_vp, _vp]),
    "fmmgen_tree_autotune": (C.c_int, [_vp, _dp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp]),
    "fmmgen_order_model_nparam": (C.c_int, []),
    "fmmgen_order_nfeatures": (C.c_int, []),
    "fmmgen_order_nclasses": (C.c_int, []),
    "fmmgen_tree_order_features": (C.c_int, [_vp, C.c_double, _vp, _vp]),
    "fmmgen_tree_order_labels": (C.c_int, [_vp, C.c_double, _vp, _vp, _vp]),
    "fmmgen_tree_set_m2l_orders": (C.c_int, [_vp, _vp, _vp]),
    "fmmgen_tree_set_order_model": (C.c_int, [_vp, _vp, C.c_float, C.c_double]),
    "fmmgen_tree_export_m2l_orders": (C.c_int, [_vp, _vp]),
    "fmmgen_mlp_predict": (C.c_int, [_vp, _vp, C.c_long, C.c_float, C.c_int, _vp, _vp]),
    "fmmgen_mlp_train_work": (C.c_long, [C.c_int]),
    "fmmgen_mlp_train_step": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp, _vp, _vp, _vp]),
    "fmmgen_mlp_adam": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_float, _vp]),
}


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m fmmgen_gb300.build` "
                               "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != OK:
        raise FMMError(rc, lib().fmmgen_last_error().decode())
    return rc


def header_functions():
    """Names of the functions include/fmmgen_gb300.h declares."""
    import re

    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z_0-9 ]*?[\s\*]+([A-Za-z_][A-Za-z_0-9]*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "defined")))
