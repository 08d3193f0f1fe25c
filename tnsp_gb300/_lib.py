"""Loads the in-tree C-ABI library ``libtnsp_gb300.so`` (declared in include/tnsp_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is usable, every entry
point raises.  Build it with ``tnsp_gb300.build.build()``.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtnsp_gb300.so")

TNSP_FP64 = 0
TNSP_FP32 = 1
TNSP_DD = 2
TNSP_MIXED = 3
TNSP_OPT_JACOBI_SWEEPS = 1
TNSP_OPT_BLOCKS_PER_SM = 2
PRECISIONS = {"fp64": TNSP_FP64, "fp32": TNSP_FP32, "dd": TNSP_DD, "mixed": TNSP_MIXED}

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_i32_p = ctypes.POINTER(ctypes.c_int32)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)
_c_u64_p = ctypes.POINTER(ctypes.c_uint64)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_void_p = ctypes.c_void_p

# name -> (restype, argtypes), exactly the declarations of include/tnsp_gb300.h
SIGNATURES = {
    "tnsp_ctx_create": (ctypes.c_int, [ctypes.POINTER(_c_void_p), ctypes.c_int, _c_void_p]),
    "tnsp_sweep_batch": (ctypes.c_int, [ctypes.POINTER(_c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "tnsp_chains_write": (ctypes.c_int, [_c_void_p, _c_i32_p]),
    "tnsp_made_create": (ctypes.c_int, [ctypes.POINTER(_c_void_p), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_uint64, ctypes.c_int]),
    "tnsp_made_destroy": (ctypes.c_int, [_c_void_p]),
    "tnsp_made_error": (ctypes.c_char_p, [_c_void_p]),
    "tnsp_made_params": (ctypes.c_int, [_c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    "tnsp_made_train": (ctypes.c_int, [_c_void_p, _c_i32_p, ctypes.c_int, ctypes.c_double, _c_dbl_p]),
    "tnsp_made_gradient": (ctypes.c_int, [_c_void_p, _c_i32_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "tnsp_made_logq": (ctypes.c_int, [_c_void_p, _c_i32_p, ctypes.c_int, _c_dbl_p]),
    "tnsp_made_sample": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_i32_p, _c_dbl_p]),
    "tnsp_holes_keep": (ctypes.c_int, [_c_void_p, ctypes.c_int]),
    "tnsp_holes_count": (ctypes.c_int, [_c_void_p, _c_i64_p]),
    "tnsp_holes_gemv": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_dbl_p, _c_dbl_p]),
    "tnsp_holes_gram": (ctypes.c_int, [_c_void_p, _c_dbl_p]),
    "tnsp_ctx_destroy": (ctypes.c_int, [_c_void_p]),
    "tnsp_last_error": (ctypes.c_char_p, [_c_void_p]),
    "tnsp_lattice_upload": (ctypes.c_int,
                            [_c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_int_p, _c_dbl_p, ctypes.c_int]),
    "tnsp_lattice_charges": (ctypes.c_int, [_c_void_p, _c_int_p, _c_int_p, _c_int_p]),
    "tnsp_lattice_fermion": (ctypes.c_int, [_c_void_p, _c_dbl_p, ctypes.c_int]),
    "tnsp_model_upload": (ctypes.c_int,
                          [_c_void_p, ctypes.c_int, _c_int_p, _c_int_p, _c_int_p, ctypes.c_int, _c_int_p, _c_dbl_p]),
    "tnsp_model_hopping": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_int_p, _c_int_p, _c_int_p, ctypes.c_int, _c_int_p,
                                          ctypes.POINTER(ctypes.c_ubyte)]),
    "tnsp_model_energy_restrict": (ctypes.c_int, [_c_void_p, ctypes.POINTER(ctypes.c_ubyte)]),
    "tnsp_chains_init": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_i32_p, _c_u64_p, ctypes.c_int, ctypes.c_int]),
    "tnsp_set_option": (ctypes.c_int, [_c_void_p, ctypes.c_int, ctypes.c_int]),
    "tnsp_resident_chains": (ctypes.c_int, [_c_void_p, _c_int_p]),
    "tnsp_sweep": (ctypes.c_int, [_c_void_p, ctypes.c_int, ctypes.c_int]),
    "tnsp_observer_reset": (ctypes.c_int, [_c_void_p]),
    "tnsp_observer_read": (ctypes.c_int, [_c_void_p, _c_dbl_p, _c_dbl_p, _c_dbl_p]),
    "tnsp_samples_read": (ctypes.c_int, [_c_void_p, _c_dbl_p, _c_dbl_p, _c_dbl_p]),
    "tnsp_chains_read": (ctypes.c_int, [_c_void_p, _c_i32_p, _c_dbl_p]),
    "tnsp_amplitude": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_i32_p, _c_dbl_p, _c_i32_p]),
    "tnsp_device_status": (ctypes.c_int, [_c_void_p, _c_i32_p]),
    "tnsp_last_timing": (ctypes.c_int, [_c_void_p, _c_dbl_p, _c_i64_p]),
    "tnsp_counters_read": (ctypes.c_int, [_c_void_p, _c_dbl_p, ctypes.c_int]),
    "tnsp_amplitude_noalloc": (ctypes.c_int, [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_int_p, _c_void_p, ctypes.c_int, ctypes.c_int, _c_void_p, _c_void_p,
        _c_void_p, _c_void_p
    ]),
}

_lib = None


def load(path=LIB_PATH):
    """Returns the loaded library (ctypes.CDLL), raising if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"tnsp_gb300 CUDA library not built: {path} is missing "
                           "(run tnsp_gb300.build.build()); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(array, ctype):
    """ctypes pointer to a contiguous numpy array (or NULL for None)."""
    if array is None:
        return ctypes.cast(None, ctypes.POINTER(ctype))
    return array.ctypes.data_as(ctypes.POINTER(ctype))
