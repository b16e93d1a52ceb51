"""ctypes binding of libaerort.so (the C ABI in include/aerort.h).

The library is built in-tree by aeroapps_gb300.build.build().  There is no CPU
fallback: if the library is missing or fails to load, every entry point raises.
"""
import ctypes
import os

from . import build as _build

_lib = None

c_int = ctypes.c_int
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
P_f = ctypes.POINTER(ctypes.c_float)
P_d = ctypes.POINTER(ctypes.c_double)
P_i = ctypes.POINTER(ctypes.c_int)


class MieTableDesc(ctypes.Structure):
    """aerort_mie_table_desc."""
    _fields_ = [("nrh", c_int), ("nbin", c_int), ("nmom", c_int), ("npol", c_int),
                ("rh", P_f), ("bext", P_f), ("bsca", P_f), ("g", P_f), ("pmom", P_f)]


_SIGNATURES = {
    "aerort_mie_create": (c_int, [c_int, ctypes.POINTER(MieTableDesc), c_int, P_f, ctypes.POINTER(c_void_p)]),
    "aerort_mie_destroy": (c_int, [c_void_p]),
    "aerort_mie_table_interp": (c_int, [c_int, P_d, c_int, P_d, c_int, c_int, c_int, P_d, P_d, P_d, P_d, c_int, P_f,
                                        c_int, P_f, P_f, P_f, P_f, P_f, P_i]),
    "aerort_get_aop_scalar": (c_int, [c_void_p, c_int, c_int, c_int, c_int, P_f, P_i, P_i, P_f, P_f, P_f, P_f, P_f]),
    "aerort_get_aop_scalar_dev": (c_int, [c_void_p, c_int, c_int, c_int, c_int, P_f, P_i, P_i, c_void_p, c_void_p,
                                          c_void_p, c_void_p, c_void_p, c_void_p]),
    "aerort_get_aop_vector": (c_int, [c_void_p, c_int, c_int, c_int, c_int, P_f, P_i, P_i, P_f, P_f, c_int, c_int,
                                      P_f, P_f, P_f, P_f]),
    "aerort_get_aop_vector_dev": (c_int, [c_void_p, c_int, c_int, c_int, c_int, P_f, P_i, P_i, c_void_p, c_void_p,
                                          c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "aerort_vlidort_scalar_lambert": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 13 +
                                      [c_double, c_int, P_d, P_d]),
    "aerort_vlidort_scalar_lambert_ex": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 13 +
                                         [c_double, c_int, P_d, P_d, P_i, P_i]),
    "aerort_vlidort_scalar_lambert_dev": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int] + [c_void_p] * 10 +
                                          [c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "aerort_vlidort_scalar_lambert_batch_dev": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int] + [c_void_p] * 14 +
                                                [c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "aerort_vlidort_scalar_lambert_batch_dev_noalloc": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int] +
                                                        [c_void_p] * 14 + [c_double] + [c_void_p] * 5),
    "aerort_vlidort_scalar_lambert_batch": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, P_i] + [P_d] * 10 +
                                            [c_double, P_d, P_d, P_i, P_i]),
    "aerort_vlidort_scalar_lambert_mixed_batch_dev": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int] +
                                                      [c_void_p] * 14 + [c_double] + [c_void_p] * 5),
    "aerort_vlidort_scalar_lambert_mixed_batch": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, P_i] + [P_d] * 10 +
                                                  [c_double, P_d, P_d, P_i, P_i]),
    "aerort_vlidort_vector_lambert": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 14 +
                                      [c_double, c_int, P_d, P_d, P_d, P_d]),
    "aerort_vlidort_vector_lambert_ex": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 14 +
                                         [c_double, c_int, P_d, P_d, P_d, P_d, P_i, P_i]),
    "aerort_vlidort_scalar_landmodis": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 14 +
                                        [c_double, c_int, P_d, P_d, P_d]),
    "aerort_vlidort_scalar_landmodis_ex": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 14 +
                                           [c_double, c_int, P_d, P_d, P_d, P_i, P_i]),
    "aerort_vlidort_scalar_landmodis_batch_dev": (c_int, [c_int] * 6 + [c_void_p] * 11 + [P_d] + [c_void_p] * 3 +
                                                  [c_double] + [c_void_p] * 6),
    "aerort_vlidort_vector_lambert_batch_dev": (c_int, [c_int] * 6 + [c_void_p] * 16 + [c_double] + [c_void_p] * 7),
    "aerort_vlidort_scalar_cx": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 15 +
                                 [c_double, c_int, P_d, P_d, P_d]),
    "aerort_vlidort_scalar_cx_ex": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 15 +
                                    [c_double, c_int, P_d, P_d, P_d, P_i, P_i]),
    "aerort_vlidort_scalar_cx_batch_dev": (c_int, [c_int] * 6 + [c_void_p] * 16 + [c_double] + [c_void_p] * 6),
    "aerort_vlidort_scalar_gisscx": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 15 +
                                     [c_double, c_int, P_d, P_d, P_d]),
    "aerort_vlidort_scalar_gisscx_ex": (c_int, [c_int, c_int, c_int, P_d, c_int, c_int, c_int, c_int] + [P_d] * 15 +
                                        [c_double, c_int, P_d, P_d, P_d, P_i, P_i]),
    "aerort_vlidort_scalar_gisscx_batch_dev": (c_int, [c_int] * 6 + [c_void_p] * 16 + [c_double] + [c_void_p] * 6),
    "aerort_get_edge_vars": (c_int, [c_int, c_int, P_f, P_f, ctypes.c_float, P_f, P_f, P_f]),
    "aerort_get_edge_vars_dev": (c_int, [c_int, c_int, c_void_p, c_void_p, ctypes.c_float, c_void_p, c_void_p,
                                         c_void_p, c_void_p]),
    "aerort_vlidort_rot_calc": (c_int, [c_int, c_int, c_int, P_d, P_d, P_d, P_d, c_double, c_int, P_d, P_d]),
    "aerort_vlidort_rot_calc_dev": (c_int, [c_int, c_int, c_int] + [c_void_p] * 7),
    "aerort_set_schedule": (c_int, [c_int, c_int, c_int, c_int]),
    "aerort_workspace_create": (c_int, [ctypes.c_size_t, ctypes.POINTER(c_void_p)]),
    "aerort_workspace_destroy": (c_int, [c_void_p]),
    "aerort_workspace_bytes_per_thread": (ctypes.c_long, [c_int, c_int, c_int]),
    "aerort_vlidort_scalar_lambert_ws_dev": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_int] +
                                             [c_void_p] * 14 + [c_double] + [c_void_p] * 5),
    "aerort_get_schedule": (c_int, [c_int, c_int, P_i, P_i]),
    "aerort_set_kernel": (c_int, [c_int, c_int, c_int]),
    "aerort_refined_count": (c_int, [c_void_p, P_i]),
    "aerort_get_kernel": (c_int, [c_int, c_int]),
    "aerort_set_moment_contraction": (c_int, [c_int]),
    "aerort_get_moment_contraction": (c_int, []),
    "aerort_probe_dfma": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p]),
    "aerort_probe_ffma": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p]),
    "aerort_last_error": (ctypes.c_char_p, []),
    "aerort_launch_count": (ctypes.c_ulonglong, []),
    "aerort_version": (c_int, []),
    "aerort_release": (c_int, []),
    "aerort_miegen_lognormal": (c_int, [c_int, P_d, c_int, P_d, c_int, P_d, P_d, c_double, c_double, c_int, c_double,
                                        c_int, c_int, P_f, P_f, P_f, P_f]),
    "aerort_miegen_lognormal_pol": (c_int, [c_int, P_d, c_int, P_d, c_int, P_d, P_d, c_double, c_double, c_int,
                                            c_double, c_int, c_int, c_int, P_f, P_f, P_f, P_f]),
}


PREC_FP64 = 0
PREC_MIXED = 1
KERNEL_THREAD = 0
KERNEL_TEAM = 1
KERNEL_AUTO = 2
KERNEL_TERMS = 3
CONTRACT_FMA = 0
CONTRACT_TF32X3 = 1


def library_path():
    return _build.LIB


def lib():
    """Load (building if needed) and return the ctypes handle of libaerort.so."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libaerort.so is not built (%s); run aeroapps_gb300.build.build()" % path)
    handle = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return _lib


def last_error():
    return lib().aerort_last_error().decode(errors="replace")


def ptr(a, kind):
    """Pointer to the data of a contiguous numpy array."""
    return a.ctypes.data_as(kind)
