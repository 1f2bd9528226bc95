"""ctypes binding of libvotca_gb300.so (the C ABI in include/votca_gb300_bse.h).

The library is built in-tree by votca_gb300.build.  There is no fallback: if
the shared library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_lib = None

c_i64 = ctypes.c_int64
c_i32 = ctypes.c_int32
c_dp = ctypes.POINTER(ctypes.c_double)
c_vp = ctypes.c_void_p


class bse_options(ctypes.Structure):
    _fields_ = [("homo", c_i64), ("rpamin", c_i64), ("qpmin", c_i64), ("vmin", c_i64), ("cmax", c_i64)]


class bse_uks_options(ctypes.Structure):
    _fields_ = [("homo_alpha", c_i64), ("homo_beta", c_i64), ("rpamin", c_i64), ("qpmin", c_i64),
                ("vmin", c_i64), ("cmax", c_i64)]


class bse_mmn_desc(ctypes.Structure):
    _fields_ = [("auxsize", c_i64), ("mmin", c_i64), ("mmax", c_i64), ("nmin", c_i64), ("nmax", c_i64)]


class bse_davidson_options(ctypes.Structure):
    _fields_ = [("iter_max", c_i64), ("tolerance", ctypes.c_double), ("max_search_space", c_i64),
                ("correction", c_i32), ("update", c_i32), ("matrix_type", c_i32), ("verbose", c_i32),
                ("fp64_polish", c_i32), ("reserved", c_i32), ("size_update", c_i64), ("initial_size", c_i64)]


class bse_davidson_result(ctypes.Structure):
    _fields_ = [("iterations", c_i64), ("info", c_i32), ("polished", c_i32), ("matvec_columns", c_i64),
                ("seconds_matvec", ctypes.c_double), ("seconds_total", ctypes.c_double),
                ("max_residual", ctypes.c_double), ("fp64_columns", c_i64), ("polish_iterations", c_i64),
                ("seconds_polish", ctypes.c_double)]


# name -> (restype, argtypes); every symbol declared in include/votca_gb300_bse.h
SIGNATURES = {
    "bse_op_create": (c_i32, [ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp), c_dp, c_dp, c_i64, c_i64,
                              ctypes.POINTER(bse_options), c_i32, ctypes.POINTER(c_vp)]),
    "bse_op_create_dense_screening": (c_i32, [ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp), c_dp, c_dp,
                                              c_i64, c_i64, ctypes.POINTER(bse_options), c_i32,
                                              ctypes.POINTER(c_vp)]),
    "bse_uks_op_create": (c_i32, [ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp), ctypes.POINTER(bse_mmn_desc),
                                  ctypes.POINTER(c_dp), c_dp, c_dp, c_i64, c_i64, c_dp, c_i64, c_i64,
                                  ctypes.POINTER(bse_uks_options), c_i32, ctypes.POINTER(c_vp)]),
    "bse_uks_op_create_dense_screening": (c_i32, [ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp),
                                                  ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp), c_dp, c_dp,
                                                  c_i64, c_i64, c_dp, c_i64, c_i64, ctypes.POINTER(bse_uks_options),
                                                  c_i32, ctypes.POINTER(c_vp)]),
    "bse_dense_op_create": (c_i32, [c_dp, c_dp, c_i64, c_i64, ctypes.POINTER(c_vp)]),
    "bse_op_destroy": (c_i32, [c_vp]),
    "bse_op_size": (c_i32, [c_vp, ctypes.POINTER(c_i64)]),
    "bse_op_matmul": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_i32, c_dp, c_i64, c_i64, c_dp, c_i64]),
    "bse_op_matmul_device": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_i32, c_vp, c_i64, c_i64, c_vp, c_i64, c_vp]),
    "bse_op_matmul_device_noalloc": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_i32, c_vp, c_i64, c_i64, c_vp, c_i64,
                                             c_vp]),
    "bse_op_diagonal": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_i32, c_dp]),
    "bse_op_diagonal_device": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_i32, c_vp, c_vp]),
    "bse_ham_matmul": (c_i32, [c_vp, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_dp, c_i64, c_i64, c_dp,
                               c_i64]),
    "bse_davidson_solve": (c_i32, [c_vp, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32),
                                   ctypes.POINTER(bse_davidson_options), c_i64, c_dp, c_i64, c_dp, c_dp, c_i64,
                                   ctypes.POINTER(bse_davidson_result)]),
    "bse_davidson_solve_batch": (c_i32, [ctypes.POINTER(c_vp), c_i64, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32),
                                         ctypes.POINTER(bse_davidson_options), c_i64, c_dp,
                                         ctypes.POINTER(c_i32), ctypes.POINTER(c_i64), c_i32]),
    "bse_op_eig_gradient": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_i32, c_dp, c_i64, c_i64, c_dp, c_dp, c_dp, c_dp]),
    "bse_op_eig_gradient_full": (c_i32, [c_vp, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_dp, c_dp, c_i64,
                                         c_i64, c_dp, c_dp, c_dp, c_dp]),
    "bse_op_eig_gradient_device": (c_i32, [c_vp, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_vp, c_vp, c_i64,
                                           c_i64, c_dp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "bse_rpa_epsilon": (c_i32, [ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp), c_dp, c_i64, c_i64, c_i64,
                                c_i64, ctypes.c_double, ctypes.c_double, c_dp]),
    "bse_cholesky_inverse": (c_i32, [c_i64, c_dp, c_i64, c_dp, c_i64]),
    "bse_positive_inverse": (c_i32, [c_i64, c_dp, c_i64, ctypes.c_double, c_dp, c_i64]),
    "bse_mmn_multiply_right": (c_i32, [ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp), c_dp, c_i64]),
    "bse_mmn_fill_3c_mo": (c_i32, [ctypes.POINTER(bse_mmn_desc), ctypes.POINTER(c_dp), c_dp, c_i64, c_dp, c_i64,
                                   c_i64]),
    "bse_aux_pseudo_inv_sqrt": (c_i32, [c_i64, c_dp, c_i64, ctypes.c_double, c_dp, c_i64, ctypes.POINTER(c_i64)]),
    "bse_aux_pseudo_inv_sqrt_gwbse": (c_i32, [c_i64, c_dp, c_i64, c_dp, c_i64, ctypes.c_double, c_dp, c_i64,
                                              ctypes.POINTER(c_i64)]),
    "bse_transition_dipoles": (c_i32, [c_dp, c_i64, c_dp, c_i64, c_i64, c_i64, c_i64, c_i64, c_i64, c_dp, c_dp,
                                       c_i64, c_i64, ctypes.c_double, c_i32, c_dp]),
    "bse_op_profile": (c_i32, [c_vp, c_i32]),
    "bse_op_profile_read": (c_i32, [c_vp, c_dp, ctypes.POINTER(c_i64), c_i32]),
    "bse_probe_fp64_tflops": (c_i32, [c_dp]),
    "bse_small_sym_eig": (c_i32, [c_i64, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), c_dp, c_dp, c_dp,
                                  ctypes.POINTER(c_i64)]),
    "bse_small_gen_eig": (c_i32, [c_i64, c_i64, c_dp, c_dp, c_dp, c_dp, ctypes.POINTER(c_i64)]),
    "bse_autotune_report": (c_i32, [ctypes.c_char_p, c_i64, ctypes.POINTER(c_i64)]),
    "bse_last_error": (ctypes.c_char_p, []),
    "bse_version": (ctypes.c_char_p, []),
}

STATUS = {0: "BSE_OK", 1: "BSE_ERR_ARGUMENT", 2: "BSE_ERR_OUT_OF_MEMORY", 3: "BSE_ERR_CUDA",
          4: "BSE_ERR_TIMEOUT", 5: "BSE_ERR_NUMERICAL", 6: "BSE_ERR_UNSUPPORTED"}


class BSEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise OSError(f"{_build.LIB} is missing; run votca_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(code):
    if code != 0:
        raise BSEError(code, load().bse_last_error().decode())
