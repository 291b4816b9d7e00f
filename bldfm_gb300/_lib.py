"""ctypes binding of libbldfm_gb300.so (declarations: include/bldfm_gb300.h).

The library is built in-tree by ``python -m bldfm_gb300.build``.  There is no
CPU fallback: if the library is missing, every solve raises.
"""

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbldfm_gb300.so")

OK = 0
ERR_ODD_MODES = -1
ERR_PRECISION = -2
ERR_ARG = -3
ERR_SPECTRUM_SHAPE = -4
ERR_BROADCAST = -5
ERR_UNSUPPORTED = -6
ERR_WORKSPACE = -7
ERR_CUDA = -8
ERR_TIMEOUT = -9
ERR_NONFINITE = -10
ERR_PROFILE = -11
ERR_HOST = -12

PREC_SINGLE = 0
PREC_DOUBLE = 1
MODE_FP64 = 0
MODE_FP32 = 1
MODE_FP64R = 2

CLOSURES = {"MOST": 0, "CONSTANT": 1, "MOSTM": 2, "OAAHOC": 3}


class Desc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("nz", ctypes.c_int32),
        ("nlx", ctypes.c_int32),
        ("nly", ctypes.c_int32),
        ("footprint", ctypes.c_int32),
        ("analytic", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("has_halo", ctypes.c_int32),
        ("xmax", ctypes.c_double),
        ("ymax", ctypes.c_double),
        ("halo", ctypes.c_double),
        ("meas_x", ctypes.c_double),
        ("meas_y", ctypes.c_double),
        ("srf_bg_conc", ctypes.c_double),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("nxe", ctypes.c_int32),
        ("nye", ctypes.c_int32),
        ("nlx", ctypes.c_int32),
        ("nly", ctypes.c_int32),
        ("px", ctypes.c_int32),
        ("py", ctypes.c_int32),
        ("nfx", ctypes.c_int32),
        ("nfy", ctypes.c_int32),
        ("out_nx", ctypes.c_int32),
        ("out_ny", ctypes.c_int32),
        ("nsolved", ctypes.c_int64),
        ("workspace_bytes", ctypes.c_int64),
    ]


class Case(ctypes.Structure):
    _fields_ = [
        ("desc", Desc),
        ("srf_flx_dev", ctypes.c_void_p),
        ("z_host", ctypes.c_void_p),
        ("prof_host", ctypes.c_void_p),
        ("levels_host", ctypes.c_void_p),
        ("nlvls", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("conc_dev", ctypes.c_void_p),
        ("flx_dev", ctypes.c_void_p),
    ]


class BatchOpts(ctypes.Structure):
    _fields_ = [
        ("threads", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("xform_lines", ctypes.c_int32),
        ("skip_check", ctypes.c_int32),
    ]


class ProfileParams(ctypes.Structure):
    """bldfm_profile_params: the arguments of one vertical_profiles evaluation."""

    _fields_ = [
        ("n", ctypes.c_int32),
        ("closure", ctypes.c_int32),
        ("meas_height", ctypes.c_double),
        ("um", ctypes.c_double),
        ("vm", ctypes.c_double),
        ("ustar", ctypes.c_double),
        ("z0", ctypes.c_double),
        ("mol", ctypes.c_double),
        ("prsc", ctypes.c_double),
        ("domain_height", ctypes.c_double),
        ("stretch", ctypes.c_double),
        ("tke", ctypes.c_double),
    ]


class SurrogateCase(ctypes.Structure):
    """bldfm_surrogate_case: the met scalars of one surrogate footprint."""

    _fields_ = [
        ("zm", ctypes.c_double),
        ("wind", ctypes.c_double),
        ("s1", ctypes.c_double),
        ("s2", ctypes.c_double),
        ("s3", ctypes.c_double),
        ("variant", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("exact_kz", ctypes.c_double),
    ]


_P = ctypes.c_void_p
_SIGS = {
    "bldfm_status_str": (ctypes.c_char_p, [ctypes.c_int]),
    "bldfm_version": (ctypes.c_char_p, []),
    "bldfm_plan": (ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_int, ctypes.POINTER(PlanInfo)]),
    "bldfm_solve": (
        ctypes.c_int,
        [ctypes.POINTER(Desc), _P, _P, _P, _P, ctypes.c_int32, _P, _P, _P, ctypes.c_size_t, _P],
    ),
    "bldfm_solve_host": (ctypes.c_int, [ctypes.POINTER(Desc), _P, _P, _P, _P, ctypes.c_int32, _P, _P]),
    "bldfm_vertical_profiles": (
        ctypes.c_int,
        [
            ctypes.c_int32,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.c_int32,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.c_double,
            ctypes.POINTER(ctypes.c_int32),
            _P,
            _P,
            _P,
        ],
    ),
    "bldfm_set_stage_timing": (ctypes.c_int, [ctypes.c_int]),
    "bldfm_stage_times": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    "bldfm_memcpy_async": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "bldfm_sweep32_flops": (ctypes.c_int, [ctypes.c_int32, _P, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]),
    "bldfm_fma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double), _P]),
    "bldfm_batch_plan": (
        ctypes.c_int,
        [ctypes.POINTER(Case), ctypes.c_int32, ctypes.POINTER(BatchOpts), ctypes.POINTER(ctypes.c_int64)],
    ),
    "bldfm_solve_batch": (
        ctypes.c_int,
        [ctypes.POINTER(Case), ctypes.c_int32, ctypes.POINTER(BatchOpts), _P, ctypes.c_size_t, _P],
    ),
    "bldfm_tc_gemm_check": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.c_int32]),
    "bldfm_surrogate_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    "bldfm_surrogate_destroy": (ctypes.c_int, [_P]),
    "bldfm_surrogate_nparams": (ctypes.c_int, []),
    "bldfm_surrogate_params": (ctypes.c_int, [_P, _P, _P]),
    "bldfm_surrogate_grads": (ctypes.c_int, [_P, _P, _P]),
    "bldfm_surrogate_train_step": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int32, ctypes.c_float, _P]),
    "bldfm_surrogate_forward": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, _P]),
    "bldfm_surrogate_batch": (ctypes.c_int, [_P]),
    "bldfm_transfer_pool_create": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_P)]),
    "bldfm_transfer_pool_destroy": (ctypes.c_int, [_P]),
    "bldfm_transfer_pool_case": (
        ctypes.c_int,
        [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)],
    ),
    "bldfm_transfer_samples": (
        ctypes.c_int,
        [_P, ctypes.c_uint64, ctypes.c_int32, ctypes.c_float, ctypes.c_float, _P, ctypes.c_float, _P, _P, _P, _P, _P],
    ),
    "bldfm_transfer_eval": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_int32, _P]),
    "bldfm_point_measurement_workspace": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_int32]),
    "bldfm_point_measurement": (
        ctypes.c_int,
        [_P, _P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, _P, _P, ctypes.c_size_t, _P],
    ),
    "bldfm_vertical_profiles_batch": (
        ctypes.c_int,
        [ctypes.c_int32, _P, _P, _P, ctypes.POINTER(ctypes.c_size_t), _P, _P, _P, ctypes.c_size_t, _P],
    ),
    "bldfm_selftest_wait_timeout": (ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_int32),
                                                    ctypes.POINTER(ctypes.c_int64)]),
    "bldfm_surrogate_plan": (ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]),
    "bldfm_surrogate_batch_plan": (
        ctypes.c_int, [ctypes.POINTER(Case), ctypes.POINTER(SurrogateCase), ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]
    ),
    "bldfm_surrogate_solve_batch": (
        ctypes.c_int, [_P, ctypes.POINTER(Case), ctypes.POINTER(SurrogateCase), ctypes.c_int32, _P, ctypes.c_size_t, _P]
    ),
    "bldfm_surrogate_solve": (
        ctypes.c_int,
        [_P, ctypes.POINTER(Desc), ctypes.POINTER(SurrogateCase), _P, _P, _P, ctypes.c_int32, _P, _P, _P,
         ctypes.c_size_t, _P],
    ),
    "bldfm_solve_noalloc": (
        ctypes.c_int,
        [ctypes.POINTER(Desc), _P, _P, _P, _P, ctypes.c_int32, _P, _P, _P, _P],
    ),
}

_lib = None


def exported_symbols():
    """Names of the C-ABI entry points this binding declares."""
    return list(_SIGS)


def load():
    """Load the in-tree CUDA library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "bldfm_gb300: CUDA library %s is not built (run `python -m bldfm_gb300.build`); "
                "there is no CPU fallback" % LIB_PATH
            )
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status, what="bldfm"):
    """Map a C-ABI status to the exception the reference raises for the same input."""
    if status == OK:
        return
    lib = load()
    msg = lib.bldfm_status_str(status).decode()
    if status in (ERR_ODD_MODES, ERR_PRECISION):
        raise ValueError(msg)
    if status == ERR_SPECTRUM_SHAPE:
        raise IndexError("boolean index did not match indexed array: " + msg)
    if status == ERR_BROADCAST:
        raise ValueError("operands could not be broadcast together: " + msg)
    if status in (ERR_ARG, ERR_UNSUPPORTED, ERR_WORKSPACE, ERR_PROFILE):
        raise ValueError("%s: %s" % (what, msg))
    if status == ERR_NONFINITE:
        raise FloatingPointError("%s: %s" % (what, msg))
    if status == ERR_HOST:
        raise MemoryError("%s: %s" % (what, msg))
    raise RuntimeError("%s: %s (status %d)" % (what, msg, status))


def ptr(a):
    """Host pointer of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)
