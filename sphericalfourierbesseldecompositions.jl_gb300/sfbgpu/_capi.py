"""ctypes binding of libsfbgpu.so (declarations in include/sfb_gpu.h).

The shared library is built in place by ``build.py``.  Loading it needs no
GPU; every compute entry point fails with SFB_ECUDA when no CUDA device is
present.  There is no CPU fallback: if the library is missing, importing
this module raises.
"""

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "libsfbgpu.so")

SFB_OK, SFB_EINVAL, SFB_ENOMEM, SFB_ENONFINITE, SFB_ERANGE, SFB_ETIMEOUT, SFB_ECUDA, SFB_ENOTSUP = range(8)
SFB_FP64, SFB_MIXED = 0, 1
SFB_F64, SFB_F32 = 0, 1
SFB_RADIAL_POLY, SFB_RADIAL_SPLINE = 0, 1
SFB_WINDOW_ZERO, SFB_WINDOW_SEPARABLE, SFB_WINDOW_DENSE = 0, 1, 2

STATUS_NAMES = {0: "SFB_OK", 1: "SFB_EINVAL", 2: "SFB_ENOMEM", 3: "SFB_ENONFINITE", 4: "SFB_ERANGE",
                5: "SFB_ETIMEOUT", 6: "SFB_ECUDA", 7: "SFB_ENOTSUP"}

_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)


class PlanDesc(C.Structure):
    _fields_ = [("nside", C.c_int64), ("lmax", C.c_int64), ("nmax", C.c_int64), ("lmax_n", _i64p),
                ("rmin", C.c_double), ("rmax", C.c_double),
                ("spl_offset", _i64p), ("spl_x", _dp), ("spl_y", _dp), ("spl_ypp", _dp),
                ("niter", C.c_int32), ("precision", C.c_int32), ("radial_mode", C.c_int32),
                ("radial_pieces", C.c_int32), ("radial_degree", C.c_int32), ("radial_tol", C.c_double)]


class Window(C.Structure):
    _fields_ = [("kind", C.c_int32), ("mask", _dp), ("w_ln", _dp), ("dense", _dp)]


class PlanInfo(C.Structure):
    _fields_ = [("npix", C.c_int64), ("nlmsize", C.c_int64), ("npairs", C.c_int64), ("nbasis", C.c_int64),
                ("radial_pieces", C.c_int32), ("radial_degree", C.c_int32), ("radial_error", C.c_double),
                ("device_bytes", C.c_int64)]


# (name, restype, argtypes) for every entry point of include/sfb_gpu.h
_PROTOS = [
    ("sfb_plan_create", C.c_int, [C.POINTER(PlanDesc), C.POINTER(C.c_void_p)]),
    ("sfb_plan_destroy", None, [C.c_void_p]),
    ("sfb_plan_get_info", C.c_int, [C.c_void_p, C.POINTER(PlanInfo)]),
    ("sfb_set_precision", C.c_int, [C.c_void_p, C.c_int32]),
    ("sfb_cat2amln", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.POINTER(Window),
                               C.c_void_p]),
    ("sfb_cat2amln_vjp", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_void_p]),
    ("sfb_field2anlm_vjp", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_void_p]),
    ("sfb_map2alm_adjoint", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    ("sfb_cat2amln_batched", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                       C.POINTER(Window), C.c_void_p]),
    ("sfb_cat2amln_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_double,
                                      C.POINTER(Window), C.c_void_p, C.c_void_p]),
    ("sfb_field2anlm", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_void_p]),
    ("sfb_field2anlm_typed", C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.c_double, C.c_double,
                                       C.c_void_p]),
    ("sfb_field2anlm_vjp_typed", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_void_p,
                                           C.c_int32]),
    ("sfb_anlm2field", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_void_p]),
    ("sfb_win_rhat_ln_separable", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double,
                                            C.c_void_p]),
    ("sfb_win_rhat_ln_dense", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_void_p]),
    ("sfb_map2alm", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    ("sfb_calc_wmix", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_int32,
                                C.c_void_p]),
    ("sfb_win_lnn", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_void_p, C.c_int64,
                              C.c_void_p]),
    ("sfb_amln2clnn", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                C.c_void_p]),
    ("sfb_winweights2galweights", C.c_int, [C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64,
                                            C.c_void_p]),
    ("sfb_winweights2galweights_noalloc", C.c_int, [C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                                    C.c_int64, C.c_void_p]),
    ("sfb_ang2pix_ring", C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    ("sfb_apply_window", C.c_int, [C.c_int64, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_double,
                                   C.c_void_p, C.c_int64, C.c_void_p, C.c_uint64, C.c_void_p,
                                   C.POINTER(C.c_int64)]),
    ("sfb_apply_window_device", C.c_int, [C.c_int64, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_double,
                                          C.c_void_p, C.c_int64, C.c_void_p, C.c_uint64, C.c_void_p,
                                          C.POINTER(C.c_int64), C.c_void_p]),
    ("sfb_set_profiling", C.c_int, [C.c_void_p, C.c_int32]),
    ("sfb_get_stage_times", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("sfb_launch_count", C.c_int64, []),
    ("sfb_selftest_wait_timeout", C.c_int, []),
    ("sfb_last_error", C.c_int, [C.c_char_p, C.c_size_t]),
]

STAGES = ["deposit", "ring_fft", "leg_analysis", "leg_synthesis", "fold", "project", "other"]

if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} not found: build the CUDA library first (python build.py)")

lib = C.CDLL(LIB_PATH)
for _name, _res, _args in _PROTOS:
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


class SFBError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def last_error():
    buf = C.create_string_buffer(1024)
    lib.sfb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status):
    if status != SFB_OK:
        raise SFBError(status, last_error())
    return status


def ptr(a):
    """Data pointer of a numpy array (None for None)."""
    return None if a is None else C.c_void_p(a.ctypes.data)
