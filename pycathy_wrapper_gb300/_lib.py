"""ctypes binding of libcathy_gb300.so (C ABI in include/cathy_gb300.h).

The library is built in-tree by :mod:`pycathy_wrapper_gb300.build`.  There is
no CPU fallback: loading fails loudly when the library cannot be built or
loaded, and every compute entry point returns CATHY_GB300_ENODEV when no CUDA
device is present.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)
u8p = C.POINTER(C.c_uint8)

OK, ENODEV, EINVAL, EMESH, ENOMEM, EUNSUP = 0, -1, -2, -3, -4, -5
_ERRS = {ENODEV: "no usable CUDA device / CUDA error", EINVAL: "invalid argument",
         EMESH: "mesh construction failed", ENOMEM: "device allocation failed",
         EUNSUP: "unsupported option"}


class CathyError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"{where}: {_ERRS.get(code, code)} ({code})")
        self.code = code


class Dem(C.Structure):
    _fields_ = [("nrow", C.c_int32), ("ncol", C.c_int32),
                ("delta_x", C.c_double), ("delta_y", C.c_double),
                ("west", C.c_double), ("south", C.c_double), ("factor", C.c_double),
                ("dem", f64p), ("zone", i32p), ("nstr", C.c_int32),
                ("zratio", f64p), ("base", C.c_double), ("ivert", C.c_int32)]


class Soil(C.Structure):
    _fields_ = [("nzone", C.c_int32)] + [
        (k, f64p) for k in ("permx", "permy", "permz", "elstor", "poros", "vgn",
                            "vgrmc", "vgpsat")] + [
        ("pmin", C.c_double), ("scf", C.c_double), ("kslope", C.c_int32),
        ("tolksl", C.c_double), ("nveg", C.c_int32), ("feddes", f64p),
        ("root_map", f64p)]


class Parm(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("iopt", "lump", "isolv", "itmxcg", "ituns",
                                          "ituns1", "ituns2", "l2norm", "nlrelx",
                                          "isimgr")] + [
        (k, C.c_double) for k in ("tetaf", "toluns", "tolswi", "ernlmx", "tolcg",
                                   "omega", "deltat", "dtmin", "dtmax", "tmax",
                                   "dtmaga", "dtmagm", "dtreds", "dtredm",
                                   "pondh_min")] + [("precond", C.c_int32),
                                                    ("isfcvg", C.c_int32)]


class BC(C.Structure):
    _fields_ = [("hspatm", C.c_int32), ("ieto", C.c_int32), ("natm", C.c_int32),
                ("atmtim", f64p), ("atminp", f64p),
                ("np", C.c_int32), ("contp", i32p), ("presc", f64p),
                ("nq", C.c_int32), ("contq", i32p), ("q", f64p),
                ("indp", C.c_int32), ("wtposition", C.c_double), ("pinit", f64p),
                ("nsf", C.c_int32), ("sfnum", i32p), ("sfnod", i32p)]


class Member(C.Structure):
    _fields_ = [("dem", Dem), ("soil", Soil), ("parm", Parm), ("bc", BC)]


class Opts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32),
                ("inner_maxit", C.c_int32), ("inner_tol", C.c_double),
                ("verbose", C.c_int32), ("graphs", C.c_int32)]


class IterRec(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("nstep", "iter", "niter", "ikmax")] + [
        (k, C.c_double) for k in ("deltat", "time", "pl2", "pinf", "pnew_ik",
                                   "pold_ik", "fl2", "finf", "lin_err", "lin_res")]


class StepRec(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("nstep", "iter", "nitert", "nback")] + [
        (k, C.c_double) for k in ("deltat", "time", "store1", "store2", "dstore",
                                   "cdstor", "vin", "cvin", "vout", "cvout",
                                   "erras", "errel", "cerras", "caeras", "sfflw",
                                   "vnd", "vnn")]


EXPORTS = {
    "cathy_gb300_version": (C.c_int32, []),
    "cathy_gb300_device_count": (C.c_int32, []),
    "cathy_gb300_mesh": (C.c_int32, [C.POINTER(Dem), C.c_int32, i32p, f64p, f64p, f64p,
                                     i32p, i32p, i32p]),
    "cathy_gb300_create": (C.c_int32, [C.c_int32, C.POINTER(Member), C.POINTER(Opts),
                                       C.POINTER(C.c_void_p)]),
    "cathy_gb300_destroy": (C.c_int32, [C.c_void_p]),
    "cathy_gb300_sizes": (C.c_int32, [C.c_void_p, C.c_int32, i32p]),
    "cathy_gb300_step": (C.c_int32, [C.c_void_p, i32p]),
    "cathy_gb300_run": (C.c_int32, [C.c_void_p, C.c_int32, i32p]),
    "cathy_gb300_get_state": (C.c_int32, [C.c_void_p, C.c_int32, f64p, f64p, f64p, i32p]),
    "cathy_gb300_get_saturation": (C.c_int32, [C.c_void_p, C.c_int32, f64p]),
    "cathy_gb300_get_seepage": (C.c_int32, [C.c_void_p, C.c_int32, i32p, f64p]),
    "cathy_gb300_set_state": (C.c_int32, [C.c_void_p, C.c_int32, f64p, C.c_double,
                                          C.c_double]),
    "cathy_gb300_num_records": (C.c_int32, [C.c_void_p, C.c_int32, i32p, i32p]),
    "cathy_gb300_get_records": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(IterRec),
                                            C.POINTER(StepRec)]),
    "cathy_gb300_get_mesh": (C.c_int32, [C.c_void_p, C.c_int32, f64p, f64p, f64p, i32p,
                                         i32p, i32p]),
    "cathy_gb300_picard_system": (C.c_int32, [C.c_void_p, C.c_int32, f64p, f64p, f64p,
                                              i32p]),
    "cathy_gb300_reset": (C.c_int32, [C.c_void_p]),
    "cathy_gb300_profile": (C.c_int32, [C.c_void_p, C.c_int32, f64p, C.POINTER(C.c_int64),
                                        f64p]),
    "cathy_gb300_autotune": (C.c_int32, [C.c_void_p, C.c_int32, i32p, f64p]),
    "cathy_gb300_set_schedule": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                             C.c_int32]),
    "cathy_gb300_phase_timers": (C.c_int32, [C.c_void_p, C.c_int32, f64p, C.c_int32]),
    "cathy_gb300_time_assembly": (C.c_int32, [C.c_void_p, C.c_int32, f64p, f64p,
                                              C.POINTER(C.c_int64)]),
    "cathy_gb300_stats": (C.c_int32, [C.c_void_p, f64p, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "cathy_gb300_timers": (C.c_int32, [C.c_void_p, f64p, C.c_int32]),
    "cathy_gb300_symslv": (C.c_int32, [i32p, i32p, i32p, i32p, i32p, i32p, f64p, f64p,
                                       i32p, i32p, i32p, f64p, f64p, f64p, f64p, f64p,
                                       f64p, f64p]),
    "cathy_gb300_nsyslv": (C.c_int32, [i32p, i32p, i32p, i32p, i32p, i32p, i32p, i32p,
                                       i32p, i32p, i32p, f64p, f64p, f64p, f64p, f64p,
                                       f64p, f64p, f64p]),
    "cathy_gb300_asspic": (C.c_int32, [i32p, i32p, i32p, i32p, f64p, f64p, f64p, f64p,
                                       f64p, f64p, f64p, f64p, f64p, f64p, f64p, f64p,
                                       f64p, f64p, f64p, f64p, i32p, i32p]),
    "cathy_gb300_lp_create": (C.c_int32, [f32p, C.c_int32, C.POINTER(C.c_void_p)]),
    "cathy_gb300_lp_destroy": (C.c_int32, [C.c_void_p]),
    "cathy_gb300_lp_params": (C.c_int32, [C.c_void_p, f32p, f32p, C.c_double,
                                          C.POINTER(C.c_int64)]),
    "cathy_gb300_lp_eval": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, i32p, i32p, f32p,
                                        u8p, f32p, f32p, f32p, C.c_float, C.c_int32, f32p,
                                        f32p, C.c_int32, f64p, f32p, f32p, f32p]),
    "cathy_gb300_attach_learned": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32]),
    "cathy_gb300_learned_stats": (C.c_int32, [C.c_void_p, f64p, C.c_int32]),
    "cathy_gb300_nsyslv_noalloc": (C.c_int32, [i32p, i32p, C.c_void_p, i32p, i32p,
                                               C.c_void_p, C.c_void_p, f64p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, f64p, f64p,
                                               C.c_void_p]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) and type the exported symbols."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"libcathy_gb300.so not found at {path}")
    L = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(code, where):
    if code != OK:
        raise CathyError(code, where)
