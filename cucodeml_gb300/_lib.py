"""ctypes binding of libgbcodeml.so (the C ABI in include/gbcodeml.h).

There is no fallback: if the library is missing or fails to load, every entry
point raises.  `build()` compiles it in-tree with nvcc when sources are newer.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

GB_OK = 0
GB_PREC_FP64 = 0
GB_PREC_FAST = 1
# gb_tune knobs (include/gbcodeml.h)
TUNE = {"mma": 1, "persist": 2, "gchunk": 3, "order": 4, "grid": 5, "checkpoint": 6}
ERRORS = {-1: "GB_ERR_ARG", -2: "GB_ERR_CUDA", -3: "GB_ERR_OOM", -4: "GB_ERR_PARAM",
          -5: "GB_ERR_TIMEOUT", -6: "GB_ERR_STATE", -7: "GB_ERR_NODEVICE"}


class Problem(C.Structure):
    _fields_ = [("ns", C.c_int), ("nnode", C.c_int), ("root", C.c_int), ("father", _ip),
                ("label", _ip), ("npatt", C.c_int), ("z", C.POINTER(C.c_ubyte)), ("fpatt", _dp),
                ("pi", _dp), ("node_scale", C.c_char_p), ("precision", C.c_int), ("device", C.c_int)]


class Params(C.Structure):
    _fields_ = [("blength", _dp), ("kappa", C.c_double), ("omega0", C.c_double),
                ("omega2", C.c_double), ("p0", C.c_double), ("p1", C.c_double)]


class Grad(C.Structure):
    _fields_ = [("d_blength", _dp), ("d_kappa", C.c_double), ("d_omega0", C.c_double),
                ("d_omega2", C.c_double), ("d_p0", C.c_double), ("d_p1", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("ms_host", C.c_double), ("ms_device", C.c_double), ("kernels", C.c_int),
                ("nscale", C.c_int), ("h2d_bytes", C.c_double), ("d2h_bytes", C.c_double)]


KCLASS = ["pmat", "prune", "mix", "bwd", "gradP", "gradH", "other"]


class GBError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None

# name -> (restype, argtypes); every symbol include/gbcodeml.h declares
SIGNATURES = {
    "gb_version": (C.c_char_p, []),
    "gb_last_error": (C.c_char_p, []),
    "gb_create": (C.c_int, [C.POINTER(Problem), C.POINTER(C.c_void_p)]),
    "gb_fault_inject": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "gb_create_unclean": (C.c_int, [C.POINTER(Problem), C.POINTER(C.c_ubyte), C.POINTER(C.c_ubyte),
                                    C.POINTER(C.c_void_p)]),
    "gb_destroy": (C.c_int, [C.c_void_p]),
    "gb_nscale": (C.c_int, [C.c_void_p]),
    "gb_eval_uvr": (C.c_int, [C.c_void_p, _dp * 3, _dp * 3, _dp * 3, _dp, _dp, _dp, _dp, _dp, _dp,
                              C.POINTER(Stats)]),
    "gb_beta_classes": (C.c_int, [C.c_double, C.c_double, C.c_int, _dp, _dp]),
    "gb_eval_clade": (C.c_int, [C.c_void_p, _dp, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp,
                                C.POINTER(Stats)]),
    "gb_se_opg_clade": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int, _dp, C.c_int, C.c_double, _dp, _dp,
                                  _dp]),
    "gb_neb_clade": (C.c_int, [C.c_void_p, _dp, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp]),
    "gb_dfun_clade_x": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_int, _dp, C.c_int, _dp, _dp]),
    "gb_eval_clade_uvr": (C.c_int, [C.c_void_p, _dp * 4, _dp * 4, _dp * 4, _dp, _dp, _dp, _dp, _dp, _dp,
                                    C.POINTER(Stats)]),
    "gb_eval": (C.c_int, [C.c_void_p, C.POINTER(Params), _dp, C.POINTER(Grad), _dp, _dp,
                          C.POINTER(Stats)]),
    "gb_eval_b": (C.c_int, [C.c_void_p, C.POINTER(Params), C.c_double, _dp, C.POINTER(Grad), _dp, _dp, _dp,
                            C.POINTER(Stats)]),
    "gb_beb": (C.c_int, [C.c_void_p, C.POINTER(Params), _dp, _dp, _dp, _dp, _dp, C.POINTER(Stats)]),
    "gb_beb_clade": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, C.POINTER(Stats)]),
    "gb_beb_clade_bl": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_double, _dp, _dp, _dp, _dp, _dp,
                                  C.POINTER(Stats)]),
    "gb_beb_tables": (C.c_int, [C.c_void_p, _dp, C.c_double, _dp, _dp, _dp, _dp, C.POINTER(Stats)]),
    "gb_beb_qf": (C.c_int, [C.c_void_p, _dp, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                            C.POINTER(Stats)]),
    "gb_neb": (C.c_int, [C.c_void_p, C.POINTER(Params), _dp, _dp]),
    "gb_ng86": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_ubyte), _dp, _dp, _dp, _dp]),
    "gb_se_opg": (C.c_int, [C.c_void_p, _ip, _dp, C.c_int, C.c_double, _dp, _dp, _dp, C.POINTER(Stats)]),
    "gb_hessian_x": (C.c_int, [C.c_void_p, _ip, C.c_int, _dp, C.c_int, C.c_double, _dp, _dp]),
    "gb_dfun_x": (C.c_int, [C.c_void_p, _ip, C.c_int, _dp, C.c_int, _dp, _dp]),
    "gb_patterns": (C.c_int, [C.c_int, C.c_int, _ip, _ip, C.POINTER(C.c_ubyte), _dp, _dp]),
    "gb_replay": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp]),
    "gb_batch_create": (C.c_int, [C.c_int, C.POINTER(Problem), C.POINTER(C.c_void_p)]),
    "gb_batch_size": (C.c_int, [C.c_void_p]),
    "gb_batch_eval": (C.c_int, [C.c_void_p, C.POINTER(Params), _dp, C.POINTER(Grad), C.POINTER(Stats)]),
    "gb_batch_submit": (C.c_int, [C.c_void_p, C.POINTER(Params), C.c_int, C.c_void_p]),
    "gb_batch_collect": (C.c_int, [C.c_void_p, _dp, C.POINTER(Grad), C.POINTER(Stats)]),
    "gb_batch_submit_b": (C.c_int, [C.c_void_p, C.POINTER(Params), _dp, C.c_int, C.c_void_p]),
    "gb_batch_omega1_grad": (C.c_int, [C.c_void_p, _dp]),
    "gb_batch_replay": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp]),
    "gb_batch_destroy": (C.c_int, [C.c_void_p]),
    "gb_profile": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _ip]),
    "gb_task_trace": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_ulonglong), C.c_int]),
    "gb_tune": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "gb_batch_tune": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "gb_batch_task_trace": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_ulonglong), C.c_int]),
    "gb_lnL_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, _ip, _ip, C.c_char_p, C.c_int, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p]),
    "gb_model_setup": (C.c_int, [_dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                 _dp, _dp, _dp, _dp, _dp]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_needed: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed:
        _build.build()
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libgbcodeml.so not found at {path}; run cucodeml_gb300.build")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != GB_OK:
        raise GBError(rc, load().gb_last_error().decode())
