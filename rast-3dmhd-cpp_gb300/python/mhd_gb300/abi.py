"""ctypes binding of the C ABI in include/mhd_gb300.h (libmhd_gb300.so).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly when the built library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent.parent   # rast-3dmhd-cpp_gb300/
LIB_PATH = PKG / "lib" / "libmhd_gb300.so"

MHD_OK = 0
MHD_ERR_INVALID, MHD_ERR_UNSUPPORTED = -1, -2
MHD_ERR_NUMERIC, MHD_ERR_DT_TOO_SMALL = -4, -5
STATUS = {0: "ok", -1: "invalid argument", -2: "unsupported configuration", -3: "CUDA error",
          -4: "non-finite or non-positive state", -5: "DT too small", -6: "out of device memory",
          -7: "device wait timed out"}

SW_LROT, SW_LMAG, SW_LPOT, SW_LREM, SW_LSHR = 0x1, 0x2, 0x4, 0x8, 0x10
PREC_FP64, PREC_FP32 = 0, 1
PATH_FUSED, PATH_PARITY = 0, 1

FIELD_IDS = {n: i for i, n in enumerate(
    ["RU", "RV", "RW", "TT", "RO", "BX", "BY", "BZ",
     "FU", "FV", "FW", "FR", "FT", "WW1", "WW2", "WW3",
     "ZRU", "ZRV", "ZRW", "ZTT", "ZRO", "ZBX", "ZBY", "ZBZ"])}

_DP = C.POINTER(C.c_double)


class MhdParams(C.Structure):
    _fields_ = [("nPx", C.c_int), ("nPy", C.c_int), ("nPz", C.c_int), ("switches", C.c_uint),
                ("ixCon", C.c_int), ("iyCon", C.c_int), ("izCon", C.c_int), ("iTCon", C.c_int), ("iBCon", C.c_int),
                ("precision", C.c_int), ("path", C.c_int), ("reserved_i", C.c_int * 5)] + \
               [(n, C.c_double) for n in ("RE", "PR", "THETA", "GRAV", "RY", "ANG", "RM", "BETA", "TP", "GAMMA",
                                           "SFF", "TB")] + \
               [(n, C.c_double) for n in ("TU", "DZTU", "DZTB")] + [("reserved_d", C.c_double * 1)] + \
               [(n, _DP) for n in ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ",
                                   "RKAPA", "DKAPA")]


class MhdConstants(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("C13", "C23", "C43", "GAM1", "GAM2", "GAM3", "ZETA1", "ZETA2",
                                           "hx", "h2x", "hy", "h2y", "hz", "h2z",
                                           "REPR", "ORE", "ORM", "OBETA", "OMX", "OMZ", "CV", "OCV")]


class MhdDiag(C.Structure):
    _fields_ = [("dt", C.c_double), ("umach", C.c_double), ("timt", C.c_double), ("total_mass", C.c_double),
                ("total_energy", C.c_double), ("max_divb", C.c_double), ("nit", C.c_longlong),
                ("flags", C.c_int), ("reserved", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class MhdPlume(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("XP", "YP", "ZP", "HH", "TC", "QFH")] + \
               [(n, C.POINTER(C.c_double)) for n in ("EXX", "WYY", "ZEE")]


class MhdStaticParams(C.Structure):
    _fields_ = [("nPEy", C.c_int), ("nPEz", C.c_int), ("nTube", C.c_int), ("reserved_i", C.c_int)] + \
               [(n, C.c_double) for n in ("zMax", "PZP", "SIGMA", "POLYS", "AMPT", "AMPB", "BFH", "BZP")] + \
               [("ZEE", C.POINTER(C.c_double)), ("reserved_d", C.c_double * 4)]


NOALLOC_MAX_CELLS = 393216


class MhdFluxesNoallocArgs(C.Structure):
    _fields_ = [("nPx", C.c_int), ("nPy", C.c_int), ("nPz", C.c_int), ("switches", C.c_uint),
                ("izCon", C.c_int), ("iTCon", C.c_int), ("iBCon", C.c_int), ("reserved_i", C.c_int)] + \
               [(n, C.c_double) for n in ("RE", "PR", "THETA", "GRAV", "RY", "ANG", "RM", "BETA", "TP", "GAMMA",
                                           "SFF", "TB")] + \
               [(n, C.c_void_p) for n in ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2",
                                          "DDZ", "RKAPA", "DKAPA")] + \
               [("state", C.c_void_p * 8), ("flux", C.c_void_p * 8)]


class MhdError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None

# (name, argtypes) of every exported entry point; tests check them all.
SIGNATURES = {
    "mhd_create": [C.POINTER(MhdParams), C.c_void_p, C.POINTER(C.c_void_p)],
    "mhd_destroy": [C.c_void_p],
    "mhd_get_constants": [C.c_void_p, C.POINTER(MhdConstants)],
    "mhd_compute_constants": [C.POINTER(MhdParams), C.POINTER(MhdConstants)],
    "mhd_device_bytes": [C.c_void_p, C.POINTER(C.c_size_t)],
    "mhd_last_error": [C.c_void_p],
    "mhd_status_string": [C.c_int],
    "mhd_upload": [C.c_void_p, C.c_int, _DP],
    "mhd_download": [C.c_void_p, C.c_int, _DP],
    "mhd_upload_state": [C.c_void_p, _DP],
    "mhd_download_state": [C.c_void_p, _DP],
    "mhd_set_time": [C.c_void_p, C.c_double, C.c_longlong],
    "mhd_init_polytrope": [C.c_void_p, _DP, C.c_double, C.c_ulonglong, C.c_double],
    "mhd_fluxes": [C.c_void_p],
    "mhd_rk_zeta0": [C.c_void_p],
    "mhd_rk_zeta": [C.c_void_p, C.c_double],
    "mhd_rk_gam": [C.c_void_p, C.c_double],
    "mhd_bcon": [C.c_void_p, C.c_double],
    "mhd_communicate": [C.c_void_p],
    "mhd_cfl_dt": [C.c_void_p, _DP, _DP],
    "mhd_step": [C.c_void_p, C.c_double, C.POINTER(MhdDiag)],
    "mhd_steps": [C.c_void_p, C.c_int, C.c_double],
    "mhd_steps_cfl": [C.c_void_p, C.c_int, C.POINTER(MhdDiag)],
    "mhd_step_host": [C.c_void_p, _DP, _DP, C.c_double],
    "mhd_steps_host": [C.c_void_p, C.c_int, _DP, _DP, C.c_double],
    "mhd_set_plume": [C.c_void_p, C.POINTER(MhdPlume)],
    "mhd_selftest_convert": [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)],
    "mhd_static_state": [C.POINTER(MhdParams), C.POINTER(MhdStaticParams), _DP],
    "mhd_static_lrem_profile": [C.POINTER(MhdParams), C.POINTER(MhdStaticParams), _DP, _DP, _DP],
    "mhd_diagnostics": [C.c_void_p, C.POINTER(MhdDiag)],
    "mhd_sync": [C.c_void_p],
    "mhd_batch_create": [C.POINTER(C.c_void_p), _DP, C.c_int, C.c_void_p, C.POINTER(C.c_void_p)],
    "mhd_batch_destroy": [C.c_void_p],
    "mhd_batch_set_tile": [C.c_void_p, C.c_int],
    "mhd_batch_tile": [C.c_void_p, C.POINTER(C.c_int)],
    "mhd_batch_autotune": [C.c_void_p, C.POINTER(C.c_int), _DP],
    "mhd_batch_steps": [C.c_void_p, C.c_int],
    "mhd_batch_steps_limited": [C.c_void_p, C.c_int, C.POINTER(C.c_int)],
    "mhd_batch_set_zrange": [C.c_void_p, C.c_int],
    "mhd_batch_zrange": [C.c_void_p, C.POINTER(C.c_int)],
    "mhd_batch_autotune_bytes": [C.c_void_p, C.POINTER(C.c_ulonglong)],
    "mhd_batch_sync": [C.c_void_p],
    "mhd_write_dat0": [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _DP, C.c_int, C.c_int, C.c_int],
    "mhd_read_dat0": [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _DP, C.c_int, C.c_int, C.c_int],
    "mhd_set_device": [C.c_int],
    "mhd_timer_start": [C.c_void_p],
    "mhd_timer_stop": [C.c_void_p, _DP],
    "mhd_profile": [C.c_void_p, C.c_int],
    "mhd_profile_read": [C.c_void_p, _DP, C.POINTER(C.c_longlong)],
    "mhd_fp64_peak": [_DP],
    "mhd_fluxes_noalloc": [C.POINTER(MhdFluxesNoallocArgs), C.c_void_p],
    "mhd_host_alloc": [C.c_size_t, C.POINTER(C.c_void_p)],
    "mhd_host_free": [C.c_void_p],
}
RESTYPES = {"mhd_last_error": C.c_char_p, "mhd_status_string": C.c_char_p}


def load(path: Path | None = None):
    """Load libmhd_gb300.so (built by __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else Path(os.environ.get("MHD_GB300_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(str(p))
    for name, argt in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = argt
        fn.restype = RESTYPES.get(name, C.c_int)
    _lib = L
    return L


def check(status: int, ctx=None) -> None:
    if status != MHD_OK:
        msg = ""
        if ctx is not None and _lib is not None:
            msg = (_lib.mhd_last_error(ctx) or b"").decode(errors="replace")
        raise MhdError(status, msg)
