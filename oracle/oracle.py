"""ctypes front end of the C restatement in oracle/mhd_oracle.c.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker.  The product path never uses it.

``OracleSim`` owns numpy arrays for the 27 slots the reference keeps as
globals (3dmhddata.h:13-19) on one global domain and exposes the reference's
hot-path entry points one for one: fluxes, step_block_ZETA0/ZETA/GAM, BCON,
communicate and step.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO / "rast-3dmhd-cpp_gb300" / "python"))
from mhd_gb300.case import Case, STATE_FIELDS, FLUX_FIELDS, ZFIELDS, coordinates, metrics  # noqa: E402

BUILD_DIR = HERE / "_build"
LIB = BUILD_DIR / "libmhd_oracle.so"
SLOTS = list(STATE_FIELDS) + list(FLUX_FIELDS) + list(ZFIELDS) + ["UU", "VV", "WW"]


def build(force: bool = False) -> Path:
    """Compile the oracle (gcc, -ffp-contract=off so no FMA contraction on any host)."""
    src = HERE / "mhd_oracle.c"
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime,
                                                             (HERE / "mhd_oracle.h").stat().st_mtime):
        tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
        subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
                        "-fPIC", "-shared", str(src), "-o", str(tmp), "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


class OrcParams(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "ny", "nz", "nPz", "lMag", "lRot", "lShr", "izCon", "iTCon",
                                        "iBCon", "nthreads", "cfl_parallel")] + \
               [(n, C.c_double) for n in ("C13", "C23", "C43", "GAM1", "GAM2", "GAM3", "ZETA1", "ZETA2",
                                           "hx", "h2x", "hy", "h2y", "hz", "h2z",
                                           "RE", "PR", "REPR", "ORE", "CV", "OCV", "GAMMA", "GRAV", "THETA",
                                           "RY", "ANG", "OMX", "OMZ", "RM", "ORM", "BETA", "OBETA", "TB", "TP",
                                           "SFF")] + \
               [(n, C.POINTER(C.c_double)) for n in ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY",
                                                      "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")] + \
               [(n, C.POINTER(C.c_double)) for n in ("EXX", "WYY", "ZEE")] + \
               [(n, C.c_double) for n in ("XP", "YP", "ZP", "HH", "TC", "QFH", "TIMT")] + \
               [("lRem", C.c_int), ("pad2_", C.c_int)] + \
               [(n, C.c_double) for n in ("TU", "DZTU", "DZTB")]


class OrcFields(C.Structure):
    _fields_ = [("a", C.POINTER(C.c_double) * len(SLOTS))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = C.CDLL(str(path))
        P, F = C.POINTER(OrcParams), C.POINTER(OrcFields)
        L.orc_set_constants.argtypes = [P, C.c_int, C.c_int, C.c_int]
        L.orc_fluxes.argtypes = [P, F]
        L.orc_rk_zeta0.argtypes = [P, F]
        L.orc_rk_zeta.argtypes = [P, F, C.c_double]
        L.orc_rk_gam.argtypes = [P, F, C.c_double]
        L.orc_bcon.argtypes = [P, F, C.c_double]
        L.orc_communicate.argtypes = [P, F]
        L.orc_cfl_dt.argtypes = [P, F, C.POINTER(C.c_double)]
        L.orc_cfl_dt.restype = C.c_double
        L.orc_steps.argtypes = [P, F, C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleSim:
    """Single-domain CPU oracle instance."""

    def __init__(self, case: Case, state: dict | None = None, nthreads: int = 1):
        self.case = case
        self.L = lib()
        self.arr = {k: np.zeros(case.shape) for k in SLOTS}
        self.m = metrics(case)
        self._metric_arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in self.m.arrays()]
        p = OrcParams()
        p.nx, p.ny, p.nz = case.nx, case.ny, case.nz
        p.lMag, p.lRot, p.lShr = int(case.lMag), int(case.lRot), int(case.lShr)
        p.izCon, p.iTCon, p.iBCon = case.izCon, case.iTCon, case.iBCon
        p.nthreads = nthreads
        for k in ("RE", "PR", "THETA", "GRAV", "RY", "ANG", "RM", "BETA", "GAMMA", "TP", "SFF"):
            setattr(p, k, float(getattr(case, k)))
        p.TB = case.tb
        names = ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")
        for n, a in zip(names, self._metric_arrays):
            setattr(p, n, _dptr(a))
        self._coord_arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in coordinates(case)]
        for n, a in zip(("EXX", "WYY", "ZEE"), self._coord_arrays):
            setattr(p, n, _dptr(a))
        for k in ("XP", "YP", "ZP", "HH", "TC", "QFH", "TU", "DZTU", "DZTB"):
            setattr(p, k, float(getattr(case, k)))
        p.lRem = int(case.lRem)
        self.L.orc_set_constants(C.byref(p), case.nPx, case.nPy, case.nPz)
        self.p = p
        self.f = OrcFields()
        for i, k in enumerate(SLOTS):
            self.f.a[i] = _dptr(self.arr[k])
        self.timt = 0.0
        if state is not None:
            self.load(state)

    def load(self, state: dict) -> None:
        for k, v in state.items():
            if k in self.arr:
                self.arr[k][...] = v

    def state(self) -> dict:
        return {k: self.arr[k].copy() for k in STATE_FIELDS}

    # reference entry points -------------------------------------------------
    def fluxes(self) -> None:
        self.p.TIMT = self.timt
        self.L.orc_fluxes(C.byref(self.p), C.byref(self.f))

    def step_block_ZETA0(self) -> None:
        self.L.orc_rk_zeta0(C.byref(self.p), C.byref(self.f))

    def step_block_ZETA(self, coef: float) -> None:
        self.L.orc_rk_zeta(C.byref(self.p), C.byref(self.f), coef)

    def step_block_GAM(self, coef: float) -> None:
        self.L.orc_rk_gam(C.byref(self.p), C.byref(self.f), coef)

    def BCON(self, timt: float | None = None) -> None:
        rc = self.L.orc_bcon(C.byref(self.p), C.byref(self.f), self.timt if timt is None else timt)
        if rc:
            raise ValueError("BCON: unsupported wall condition")

    def communicate(self) -> None:
        self.L.orc_communicate(C.byref(self.p), C.byref(self.f))

    def cfl_dt(self) -> tuple[float, float]:
        um = C.c_double(0.0)
        dt = self.L.orc_cfl_dt(C.byref(self.p), C.byref(self.f), C.byref(um))
        return dt, um.value

    def steps(self, n: int, dt: float | None = None) -> np.ndarray:
        """n RK3 steps; dt None uses the case's fixed dt, dt <= 0 the CFL step."""
        d = self.case.dt if dt is None else dt
        t = C.c_double(self.timt)
        hist = np.zeros(max(n, 1))
        rc = self.L.orc_steps(C.byref(self.p), C.byref(self.f), n, d, C.byref(t), _dptr(hist))
        if rc:
            raise ValueError("step: unsupported wall condition")
        self.timt = t.value
        return hist[:n]
