"""Host-side mirror of the reference's per-timestep interface over the C ABI.

``Simulation`` exposes the reference's entry points under their own names
(fluxes, step_block_ZETA0/ZETA/GAM, BCON, communicate, step; 3dmhdsub.h:18-22,
3dmhdmpi.h:11) so a test or a driver reads like the reference's own code,
while every call runs on the GPU through libmhd_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .case import Case, STATE_FIELDS, coordinates, metrics


def params_for(case: Case, path: str = "fused", precision: str = "fp64") -> tuple[abi.MhdParams, list]:
    """mhd_params for a case; returns the struct and the arrays it points to."""
    m = metrics(case)
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in m.arrays()]
    p = abi.MhdParams()
    p.nPx, p.nPy, p.nPz = case.nPx, case.nPy, case.nPz
    p.switches = (abi.SW_LROT if case.lRot else 0) | (abi.SW_LMAG if case.lMag else 0) | \
                 (abi.SW_LSHR if case.lShr else 0) | (abi.SW_LREM if case.lRem else 0)
    p.TU, p.DZTU, p.DZTB = float(case.TU), float(case.DZTU), float(case.DZTB)
    p.ixCon = p.iyCon = 0
    p.izCon, p.iTCon, p.iBCon = case.izCon, case.iTCon, case.iBCon
    p.precision = abi.PREC_FP64 if precision == "fp64" else abi.PREC_FP32
    p.path = abi.PATH_FUSED if path == "fused" else abi.PATH_PARITY
    for k in ("RE", "PR", "THETA", "GRAV", "RY", "ANG", "RM", "BETA", "TP", "GAMMA", "SFF"):
        setattr(p, k, float(getattr(case, k)))
    p.TB = case.tb
    names = ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")
    for n, a in zip(names, keep):
        setattr(p, n, a.ctypes.data_as(C.POINTER(C.c_double)))
    return p, keep


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def static_state(case: Case, nPEy: int | None = None, nPEz: int | None = None) -> dict:
    """The reference's fresh-start state for ``case`` (Static() and
    communicate(), 3dmhdphsic.h:549-763, 3dmhd.cpp:111-142) from
    mhd_static_state: a dict field -> (nz, ny, nx) array.  The Bx layer
    depends on the z split of the run reproduced (default: the case's
    nPEy x nPEz).  Host computation; no GPU is needed."""
    L = abi.load()
    p, keep = params_for(case)
    sp = abi.MhdStaticParams()
    sp.nPEy = case.nPEy if nPEy is None else nPEy
    sp.nPEz = case.nPEz if nPEz is None else nPEz
    sp.nTube = case.nTube
    for k in ("zMax", "PZP", "SIGMA", "POLYS", "AMPT", "AMPB", "BFH", "BZP"):
        setattr(sp, k, float(getattr(case, k)))
    zee = np.ascontiguousarray(coordinates(case)[2], dtype=np.float64)
    sp.ZEE = _dp(zee)
    out = np.empty((case.nfields,) + case.shape, dtype=np.float64)
    abi.check(L.mhd_static_state(C.byref(p), C.byref(sp), _dp(out)))
    return {k: out[i] for i, k in enumerate(STATE_FIELDS[:case.nfields])}


def static_lrem_profile(case: Case) -> dict:
    """With lRem, the conductivity profile and wall values Static() derives
    with its background (3dmhdphsic.h:565-594): RKAPA and DKAPA of every z
    plane (ghosts included) and TU, DZTU, DZTB (mhd_static_lrem_profile)."""
    L = abi.load()
    p, keep = params_for(case)
    sp = abi.MhdStaticParams()
    sp.zMax = float(case.zMax)
    rk, drk, walls = np.empty(case.nz), np.empty(case.nz), np.empty(3)
    abi.check(L.mhd_static_lrem_profile(C.byref(p), C.byref(sp), _dp(rk), _dp(drk), _dp(walls)))
    return {"RKAPA": rk, "DKAPA": drk, "TU": float(walls[0]), "DZTU": float(walls[1]), "DZTB": float(walls[2])}


class Simulation:
    """One device-resident 3dmhd instance."""

    def __init__(self, case: Case, path: str = "fused", precision: str = "fp64", metric_override: dict | None = None):
        self.case = case
        self.L = abi.load()
        p, keep = params_for(case, path, precision)
        if metric_override:
            names = ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")
            for j, n in enumerate(names):
                if n in metric_override:
                    keep[j] = np.ascontiguousarray(metric_override[n], dtype=np.float64)
                    setattr(p, n, _dp(keep[j]))
        ctx = C.c_void_p()
        st = self.L.mhd_create(C.byref(p), None, C.byref(ctx))
        if st != abi.MHD_OK:
            raise abi.MhdError(st, "mhd_create failed")
        self.ctx = ctx
        if case.iTCon == 2 or (case.TP != 0.0 and case.iTCon in (0, 1)):
            self.set_plume()
        self._keep = keep
        self.timt = 0.0

    # ---- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.L.mhd_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st: int) -> None:
        abi.check(st, self.ctx)

    def constants(self) -> dict:
        k = abi.MhdConstants()
        self._ck(self.L.mhd_get_constants(self.ctx, C.byref(k)))
        return {n: getattr(k, n) for n, _ in k._fields_}

    def device_bytes(self) -> int:
        b = C.c_size_t()
        self._ck(self.L.mhd_device_bytes(self.ctx, C.byref(b)))
        return b.value

    # ---- transfers --------------------------------------------------------
    def upload(self, field: str, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.case.shape
        self._ck(self.L.mhd_upload(self.ctx, abi.FIELD_IDS[field], _dp(a)))
        self._ck(self.L.mhd_sync(self.ctx))

    def download(self, field: str) -> np.ndarray:
        out = np.empty(self.case.shape)
        self._ck(self.L.mhd_download(self.ctx, abi.FIELD_IDS[field], _dp(out)))
        return out

    def upload_state(self, state: dict) -> None:
        for k in STATE_FIELDS[:self.case.nfields]:
            self.upload(k, state[k])

    def download_state(self) -> dict:
        return {k: self.download(k) for k in STATE_FIELDS[:self.case.nfields]}

    def init_on_device(self) -> None:
        """The case's synthetic initial state generated on the GPU
        (case.device_initial_state is its host mirror)."""
        from .case import z_coordinate
        zc = np.ascontiguousarray(z_coordinate(self.case), dtype=np.float64)
        self._ck(self.L.mhd_init_polytrope(self.ctx, _dp(zc), float(self.case.noise), int(self.case.seed) & (2**64 - 1),
                                           float(self.case.bz0)))

    def set_time(self, timt: float, nit: int = 0) -> None:
        self.timt = timt
        self._ck(self.L.mhd_set_time(self.ctx, timt, nit))

    def set_plume(self) -> None:
        """Plume parameters and coordinates of the case (mhd_set_plume)."""
        self._plume_coords = [np.ascontiguousarray(a, dtype=np.float64) for a in coordinates(self.case)]
        pl = abi.MhdPlume()
        for k in ("XP", "YP", "ZP", "HH", "TC", "QFH"):
            setattr(pl, k, float(getattr(self.case, k)))
        pl.EXX, pl.WYY, pl.ZEE = (_dp(a) for a in self._plume_coords)
        self._ck(self.L.mhd_set_plume(self.ctx, C.byref(pl)))

    # ---- the reference's entry points ---------------------------------------
    def fluxes(self) -> None:
        self._ck(self.L.mhd_fluxes(self.ctx))

    def step_block_ZETA0(self) -> None:
        self._ck(self.L.mhd_rk_zeta0(self.ctx))

    def step_block_ZETA(self, coef: float) -> None:
        self._ck(self.L.mhd_rk_zeta(self.ctx, coef))

    def step_block_GAM(self, coef: float) -> None:
        self._ck(self.L.mhd_rk_gam(self.ctx, coef))

    def BCON(self, timt: float | None = None) -> None:
        self._ck(self.L.mhd_bcon(self.ctx, self.timt if timt is None else timt))

    def communicate(self) -> None:
        self._ck(self.L.mhd_communicate(self.ctx))

    def cfl_dt(self) -> tuple[float, float]:
        dt, um = C.c_double(), C.c_double()
        self._ck(self.L.mhd_cfl_dt(self.ctx, C.byref(dt), C.byref(um)))
        return dt.value, um.value

    def step(self, dt: float | None = None) -> dict:
        """One RK3 step; dt None uses the case's fixed dt, dt <= 0 the CFL step."""
        d = abi.MhdDiag()
        self._ck(self.L.mhd_step(self.ctx, self.case.dt if dt is None else dt, C.byref(d)))
        self.timt = d.timt
        return d.as_dict()

    def steps(self, n: int, dt: float | None = None) -> None:
        self._ck(self.L.mhd_steps(self.ctx, n, self.case.dt if dt is None else dt))

    def step_host(self, host_in, host_out, dt: float | None = None) -> None:
        """One fused step from a host state to a host state (mhd_step_host);
        host_in / host_out are float64 arrays of nf x nz x ny x nx (or None),
        the upload / step / download overlapped slab by slab."""
        self._ck(self.L.mhd_step_host(self.ctx, self._host_ptr(host_in), self._host_ptr(host_out),
                                      self.case.dt if dt is None else dt))

    def steps_host(self, n: int, host_in, host_out, dt: float | None = None) -> None:
        """n fused steps through host memory (mhd_steps_host): step 0 reads
        host_in, every later step the previous result in host_out, and every
        step writes host_out; the steps are enqueued back to back."""
        self._ck(self.L.mhd_steps_host(self.ctx, n, self._host_ptr(host_in), self._host_ptr(host_out),
                                       self.case.dt if dt is None else dt))

    def _host_ptr(self, a):
        """A float64 state array of nf x nz x ny x nx as a double pointer (None: NULL)."""
        if a is None:
            return None
        assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.case.nfields * self.ncell_all
        return _dp(a)

    @property
    def ncell_all(self) -> int:
        return self.case.nx * self.case.ny * self.case.nz

    def steps_cfl(self, n: int, check: bool = True) -> tuple[int, dict]:
        """n steps with the CFL dt of each (the reference's run mode).
        Returns (status, diag); status MHD_ERR_DT_TOO_SMALL is the halt of
        3dmhd.cpp:292 and raises only when check is set."""
        d = abi.MhdDiag()
        st = self.L.mhd_steps_cfl(self.ctx, n, C.byref(d))
        if st in (abi.MHD_OK, abi.MHD_ERR_DT_TOO_SMALL):
            self.timt = d.timt
        if check:
            self._ck(st)
        return st, d.as_dict()

    # ---- timing on the context's stream -------------------------------------
    def timer_start(self) -> None:
        self._ck(self.L.mhd_timer_start(self.ctx))

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._ck(self.L.mhd_timer_stop(self.ctx, C.byref(ms)))
        return ms.value

    def profile(self, enable: bool) -> None:
        self._ck(self.L.mhd_profile(self.ctx, int(enable)))

    def profile_read(self) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_longlong()
        self._ck(self.L.mhd_profile_read(self.ctx, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def sync(self) -> None:
        self._ck(self.L.mhd_sync(self.ctx))

    def diagnostics(self, check: bool = True) -> dict:
        d = abi.MhdDiag()
        st = self.L.mhd_diagnostics(self.ctx, C.byref(d))
        if check:
            self._ck(st)
        return d.as_dict()


class Batch:
    """Ragged batch of FP64 fused-path Simulations stepped together
    (one persistent launch per substage, CUDA-graph step, autotuned tile)."""

    TILES = ("32x4", "32x8", "16x8")

    def __init__(self, sims: list, dts: list | None = None):
        self.L = abi.load()
        self.sims = list(sims)
        n = len(self.sims)
        ctxs = (C.c_void_p * n)(*[s.ctx.value for s in self.sims])
        d = np.ascontiguousarray([s.case.dt if dts is None else dts[i] for i, s in enumerate(self.sims)],
                                 dtype=np.float64)
        self._dts = d
        b = C.c_void_p()
        st = self.L.mhd_batch_create(ctxs, _dp(d), n, None, C.byref(b))
        if st != abi.MHD_OK:
            raise abi.MhdError(st, "mhd_batch_create failed")
        self.b = b

    def close(self) -> None:
        if getattr(self, "b", None):
            self.L.mhd_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tile(self, tile: int) -> None:
        abi.check(self.L.mhd_batch_set_tile(self.b, tile))

    def tile(self) -> int:
        t = C.c_int()
        abi.check(self.L.mhd_batch_tile(self.b, C.byref(t)))
        return t.value

    def autotune(self, report: bool = True) -> tuple[int, list]:
        chosen = C.c_int()
        ms = np.zeros(3)
        abi.check(self.L.mhd_batch_autotune(self.b, C.byref(chosen), _dp(ms) if report else None))
        return chosen.value, list(ms)

    def steps(self, n: int) -> None:
        abi.check(self.L.mhd_batch_steps(self.b, n))
        for s in self.sims:
            s.timt += n * s.case.dt

    def steps_limited(self, n: int, max_steps) -> None:
        """n batched steps in which instance i takes only min(n, max_steps[i])."""
        lim = (C.c_int * len(self.sims))(*[int(m) for m in max_steps])
        abi.check(self.L.mhd_batch_steps_limited(self.b, n, lim))
        for s, m in zip(self.sims, max_steps):
            s.timt += min(n, int(m)) * s.case.dt

    def set_zrange(self, zmax: int) -> None:
        abi.check(self.L.mhd_batch_set_zrange(self.b, zmax))

    def zrange(self) -> int:
        z = C.c_int()
        abi.check(self.L.mhd_batch_zrange(self.b, C.byref(z)))
        return z.value

    def autotune_bytes(self) -> int:
        v = C.c_ulonglong()
        abi.check(self.L.mhd_batch_autotune_bytes(self.b, C.byref(v)))
        return v.value

    def sync(self) -> None:
        abi.check(self.L.mhd_batch_sync(self.b))
