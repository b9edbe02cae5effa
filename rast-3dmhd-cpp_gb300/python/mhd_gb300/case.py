"""Run description and host-side initial state for one 3dmhd instance.

A ``Case`` carries what the reference keeps in 3dmhdparam.h (grid sizes and
physics switches, 3dmhdparam.h:8-17,25-27,86-107) and in setup()'s ``par[]``
table (3dmhdset.h:7-24), plus the pieces of a synthetic run the reference
does not have: a tanh-stretched z grid, a polytropic layer with seeded
Gaussian temperature noise, a uniform vertical field and a fixed time step.

Arrays follow the reference layout ``f[z][y][x]`` (x fastest, 3dmhddata.h:8)
on the single global domain with one ghost cell per side:
``nx = nPx + 2``, ``ny = nPy + 2``, ``nz = nPz + 2``.  z is depth: index 1 is
the top wall and index nz-2 the bottom wall.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field

import numpy as np

# Field order of the state, of the checkpoint records (3dmhdio.h:23-33) and of
# the C-ABI field ids.
STATE_FIELDS = ("RU", "RV", "RW", "TT", "RO", "BX", "BY", "BZ")
FLUX_FIELDS = ("FU", "FV", "FW", "FR", "FT", "WW1", "WW2", "WW3")
ZFIELDS = ("ZRU", "ZRV", "ZRW", "ZTT", "ZRO", "ZBX", "ZBY", "ZBZ")


def f32(v: float) -> float:
    """Value of a C ``float`` literal widened to double (e.g. ``0.2f``)."""
    return float(np.float32(v))


GAMMA_DEFAULT = float(np.float32(5.0) / np.float32(3.0))  # par[53] = 5.0f / 3.0f, 3dmhdset.h:23


@dataclass
class Case:
    nPx: int
    nPy: int
    nPz: int
    lMag: bool = True
    lRot: bool = False
    lShr: bool = False
    lRem: bool = False      # Rempel relaxation (3dmhdparam.h:14); needs TU, DZTU, DZTB
    izCon: int = 0          # 0 fixed bottom temperature TB, 1 fixed flux (3dmhdsub.h:842-864)
    iTCon: int = 0          # 0/1/4 upper temperature condition (3dmhdsub.h:750-810)
    iBCon: int = 0          # 0: Bz = 0 on both walls (3dmhdsub.h:811-817,865-871)
    RE: float = 100.0
    PR: float = 1.0
    THETA: float = 4.5
    GRAV: float = 9.0
    RY: float = 10.0
    ANG: float = 0.0
    RM: float = 100.0
    BETA: float = 2.0
    TP: float = 0.0
    # plume: top-boundary cooling spot (TP != 0, iTCon 0/1) and internal heat
    # source (iTCon 2) at (XP, YP, ZP), width HH, time scales TC, QFH
    # (3dmhd.cpp:413-426; 3dmhdsub.h:443-459,750-778)
    XP: float = 0.0
    YP: float = 0.0
    ZP: float = 0.0
    HH: float = 0.0
    TC: float = 0.0
    QFH: float = 0.0
    # lRem wall values of the static model (Static(), 3dmhdphsic.h:592-594)
    TU: float = 1.0
    DZTU: float = 0.0
    DZTB: float = 0.0
    xMax: float = 6.0
    yMax: float = 6.0
    zMax: float = 2.0
    # fresh-start model of Static() (3dmhdphsic.h:549-763; par[8..10], par[19..22]):
    # conductivity step at zz = PZP of width SIGMA to the polytrope of index
    # POLYS, temperature noise AMPT, Gaussian Bx layer AMPB of FWHM BFH at BZP
    PZP: float = 0.0
    SIGMA: float = 0.0
    POLYS: float = 0.0
    AMPT: float = 0.0
    AMPB: float = 0.0
    BFH: float = 0.0
    BZP: float = 0.0
    # flux-tube model of tube() (3dmhdparam.h:124, 3dmhdphsic.h:765-1027; lMag with
    # AMPB = 0): model number and par[34..38] (XCENT, ZCENT, R_MAX, C_MT, A)
    nTube: int = 0
    XCENT: float = 0.0
    ZCENT: float = 0.0
    R_MAX: float = 0.0
    C_MT: float = 0.0
    A_TUBE: float = 0.0
    GAMMA: float = GAMMA_DEFAULT
    SFF: float = f32(0.8)   # 3dmhdparam.h:111
    z_stretch: float = 1.5  # tanh stretch factor; 0 gives the reference's uniform grid
    TB: float | None = None  # bottom temperature; default is the polytrope's 1 + THETA*zMax
    seed: int = 0
    noise: float = 1e-3     # relative Gaussian temperature noise
    bz0: float = 1e-3       # uniform vertical field in the interior
    dt: float = 1e-4
    # decomposition of the multi-rank reference oracle (needs nPEz >= 2, 3dmhdparam.h:20)
    nPEy: int = 2
    nPEz: int = 2
    name: str = ""

    # ---- derived sizes -------------------------------------------------
    @property
    def nx(self) -> int:
        return self.nPx + 2

    @property
    def ny(self) -> int:
        return self.nPy + 2

    @property
    def nz(self) -> int:
        return self.nPz + 2

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.nz, self.ny, self.nx)

    @property
    def cells(self) -> int:
        return self.nPx * self.nPy * self.nPz

    @property
    def tb(self) -> float:
        return float(self.TB) if self.TB is not None else 1.0 + self.THETA * self.zMax

    @property
    def nfields(self) -> int:
        return 8 if self.lMag else 5

    def replace(self, **kw) -> "Case":
        return dataclasses.replace(self, **kw)

    def to_dict(self) -> dict:
        return dataclasses.asdict(self)


# ---------------------------------------------------------------------------
# grid metrics
# ---------------------------------------------------------------------------
def uniform_metric(n_interior: int, umax: float):
    """Metric arrays of the uniform grid, as mkGrid(nGrid=0) and the Jacobi
    routines build them (3dmhdphsic.h:36-41,79-156): dxi/du = 1/umax,
    d2xi/du2 = 0, DD = (1/(n-1)) / (dxi/du).  Ghost entries repeat the walls."""
    n = n_interior + 2
    orx = f32(np.float32(1.0) / np.float32(n_interior - 1))
    d1 = np.full(n, 1.0 / umax)
    d2 = np.zeros(n)
    dd = np.full(n, orx * (1.0 / d1[0]))
    return d1, d2, dd


def tanh_metric(n_interior: int, umax: float, s: float):
    """Symmetric tanh clustering towards both walls.

    u(xi) = umax/2 * (1 + tanh(s(2xi-1))/tanh(s)),  xi in [0, 1].
    Returns dxi/du and d2xi/du2 at the n_interior nodes (plus repeated ghost
    entries) and the DD spacing array used by the CFL estimate.
    """
    if s == 0.0:
        return uniform_metric(n_interior, umax)
    xi = np.arange(n_interior, dtype=np.float64) / (n_interior - 1)
    a = s * (2.0 * xi - 1.0)
    th = np.tanh(a)
    sech2 = 1.0 - th * th
    ts = np.tanh(s)
    du = umax * s * sech2 / ts                        # du/dxi
    d2u = -4.0 * umax * s * s * th * sech2 / ts       # d2u/dxi2
    dxidu = 1.0 / du
    d2xidu2 = -d2u / (du * du * du)
    orx = 1.0 / (n_interior - 1)
    dd = orx * (1.0 / dxidu)
    pad = lambda v: np.concatenate([[v[0]], v, [v[-1]]])
    return pad(dxidu), pad(d2xidu2), pad(dd)


def coordinates(case: Case) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """EXX, WYY, ZEE: the x, y, z coordinates of every index (x and y
    uniform, extended linearly into the ghosts; z from z_coordinate)."""
    x = case.xMax * (np.arange(case.nx, dtype=np.float64) - 1.0) / (case.nPx - 1)
    y = case.yMax * (np.arange(case.ny, dtype=np.float64) - 1.0) / (case.nPy - 1)
    return x, y, z_coordinate(case)


def z_coordinate(case: Case) -> np.ndarray:
    """Depth of every z index (ghosts repeat the walls)."""
    n = case.nPz
    xi = np.arange(n, dtype=np.float64) / (n - 1)
    if case.z_stretch == 0.0:
        z = case.zMax * xi
    else:
        s = case.z_stretch
        z = 0.5 * case.zMax * (1.0 + np.tanh(s * (2.0 * xi - 1.0)) / np.tanh(s))
    return np.concatenate([[z[0]], z, [z[-1]]])


@dataclass
class Metrics:
    dxxdx: np.ndarray
    d2xxdx2: np.ndarray
    DDX: np.ndarray
    dyydy: np.ndarray
    d2yydy2: np.ndarray
    DDY: np.ndarray
    dzzdz: np.ndarray
    d2zzdz2: np.ndarray
    DDZ: np.ndarray
    RKAPA: np.ndarray
    DKAPA: np.ndarray

    def arrays(self):
        return [self.dxxdx, self.d2xxdx2, self.DDX, self.dyydy, self.d2yydy2, self.DDY,
                self.dzzdz, self.d2zzdz2, self.DDZ, self.RKAPA, self.DKAPA]


def metrics(case: Case) -> Metrics:
    dx = uniform_metric(case.nPx, case.xMax)
    dy = uniform_metric(case.nPy, case.yMax)
    dz = tanh_metric(case.nPz, case.zMax, case.z_stretch)
    # PZP = 0: constant conductivity profile (3dmhd.cpp:478-482)
    rk = np.ones(case.nz)
    dk = np.zeros(case.nz)
    return Metrics(*dx, *dy, *dz, rk, dk)


# ---------------------------------------------------------------------------
# initial state
# ---------------------------------------------------------------------------
def periodic_fill(a: np.ndarray) -> None:
    """x/y ghosts become periodic images (final semantics of comm_mpi,
    3dmhdmpi.h:32-143, on one domain): index 0 <- n-2, index n-1 <- 1."""
    a[:, 0, :] = a[:, -2, :]
    a[:, -1, :] = a[:, 1, :]
    a[:, :, 0] = a[:, :, -2]
    a[:, :, -1] = a[:, :, 1]


def initial_state(case: Case) -> dict[str, np.ndarray]:
    """Polytrope T = 1 + THETA*z, rho = T**m with m = GRAV/THETA - 1, seeded
    multiplicative Gaussian temperature noise on the interior, a uniform Bz on
    interior planes (zero on the walls, where iBCon=0 pins it), zero momenta.
    The z ghost planes hold the noise-free wall values."""
    nz, ny, nx = case.shape
    z = z_coordinate(case)
    m = case.GRAV / case.THETA - 1.0
    T1 = 1.0 + case.THETA * z
    R1 = T1 ** m
    TT = np.broadcast_to(T1[:, None, None], case.shape).copy()
    RO = np.broadcast_to(R1[:, None, None], case.shape).copy()
    rng = np.random.default_rng(case.seed)
    noise = rng.standard_normal((case.nPz, case.nPy, case.nPx))
    TT[1:-1, 1:-1, 1:-1] *= 1.0 + case.noise * noise
    st = {k: np.zeros(case.shape) for k in STATE_FIELDS}
    st["TT"] = TT
    st["RO"] = RO
    if case.lMag:
        st["BZ"][2:-2, :, :] = case.bz0
    if case.lShr:
        # moving-wall shear runs start from the wall velocities BCON imposes
        # (3dmhdsub.h:729-734,821-826): rho*v = +rho on top, -rho at the bottom
        st["RV"][1] = RO[1]
        st["RV"][-2] = -RO[-2]
    for k in STATE_FIELDS:
        periodic_fill(st[k])
    return st


_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def device_initial_state(case: Case) -> dict[str, np.ndarray]:
    """Host mirror of the device initial state (mhd_init_polytrope): the same
    polytrope as initial_state, with the Gaussian noise drawn by Box-Muller
    from splitmix64 of (seed, interior cell index) instead of numpy's stream."""
    nz, ny, nx = case.shape
    z = z_coordinate(case)
    m = case.GRAV / case.THETA - 1.0
    T1 = 1.0 + case.THETA * z
    R1 = T1 ** m
    cell = np.arange(case.nPz * case.nPy * case.nPx, dtype=np.uint64)
    seed = np.uint64(int(case.seed) & 0xFFFFFFFFFFFFFFFF)
    h1 = _splitmix64(seed ^ _splitmix64(np.uint64(2) * cell))
    h2 = _splitmix64(seed ^ _splitmix64(np.uint64(2) * cell + np.uint64(1)))
    u1 = ((h1 >> np.uint64(11)) + np.uint64(1)).astype(np.float64) * (1.0 / 9007199254740992.0)
    u2 = ((h2 >> np.uint64(11)) + np.uint64(1)).astype(np.float64) * (1.0 / 9007199254740992.0)
    gauss = (np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)).reshape(case.nPz, case.nPy, case.nPx)
    TT = np.broadcast_to(T1[:, None, None], case.shape).copy()
    RO = np.broadcast_to(R1[:, None, None], case.shape).copy()
    TT[1:-1, 1:-1, 1:-1] *= 1.0 + case.noise * gauss
    st = {k: np.zeros(case.shape) for k in STATE_FIELDS}
    st["TT"], st["RO"] = TT, RO
    if case.lMag:
        st["BZ"][2:-2, :, :] = case.bz0
    if case.lShr:
        st["RV"][1] = RO[1]
        st["RV"][-2] = -RO[-2]
    for k in STATE_FIELDS:
        periodic_fill(st[k])
    return st


def small_cases() -> dict[str, Case]:
    """Small switch-coverage cases shared by the golden fixtures and the
    parity tests (grid sizes the CPU oracle finishes in well under a second)."""
    base = dict(nPx=12, nPy=8, nPz=8, nPEy=2, nPEz=2, seed=7, noise=1e-2, bz0=1e-2, dt=2e-4)
    return {
        "mhd_fixedT": Case(name="mhd_fixedT", **base),
        "mhd_rot_shr": Case(name="mhd_rot_shr", lRot=True, lShr=True, **base),
        "hydro_default_bc": Case(name="hydro_default_bc", lMag=False, izCon=1, iTCon=4, TP=f32(0.1), **base),
        "mhd_rot_flux": Case(name="mhd_rot_flux", lRot=True, ANG=0.3, izCon=1, iTCon=1, **base),
        "hydro_shr": Case(name="hydro_shr", lMag=False, lShr=True, izCon=0, iTCon=4, TP=f32(0.1), **base),
    }


def plume_cases() -> dict[str, Case]:
    """Cases with the plume terms: the cooling spot on the top wall (TP != 0
    with iTCon 0, time-dependent through TC, and with iTCon 1) and the
    internal heat sink (iTCon 2, time-dependent through TC and QFH)."""
    base = dict(nPx=12, nPy=8, nPz=8, nPEy=2, nPEz=2, seed=7, noise=1e-2, bz0=1e-2, dt=2e-4,
                XP=3.0, YP=3.0, HH=1.5)
    return {
        "plume_top0": Case(name="plume_top0", iTCon=0, TP=0.4, TC=0.01, **base),
        "plume_top1": Case(name="plume_top1", lMag=False, iTCon=1, izCon=1, TP=0.3, **base),
        "plume_src2": Case(name="plume_src2", lRot=True, iTCon=2, TP=2.0, TC=1e-4, QFH=2e-4,
                           **dict(base, HH=1.0, ZP=1.0)),
    }


def lrem_cases() -> dict[str, Case]:
    """lRem (Rempel relaxation) cases on one y rank (the reference's
    horizontal_mean sums over every rank when nPEy > 1, 3dmhdsub.h:714-717):
    a fixed top temperature TU with iTCon 0 and the fixed-gradient walls
    (DZTU, DZTB) with iTCon 1, izCon 1."""
    base = dict(nPx=12, nPy=8, nPz=8, nPEy=1, nPEz=2, seed=7, noise=1e-2, bz0=1e-2, dt=2e-4, lRem=True)
    return {
        "lrem_fixedT": Case(name="lrem_fixedT", iTCon=0, izCon=0, TU=1.05, **base),
        "lrem_flux": Case(name="lrem_flux", lMag=False, lRot=True, iTCon=1, izCon=1, DZTU=-0.03, DZTB=0.02, **base),
    }


def static_cases() -> dict[str, Case]:
    """Fresh-start cases of Static(): the polytrope with a Bx layer and noise
    on 2 x 2 ranks, the conductivity step (PZP, SIGMA, POLYS) on 1 x 4 ranks
    with a layer that meets the z-rank edges, lShr's RV noise with the
    zero field of tube() (nTube = 0), and lRem's ODE background."""
    base = dict(nPx=12, nPy=8, nPz=8, seed=7)
    return {
        "static_layer": Case(name="static_layer", nPEy=2, nPEz=2, AMPT=0.02, AMPB=0.1, BFH=0.5, BZP=1.2, **base),
        "static_kappa": Case(name="static_kappa", lMag=True, nPEy=1, nPEz=4, PZP=0.6, SIGMA=0.1, POLYS=1.5,
                             AMPT=0.05, AMPB=0.3, BFH=0.8, BZP=0.9, **base),
        "static_shr": Case(name="static_shr", lShr=True, lRot=True, nPEy=2, nPEz=2, AMPT=0.03, **base),
        "static_hydro": Case(name="static_hydro", lMag=False, nPEy=4, nPEz=2, PZP=0.3, SIGMA=0.05, POLYS=1.0,
                             AMPT=0.01, **base),
        # lRem: the ODE background of getbackground (zMax = 1.5: no level at
        # depth 2, where the reference's integration aborts)
        "static_lrem": Case(name="static_lrem", lMag=True, lRem=True, zMax=1.5, nPEy=2, nPEz=2, AMPT=0.02,
                            AMPB=0.1, BFH=0.5, BZP=0.9, **base),
    }


def config0() -> Case:
    """64x64x32 plain FP64 MHD run: polytrope index 1 (THETA=4.5, GRAV=9,
    density contrast 10), tanh z grid (1.5), noise 1e-3, Bz=1e-3, 1/Re=1e-2,
    Pr=1, Pm=1, dt=1e-4, 100 steps; the oracle runs it on 2x2 ranks."""
    return Case(name="config0_64x64x32", nPx=64, nPy=64, nPz=32, lMag=True, seed=1, nPEy=2, nPEz=2)


def config3() -> Case:
    """256x256x128 MHD seeded as the plain-method configuration but with
    noise amplitude 1e-2: the FP32-storage precision run (1000 steps)."""
    return Case(name="config3_256x256x128", nPx=256, nPy=256, nPz=128, lMag=True, noise=1e-2, seed=1, nPEy=2, nPEz=2)


def config2_batch(n: int = 64, seed: int = 2) -> list:
    """64 independent FP64 MHD instances of uneven sizes: nx = ny from
    {32, 48, 64, 96, 128}, nz from {32, 64}, per-instance seed, 1/Re
    log-uniform in [3e-3, 3e-2], Bz0 log-uniform in [1e-4, 1e-2]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nxy = int(rng.choice([32, 48, 64, 96, 128]))
        nz = int(rng.choice([32, 64]))
        ore = float(np.exp(rng.uniform(np.log(3e-3), np.log(3e-2))))
        bz = float(np.exp(rng.uniform(np.log(1e-4), np.log(1e-2))))
        out.append(Case(name=f"batch{i}", nPx=nxy, nPy=nxy, nPz=nz, lMag=True, RE=1.0 / ore, bz0=bz,
                        seed=int(rng.integers(1 << 30))))
    return out


def config1() -> Case:
    """512x512x256 FP64 MHD with rotation 0.1 about z and the shear switch."""
    return Case(name="config1_512x512x256", nPx=512, nPy=512, nPz=256, lMag=True, lRot=True, lShr=True,
                RY=10.0, ANG=0.0, seed=1, nPEy=4, nPEz=4)
