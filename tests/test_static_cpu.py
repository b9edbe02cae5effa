"""The fresh-start initial state (mhd_static_state) against the reference's
own Static() + communicate() (3dmhdphsic.h:549-763, 3dmhd.cpp:111-142).

The fixtures were written by tests/golden/make_golden.py from the compiled
reference (harness mode 5) on its rank grid; the library computes the same
state on the host.  Bit-exact: the background integration, the RAN2 noise and
the field layer use the reference's expressions, and exp/tanh/log come from
the same host libm as the fixtures'.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN

from mhd_gb300 import abi
from mhd_gb300.case import STATE_FIELDS, Case, coordinates
from mhd_gb300.sim import static_state


def _cases():
    return json.loads((GOLDEN / "static_cases.json").read_text())


def _case(name) -> Case:
    return Case(**_cases()[name])


@pytest.mark.parametrize("name", sorted(_cases()))
def test_static_matches_reference_fixture(name):
    case = _case(name)
    ref = np.load(GOLDEN / f"{name}.npz")
    assert np.array_equal(ref["ZEE"], coordinates(case)[2])
    got = static_state(case)
    for k in STATE_FIELDS[:case.nfields]:
        a, b = ref["static_" + k], got[k]
        bad = np.argwhere(a != b)
        assert bad.size == 0, f"{name} {k}: {len(bad)} cells differ, first {bad[:3].tolist()}"


def test_static_layer_gaps_follow_the_z_ranks():
    """Static() fills the Bx layer on local planes 2..nRz+1 of every rank
    (3dmhdphsic.h:685), so plane 1 of every z rank above the lowest has none."""
    case = _case("static_kappa")  # nPEz = 4, nRz = 2
    bx = static_state(case)["BX"][:, 4, 4]
    nrz = case.nPz // case.nPEz
    for g in range(case.nz):
        gap = g < 2 or (g <= case.nPz and (g - 1) % nrz == 0)
        assert (bx[g] == 0.0) == gap, (g, bx.tolist())
    # another z split moves the gaps; the noise is drawn in global plane,
    # row, column order on every rank grid (ranks own consecutive planes/rows)
    mine = static_state(case)
    assert not np.array_equal(static_state(case, 1, 2)["BX"], mine["BX"])
    nolayer = case.replace(AMPB=0.0)
    t = static_state(nolayer, 1, 4)["TT"]
    for grid in ((1, 2), (2, 2), (4, 1), (8, 8)):
        assert np.array_equal(static_state(nolayer, *grid)["TT"], t), grid
    base = case.replace(AMPT=0.0, AMPB=0.0)
    t1, t2 = static_state(base, 1, 4)["TT"], static_state(base, 2, 2)["TT"]
    assert np.array_equal(t1, t2)
    prof = t1[:, 3, 3]
    assert np.all(np.diff(prof[1:-1]) > 0)  # temperature rises with depth
    assert np.all(t1 == prof[:, None, None])  # horizontally uniform without noise


def test_static_shr_noise_goes_into_rv():
    case = _case("static_shr")
    s = static_state(case)
    assert np.all(s["TT"] == 1.0) and np.all(s["RO"] == 1.0)
    rv = s["RV"][1:-1, 1:-1, 1:-1]
    assert np.abs(rv).max() <= 0.5 * case.AMPT and rv.std() > 0.0
    for k in ("BX", "BY", "BZ", "RU", "RW"):
        assert not s[k].any()
    # periodic x / y ghosts
    assert np.array_equal(s["RV"][:, 0, :], s["RV"][:, -2, :])
    assert np.array_equal(s["RV"][:, :, -1], s["RV"][:, :, 1])


def test_static_rejects_what_is_not_built():
    import ctypes as C
    from mhd_gb300.sim import params_for
    L = abi.load()
    case = _case("static_layer")
    out = np.empty((case.nfields,) + case.shape)
    zee = np.ascontiguousarray(coordinates(case)[2])
    sp = abi.MhdStaticParams(nPEy=2, nPEz=2, zMax=case.zMax)
    sp.ZEE = zee.ctypes.data_as(C.POINTER(C.c_double))
    dp = out.ctypes.data_as(C.POINTER(C.c_double))
    p, _keep = params_for(case.replace(lRem=True, lShr=True))  # lRem with lShr has no reference behaviour
    assert L.mhd_static_state(C.byref(p), C.byref(sp), dp) == abi.MHD_ERR_UNSUPPORTED
    p, _keep = params_for(case)
    sp.nPEz = 3  # nPz = 8 does not split over 3 z ranks
    assert L.mhd_static_state(C.byref(p), C.byref(sp), dp) == abi.MHD_ERR_INVALID
    sp.nPEz = 2
    sp.nTube = 4  # tube models give the reference no state
    assert L.mhd_static_state(C.byref(p), C.byref(sp), dp) == abi.MHD_ERR_UNSUPPORTED
    sp.nTube = 6
    assert L.mhd_static_state(C.byref(p), C.byref(sp), dp) == abi.MHD_ERR_INVALID
    sp.nTube = 0
    sp.ZEE = None
    assert L.mhd_static_state(C.byref(p), C.byref(sp), dp) == abi.MHD_ERR_INVALID


def test_reference_tube_model_aborts():
    """tube() with nTube = 1 (a twisted Gaussian tube) integrates its pressure
    balance with qromb, whose polint divides by ho - hp = 0 on its first pass
    (3dmhdphsic.h:199-208), so the reference aborts: there is no state to match."""
    refcase = pytest.importorskip("refcase")
    if not refcase.reference_available():
        pytest.skip("reference sources not present")
    case = _case("static_layer").replace(AMPB=0.0, AMPT=0.0, nTube=1, XCENT=3.0, ZCENT=1.0, R_MAX=0.5,
                                         C_MT=0.1, A_TUBE=0.3, name="static_tube1")
    with pytest.raises(RuntimeError, match="Failure in polint"):
        refcase.run(case, {k: np.zeros(case.shape) for k in STATE_FIELDS}, "static", 0, timeout=300)


def test_static_live_reference_other_rank_grid():
    """The compiled reference on a rank grid no fixture uses (1 x 4 ranks for
    the 2 x 2 case: other layer gaps), where the reference sources are present."""
    refcase = pytest.importorskip("refcase")
    if not refcase.reference_available():
        pytest.skip("reference sources not present")
    case = _case("static_layer").replace(nPEy=1, nPEz=4, name="static_layer_1x4")
    r = refcase.run(case, {k: np.zeros(case.shape) for k in STATE_FIELDS}, "static", 0)
    got = static_state(case)
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(r[k], got[k]), k


def test_static_lrem_profile_matches_reference_fixture():
    """lRem's background (getbackground: RK4 steps under step doubling from
    depth 2, 3dmhdphsic.h:357-522) also gives RKAPA / DKAPA of every plane
    and the wall values TU, DZTU, DZTB (3dmhdphsic.h:565-594): bit-identical
    with the compiled reference."""
    from mhd_gb300.sim import static_lrem_profile
    case = _case("static_lrem")
    ref = np.load(GOLDEN / "static_lrem.npz")
    got = static_lrem_profile(case)
    assert np.array_equal(got["RKAPA"], ref["static_RKAPA"])
    assert np.array_equal(got["DKAPA"], ref["static_DKAPA"])
    assert [got["TU"], got["DZTU"], got["DZTB"]] == ref["static_walls"].tolist()
    assert np.all(np.diff(got["RKAPA"][1:-1]) != 0.0)


def test_static_lrem_aborts_where_the_reference_does():
    """With zMax = 2 the last level lies at depth 2, where the integration
    starts: the reference's first step is clipped to zero and it aborts
    ("Stepsize not significant in RKQC", 3dmhdphsic.h:480-483); the library
    returns MHD_ERR_NUMERIC for the state and the profile."""
    import ctypes as C
    from mhd_gb300.sim import params_for
    case = _case("static_lrem").replace(zMax=2.0, name="static_lrem_z2")
    L = abi.load()
    p, _keep = params_for(case)
    sp = abi.MhdStaticParams(nPEy=2, nPEz=2, zMax=2.0)
    zee = np.ascontiguousarray(coordinates(case)[2])
    sp.ZEE = zee.ctypes.data_as(C.POINTER(C.c_double))
    out = np.empty((case.nfields,) + case.shape)
    assert L.mhd_static_state(C.byref(p), C.byref(sp), out.ctypes.data_as(C.POINTER(C.c_double))) == \
        abi.MHD_ERR_NUMERIC
    rk, drk, walls = np.empty(case.nz), np.empty(case.nz), np.empty(3)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    assert L.mhd_static_lrem_profile(C.byref(p), C.byref(sp), dp(rk), dp(drk), dp(walls)) == abi.MHD_ERR_NUMERIC
    refcase = pytest.importorskip("refcase")
    if not refcase.reference_available():
        return
    with pytest.raises(RuntimeError, match="Stepsize not significant in RKQC"):
        refcase.run(case, {k: np.zeros(case.shape) for k in STATE_FIELDS}, "static", 0, timeout=300)
