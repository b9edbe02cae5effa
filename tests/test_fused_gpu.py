"""The fused FP64 path (one pass per RK3 substage, FMA on) against the
oracle.  Tolerance: 1e-12 of each field's max-norm after one step; the
drift after N steps is bounded and printed."""
import itertools

import numpy as np
import pytest

from conftest import load_golden
from gpu_util import oracle_for, rel_err, sim_from_fixture
from mhd_gb300.case import Case, STATE_FIELDS, config0, initial_state, small_cases
from mhd_gb300.sim import Simulation

pytestmark = pytest.mark.gpu
TOL_ONE_STEP = 1e-12


def run_pair(case, nsteps, st=None):
    st = initial_state(case) if st is None else st
    sim = Simulation(case, path="fused")
    sim.upload_state(st)
    sim.communicate()
    for _ in range(nsteps):
        sim.step(case.dt)
    o = oracle_for(case, st)
    o.steps(nsteps)
    got = sim.download_state()
    sim.close()
    return got, o


SWITCHES = list(itertools.product([True, False], [True, False], [True, False]))


@pytest.mark.parametrize("mag,rot,shr", SWITCHES)
def test_one_step_all_switch_sets(mag, rot, shr):
    base = small_cases()["mhd_fixedT"]
    case = base.replace(lMag=mag, lRot=rot, lShr=shr, ANG=0.3, nPx=20, nPy=12, nPz=10)
    got, o = run_pair(case, 1)
    for k in STATE_FIELDS[:case.nfields]:
        e = rel_err(got[k], o.arr[k])
        assert e <= TOL_ONE_STEP, (k, e)


@pytest.mark.parametrize("mag,rot,shr", SWITCHES)
def test_one_step_isotropic_xy(mag, rot, shr):
    """Equal x and y spacings (nPx = nPy, xMax = yMax; the cases above have
    nPx != nPy) run the isotropic instantiation, in which the x and y parts
    of the advection and induction terms share one metric product."""
    base = small_cases()["mhd_fixedT"]
    case = base.replace(lMag=mag, lRot=rot, lShr=shr, ANG=0.3, nPx=16, nPy=16, nPz=10)
    got, o = run_pair(case, 1)
    for k in STATE_FIELDS[:case.nfields]:
        e = rel_err(got[k], o.arr[k])
        assert e <= TOL_ONE_STEP, (k, e)


@pytest.mark.parametrize("name", sorted(small_cases()))
def test_one_step_boundary_variants(name):
    case = small_cases()[name]
    got, o = run_pair(case, 1)
    for k in STATE_FIELDS[:case.nfields]:
        assert rel_err(got[k], o.arr[k]) <= TOL_ONE_STEP, k


def test_ghost_images_bit_exact_after_fused_steps():
    case = small_cases()["mhd_rot_shr"].replace(nPx=40, nPy=9)
    sim = Simulation(case, path="fused")
    sim.upload_state(initial_state(case))
    sim.communicate()
    sim.steps(2, case.dt)
    for k in STATE_FIELDS:
        a = sim.download(k)[1:-1]
        assert np.array_equal(a[:, 0, :], a[:, -2, :]) and np.array_equal(a[:, -1, :], a[:, 1, :]), k
        assert np.array_equal(a[:, :, 0], a[:, :, -2]) and np.array_equal(a[:, :, -1], a[:, :, 1]), k
    sim.close()


@pytest.mark.parametrize("shape", [(33, 5, 4), (64, 16, 6), (7, 31, 5), (96, 48, 8)])
def test_ragged_sizes(shape):
    nx, ny, nz = shape
    case = small_cases()["mhd_rot_shr"].replace(nPx=nx, nPy=ny, nPz=nz)
    got, o = run_pair(case, 1)
    for k in STATE_FIELDS:
        assert rel_err(got[k], o.arr[k]) <= TOL_ONE_STEP, k


def test_config0_drift_100_steps(capsys):
    """Plain-method configuration 64x64x32, 100 steps: fused vs oracle."""
    case = config0()
    got, o = run_pair(case, 100)
    errs = {k: rel_err(got[k], o.arr[k]) for k in STATE_FIELDS}
    with capsys.disabled():
        print("\nconfig0 100-step fused-vs-oracle relative max error:",
              {k: f"{v:.2e}" for k, v in errs.items()})
    for k, v in errs.items():
        assert v <= 1e-9, (k, v)


def test_diagnostics_and_cfl():
    case = small_cases()["mhd_fixedT"]
    st = initial_state(case)
    sim = Simulation(case, path="fused")
    sim.upload_state(st)
    sim.communicate()
    d0 = sim.diagnostics()
    assert d0["flags"] == 0 and d0["total_mass"] > 0
    o = oracle_for(case, st)
    dt_o, um_o = o.cfl_dt()
    dt_g, um_g = sim.cfl_dt()
    assert dt_g == dt_o and um_g == um_o
    sim.close()


def test_nan_state_is_reported():
    case = small_cases()["mhd_fixedT"]
    st = initial_state(case)
    st["TT"][3, 3, 3] = np.nan
    sim = Simulation(case, path="fused")
    sim.upload_state(st)
    d = sim.diagnostics(check=False)
    assert d["flags"] & 1
    from mhd_gb300.abi import MhdError
    with pytest.raises(MhdError):
        sim.diagnostics()
    sim.close()


def test_device_initial_state_matches_host_mirror():
    from mhd_gb300.case import device_initial_state
    case = small_cases()["mhd_rot_shr"].replace(nPx=24, nPy=10, nPz=8, seed=12345)
    sim = Simulation(case, path="fused")
    sim.init_on_device()
    got = sim.download_state()
    sim.close()
    want = device_initial_state(case)
    for k in STATE_FIELDS:
        scale = max(np.abs(want[k]).max(), 1e-300)
        assert np.abs(got[k] - want[k]).max() / scale <= 1e-13, k
    # the noise is a standard normal sample
    from mhd_gb300.case import z_coordinate
    t1 = 1.0 + case.THETA * z_coordinate(case)
    g = (want["TT"][1:-1, 1:-1, 1:-1] / t1[1:-1, None, None] - 1) / case.noise
    assert abs(g.mean()) < 0.2 and 0.8 < g.std() < 1.2


def test_config1_full_size_one_step(capsys):
    """512x512x256 with lMag, lRot and lShr: one fused step against the
    oracle on every cell (the 64x64x32 sub-blocks and the rest)."""
    from mhd_gb300.case import config1
    case = config1()
    st = initial_state(case)
    sim = Simulation(case, path="fused")
    sim.upload_state(st)
    sim.communicate()
    sim.step(case.dt)
    got = sim.download_state()
    sim.close()
    o = oracle_for(case, st, nthreads=16)
    o.steps(1)
    errs = {k: rel_err(got[k], o.arr[k]) for k in STATE_FIELDS}
    # 64x64x32 sub-blocks, as the configuration asks: the worst block per field
    worst = {}
    for k in STATE_FIELDS:
        ref = o.arr[k]
        scale = np.abs(ref[1:-1]).max()
        w = 0.0
        for z0 in range(1, case.nz - 1, 32):
            for y0 in range(1, case.ny - 1, 64):
                for x0 in range(1, case.nx - 1, 64):
                    sl = np.s_[z0:z0 + 32, y0:y0 + 64, x0:x0 + 64]
                    w = max(w, np.abs(got[k][sl] - ref[sl]).max() / scale)
        worst[k] = w
    with capsys.disabled():
        print("\n512x512x256 one fused step vs oracle, worst 64x64x32 block:", {k: f"{v:.1e}" for k, v in worst.items()})
    for k in STATE_FIELDS:
        assert errs[k] <= TOL_ONE_STEP and worst[k] <= TOL_ONE_STEP, k


@pytest.mark.parametrize("mag,shr", [(True, True), (True, False), (False, True), (False, False)])
def test_stretched_xy_grid_general_path(mag, shr):
    """Caller-supplied non-uniform x/y metrics (tanh-stretched, d2xxdx2 and
    d2yydy2 nonzero) run the general instantiation of the fused substage (the
    uniform one relies on per-z tables); one step against the oracle fed the
    same metric arrays."""
    import oracle
    from gpu_util import METRIC_NAMES
    from mhd_gb300.case import tanh_metric
    case = small_cases()["mhd_rot_flux"].replace(lMag=mag, lShr=shr, nPx=24, nPy=16, nPz=12)
    dxm, dym = tanh_metric(case.nPx, case.xMax, 0.8), tanh_metric(case.nPy, case.yMax, 0.6)
    mo = {"dxxdx": dxm[0], "d2xxdx2": dxm[1], "DDX": dxm[2], "dyydy": dym[0], "d2yydy2": dym[1], "DDY": dym[2]}
    st = initial_state(case)
    sim = Simulation(case, path="fused", metric_override=mo)
    sim.upload_state(st)
    sim.communicate()
    sim.step(case.dt)
    got = sim.download_state()
    sim.close()
    o = oracle.OracleSim(case, st)
    for n, a in mo.items():
        o._metric_arrays[METRIC_NAMES.index(n)][:] = a  # the oracle reads these arrays in place
    o.communicate()
    o.steps(1)
    for k in STATE_FIELDS[:case.nfields]:
        e = rel_err(got[k], o.arr[k])
        assert e <= TOL_ONE_STEP, (k, e)
