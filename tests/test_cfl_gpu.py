"""The reference's run mode, a CFL dt for every step (step(),
3dmhdsub.h:36-106, in the loop of 3dmhd.cpp:271-331), through
mhd_steps_cfl.  On the fused FP64 path the dt is reduced into a
device-resident record that the substage kernels read, so n steps run
without a host round trip; the parity and FP32-storage paths read dt back
each step.  A dt below 1e-8 halts the run (3dmhd.cpp:292)."""
import numpy as np
import pytest

from conftest import load_golden
from gpu_util import rel_err, sim_from_fixture
from mhd_gb300 import abi
from mhd_gb300.case import STATE_FIELDS, Case, initial_state, metrics
from mhd_gb300.sim import Simulation

import oracle

pytestmark = pytest.mark.gpu
TOL_ONE_STEP = 1e-12


@pytest.mark.parametrize("name", ["mhd_fixedT", "hydro_default_bc"])
def test_parity_path_steps_cfl_bit_exact_vs_reference(name):
    case, g = load_golden(name)
    sim = sim_from_fixture(case, g, "parity")
    st, d = sim.steps_cfl(2)
    assert st == abi.MHD_OK and d["nit"] == 2
    assert d["dt"] == g["cfl2_dt"][1]
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(sim.download(k), g["cfl2_" + k]), k
    sim.close()


@pytest.mark.parametrize("name", ["mhd_fixedT", "hydro_default_bc"])
def test_fused_device_dt_vs_reference(name):
    """The first dt comes from the reference's own initial state, so it is
    bit-exact; the second is reduced over the fused state (1e-12 of the
    reference's), and the state after two steps agrees to 1e-12 per field."""
    case, g = load_golden(name)
    sim = sim_from_fixture(case, g, "fused")
    _, d1 = sim.steps_cfl(1)
    assert d1["dt"] == g["cfl2_dt"][0]
    _, d2 = sim.steps_cfl(1)
    assert abs(d2["dt"] - g["cfl2_dt"][1]) <= TOL_ONE_STEP * g["cfl2_dt"][1]
    # TIMT = TIMI + TIMC with TIMC the running sum of DT (3dmhdsub.h:150-152)
    assert d2["timt"] == 0.0 + (d1["dt"] + d2["dt"]) and d2["nit"] == 2
    for k in STATE_FIELDS[:case.nfields]:
        assert rel_err(sim.download(k), g["cfl2_" + k]) <= 2 * TOL_ONE_STEP, k
    sim.close()


@pytest.mark.parametrize("lmag,lshr", [(True, True), (False, False)])
def test_device_record_equals_host_cfl_steps(lmag, lshr):
    """20 steps with the dt kept on the device equal, bit for bit, 20 steps
    whose CFL dt went through the host (same reductions, same kernels)."""
    case = Case(nPx=40, nPy=48, nPz=24, lMag=lmag, lRot=True, lShr=lshr, seed=5, name="cfl")
    st0 = initial_state(case)
    a, b = Simulation(case), Simulation(case)
    for s in (a, b):
        s.upload_state(st0)
        s.communicate()
    _, da = a.steps_cfl(20)
    for _ in range(20):
        db = b.step(0.0)
    assert da["dt"] == db["dt"] and da["timt"] == db["timt"] and da["nit"] == db["nit"] == 20
    assert da["umach"] == db["umach"]
    ga, gb = a.download_state(), b.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(ga[k], gb[k]), k
    a.close()
    b.close()


def test_halt_leaves_state_unchanged():
    """SFF = 1e-12 makes every CFL dt fall below 1e-8: after one fixed-dt
    step the halted steps leave the state as it was, bit for bit, and report
    MHD_ERR_DT_TOO_SMALL with nit and timt of the last completed step."""
    case = Case(nPx=32, nPy=32, nPz=16, lMag=True, seed=9, SFF=1e-12, name="halt")
    sim = Simulation(case)
    sim.upload_state(initial_state(case))
    sim.communicate()
    sim.step(case.dt)
    before = sim.download_state()
    st, d = sim.steps_cfl(5, check=False)
    assert st == abi.MHD_ERR_DT_TOO_SMALL
    assert d["nit"] == 1 and d["timt"] == case.dt and 0.0 < d["dt"] < 1e-8
    after = sim.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(before[k], after[k]), k
    # the host-side CFL step halts the same way
    with pytest.raises(abi.MhdError):
        sim.step(0.0)
    # and a fixed-dt step still runs afterwards
    sim.step(case.dt)
    assert sim.diagnostics()["nit"] == 2
    sim.close()


def test_fp32_device_record_equals_host_cfl_steps():
    """FP32 storage: 12 steps with the dt kept on the device equal, bit for
    bit, 12 steps whose CFL dt went through the host; the dt is the FP64
    reduction over the widened FP32 state."""
    case = Case(nPx=40, nPy=32, nPz=24, lMag=True, lRot=True, seed=8, name="cfl32")
    st0 = initial_state(case)
    a, b = Simulation(case, precision="fp32"), Simulation(case, precision="fp32")
    for s in (a, b):
        s.upload_state(st0)
        s.communicate()
    _, da = a.steps_cfl(12)
    for _ in range(12):
        db = b.step(0.0)
    assert da["dt"] == db["dt"] and da["timt"] == db["timt"] and da["nit"] == db["nit"] == 12
    ga, gb = a.download_state(), b.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(ga[k], gb[k]), k
    a.close()
    b.close()


def test_fp32_halt_leaves_state_unchanged():
    case = Case(nPx=32, nPy=32, nPz=16, lMag=True, seed=9, SFF=1e-12, name="halt32")
    sim = Simulation(case, precision="fp32")
    sim.upload_state(initial_state(case))
    sim.communicate()
    sim.step(case.dt)
    before = sim.download_state()
    st, d = sim.steps_cfl(4, check=False)
    assert st == abi.MHD_ERR_DT_TOO_SMALL and d["nit"] == 1
    after = sim.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(before[k], after[k]), k
    sim.step(case.dt)
    sim.close()


def test_fp32_storage_steps_cfl():
    """The FP32-storage form takes the CFL dt from its FP64 reduction; its
    first dt equals the FP64 one to the FP32 storage rounding."""
    case = Case(nPx=32, nPy=32, nPz=32, lMag=True, seed=3, name="cfl32")
    st0 = initial_state(case)
    s64, s32 = Simulation(case), Simulation(case, precision="fp32")
    for s in (s64, s32):
        s.upload_state(st0)
        s.communicate()
    _, d64 = s64.steps_cfl(3)
    _, d32 = s32.steps_cfl(3)
    assert d32["nit"] == 3
    assert abs(d32["dt"] - d64["dt"]) <= 1e-5 * d64["dt"]
    s64.close()
    s32.close()


# ---- the row-filtered CFL reduction against the oracle, bit for bit ----------
def _cfl_pair(case, st, ddx=None):
    mo = {"DDX": ddx} if ddx is not None else None
    sim = Simulation(case, metric_override=mo)
    sim.upload_state(st)
    got = sim.cfl_dt()
    o = oracle.OracleSim(case, st)
    if ddx is not None:
        o._metric_arrays[2][:] = ddx      # the oracle reads DDX through this array
    want = o.cfl_dt()
    sim.close()
    return got, want


def _random_flow(case, seed, amp):
    st = initial_state(case)
    rng = np.random.default_rng(seed)
    for k in ("RU", "RV", "RW"):
        st[k] = amp * rng.standard_normal(case.shape) * st["RO"]
    if case.lMag:
        for k in ("BX", "BY", "BZ"):
            st[k] = 1e-2 * rng.standard_normal(case.shape)
    return st


@pytest.mark.parametrize("lmag", [True, False])
@pytest.mark.parametrize("kind", ["initial", "flow", "ties", "tiny_and_odd", "nan_cell"])
def test_cfl_reduction_bit_exact(lmag, kind):
    """DT and UMACH of mhd_cfl_dt equal the oracle's cell-by-cell reduction
    (the reference's loop) bit for bit: zero momenta, a random flow, a state
    where every cell ties, states with tiny, huge, negative and non-finite
    values (cells the FP32 estimate cannot certify)."""
    case = Case(nPx=70, nPy=36, nPz=20, lMag=lmag, seed=11, name="cflx")
    if kind == "initial":
        st = initial_state(case)
    elif kind == "flow":
        st = _random_flow(case, 1, 3e-2)
    elif kind == "ties":
        st = initial_state(case)
        st["TT"][...] = 2.0
        st["RO"][...] = 0.5
        st["RU"][...] = 0.01
        st["RV"][...] = -0.02
        st["RW"][...] = 0.0
    elif kind == "tiny_and_odd":
        st = _random_flow(case, 2, 1e-25)
        st["RU"][7, 9, 11] = 3e-3                  # one real flow cell
        st["RV"][5, 20, 40] = 1e30                 # beyond the float range
        st["TT"][9, 3, 3] = -0.5                   # negative temperature
        st["RO"][12, 30, 60] = 1e-30               # density far below the certified range
        st["RW"][3, 4, 5] = 1e-300                 # subnormal-range input
    else:
        st = _random_flow(case, 3, 1e-2)
        st["TT"][6, 6, 6] = np.nan
        st["RU"][8, 8, 8] = np.nan
    got, want = _cfl_pair(case, st)
    assert got[0] == want[0] or (np.isnan(got[0]) and np.isnan(want[0])), (got, want)
    assert got[1] == want[1] or (np.isnan(got[1]) and np.isnan(want[1])), (got, want)


def test_cfl_reduction_varying_dd_rows():
    """A non-uniform DDX makes DD vary along rows where it drops below
    min(DDZ, DDY): those rows take the cell-by-cell path; the result stays
    bit-exact."""
    case = Case(nPx=64, nPy=24, nPz=16, lMag=True, seed=4, name="cfldd")
    st = _random_flow(case, 4, 2e-2)
    base = float(metrics(case).DDX[1])
    x = np.arange(case.nx)
    ddx = base * (1.0 + 0.6 * np.sin(0.37 * x))
    got, want = _cfl_pair(case, st, ddx=ddx)
    assert got == want


def test_cfl_reduction_after_fused_steps():
    """The reduction over states the fused path produced (the adaptive run)."""
    case = Case(nPx=96, nPy=64, nPz=32, lMag=True, lRot=True, seed=6, noise=1e-2, name="cflrun")
    sim = Simulation(case)
    sim.upload_state(initial_state(case))
    sim.communicate()
    sim.steps_cfl(30)
    st = sim.download_state()
    got = sim.cfl_dt()
    sim.close()
    want = oracle.OracleSim(case, st).cfl_dt()
    assert got == want


@pytest.mark.parametrize("kind", ["run", "ties", "tiny_and_odd", "cancel", "guard_edge"])
def test_fp32_cfl_reduction_bit_exact(kind):
    """FP32 storage: the filtered reduction estimates from the stored floats
    (ro and T summed with the profile in FP32) and reduces the widened FP64
    state (profile + deviation) exactly; DT and UMACH equal the oracle's
    cell-by-cell reduction over the state mhd_download_state returns (the same
    FP64 values), bit for bit, for an evolved flow, a state of ties, tiny,
    subnormal-float, huge and negative values, and the fastest cells where
    density or temperature fall far below the profile (the FP32 sum cancels:
    not certified) or just inside and outside the 4:1 cancellation bound."""
    case = Case(nPx=70, nPy=36, nPz=20, lMag=True, lRot=True, seed=12, noise=1e-2, name="cfl32x")
    sim = Simulation(case, precision="fp32")
    if kind == "run":
        sim.upload_state(initial_state(case))
        sim.communicate()
        sim.steps_cfl(10)
    else:
        if kind == "ties":
            st = initial_state(case)
            st["TT"][...] = 2.0
            st["RO"][...] = 0.5
            st["RU"][...] = 0.01
            st["RV"][...] = -0.02
            st["RW"][...] = 0.0
        elif kind == "cancel":
            # momenta keep the unscaled density, so these cells are the fastest
            st = _random_flow(case, 6, 3e-2)
            st["RO"][8:11, 10:14, 20:30] *= 0.05
            st["TT"][4:6, 20:22, 50:60] *= 0.1
        elif kind == "guard_edge":
            st = _random_flow(case, 7, 3e-2)
            st["RO"][3:6, 5:9, 10:20] *= 0.26             # profile / density about 3.8: estimated
            st["RO"][14:17, 25:29, 40:50] *= 0.24         # about 4.2: evaluated exactly
            st["TT"][10:12, 15:18, 30:35] *= 0.26
            st["TT"][16:18, 2:5, 60:66] *= 0.24
        else:
            st = _random_flow(case, 5, 1e-25)
            st["RU"][7, 9, 11] = 3e-3                  # one real flow cell
            st["RV"][4, 10, 20] = 1e-41                # a subnormal float once stored
            st["BX"][5, 5, 5] = 3e-44                  # subnormal field value
            st["RV"][5, 20, 40] = 1e30                 # huge momentum
            st["TT"][9, 3, 3] = -0.5                   # negative temperature
        sim.upload_state(st)
        sim.communicate()
    state = sim.download_state()
    got = sim.cfl_dt()
    sim.close()
    want = oracle.OracleSim(case, state).cfl_dt()
    assert got[0] == want[0] or (np.isnan(got[0]) and np.isnan(want[0])), (got, want)
    assert got[1] == want[1] or (np.isnan(got[1]) and np.isnan(want[1])), (got, want)
