"""FP32-storage form: fields stored and stenciled in FP32 (RO and TT as
deviations from FP64 reference profiles); the equation of state, the
profiles' hydrostatic residual, the RK3 register and the reductions in FP64.
Checked against the oracle and the FP64 paths."""
import ctypes as C
import itertools

import numpy as np
import pytest

from gpu_util import oracle_for, rel_err
from mhd_gb300.case import STATE_FIELDS, config0, initial_state, small_cases
from mhd_gb300 import abi
from mhd_gb300.sim import Simulation

pytestmark = pytest.mark.gpu


def l2_rel(a, b):
    a, b = a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1]
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / n if n > 0 else np.linalg.norm(a - b)


def test_upload_download_round_trip():
    case = small_cases()["mhd_fixedT"]
    st = initial_state(case)
    sim = Simulation(case, precision="fp32")
    sim.upload_state(st)
    got = sim.download_state()
    for k in STATE_FIELDS:
        scale = max(np.abs(st[k]).max(), 1e-300)
        assert np.abs(got[k] - st[k]).max() / scale <= 2e-7, k
    sim.close()


@pytest.mark.parametrize("name", sorted(small_cases()))
def test_one_step_close_to_fp64(name):
    case = small_cases()[name]
    st = initial_state(case)
    sim = Simulation(case, precision="fp32")
    sim.upload_state(st)
    sim.communicate()
    sim.step(case.dt)
    got = sim.download_state()
    sim.close()
    o = oracle_for(case, st)
    o.steps(1)
    for k in STATE_FIELDS[:case.nfields]:
        assert rel_err(got[k], o.arr[k]) <= 1e-5, (k, rel_err(got[k], o.arr[k]))


@pytest.mark.parametrize("mag,rot,shr", list(itertools.product([True, False], [True, False], [True, False])))
def test_one_step_all_switch_sets_fp32(mag, rot, shr):
    """Every lMag / lRot / lShr combination with FP32 storage, one step
    against the oracle: 1e-5 of each field's max-norm."""
    case = small_cases()["mhd_fixedT"].replace(lMag=mag, lRot=rot, lShr=shr, ANG=0.3, nPx=20, nPy=12, nPz=10)
    st = initial_state(case)
    sim = Simulation(case, precision="fp32")
    sim.upload_state(st)
    sim.communicate()
    sim.step(case.dt)
    got = sim.download_state()
    sim.close()
    o = oracle_for(case, st)
    o.steps(1)
    for k in STATE_FIELDS[:case.nfields]:
        assert rel_err(got[k], o.arr[k]) <= 1e-5, (k, rel_err(got[k], o.arr[k]))


def test_headline_physics_100_steps_l2_error(capsys):
    """lMag + lRot (0.1 about z) + lShr at 64x64x32, 100 steps: FP32 storage
    (with lShr's persistent FP64 temperature right-hand side) against the FP64
    fused path, every field within 1e-5 relative L2."""
    from mhd_gb300.case import config1
    case = config1().replace(nPx=64, nPy=64, nPz=32, noise=1e-2, name="config1_physics_64x64x32")
    st = initial_state(case)
    res = {}
    for prec in ("fp64", "fp32"):
        sim = Simulation(case, precision=prec)
        sim.upload_state(st)
        sim.communicate()
        sim.steps(100, case.dt)
        res[prec] = sim.download_state()
        sim.close()
    errs = {k: l2_rel(res["fp32"][k], res["fp64"][k]) for k in STATE_FIELDS}
    with capsys.disabled():
        print("\nFP32-storage vs FP64, lMag+lRot+lShr 64x64x32, 100 steps, relative L2:",
              {k: f"{v:.2e}" for k, v in errs.items()})
    for k, v in errs.items():
        assert v <= 1e-5, (k, v)


def test_ghost_images_exact_in_fp32():
    case = small_cases()["mhd_rot_shr"].replace(nPx=40, nPy=9)
    sim = Simulation(case, precision="fp32")
    sim.upload_state(initial_state(case))
    sim.communicate()
    sim.steps(2, case.dt)
    for k in STATE_FIELDS:
        a = sim.download(k)[1:-1]
        assert np.array_equal(a[:, 0, :], a[:, -2, :]) and np.array_equal(a[:, -1, :], a[:, 1, :]), k
        assert np.array_equal(a[:, :, 0], a[:, :, -2]) and np.array_equal(a[:, :, -1], a[:, :, 1]), k
    sim.close()


def test_config0_200_steps_l2_error(capsys):
    """64x64x32 MHD, 200 steps: FP32 storage vs the FP64 fused path."""
    case = config0().replace(noise=1e-2)
    st = initial_state(case)
    res = {}
    for prec in ("fp64", "fp32"):
        sim = Simulation(case, precision=prec)
        sim.upload_state(st)
        sim.communicate()
        sim.steps(200, case.dt)
        res[prec] = (sim.download_state(), sim.diagnostics())
        sim.close()
    errs = {k: l2_rel(res["fp32"][0][k], res["fp64"][0][k]) for k in STATE_FIELDS}
    with capsys.disabled():
        print("\nFP32-storage vs FP64, 64x64x32, 200 steps, relative L2:", {k: f"{v:.2e}" for k, v in errs.items()})
        print("mass", res["fp64"][1]["total_mass"], res["fp32"][1]["total_mass"])
    for k, v in errs.items():
        assert v <= 1e-5, (k, v)
    assert abs(res["fp32"][1]["total_mass"] / res["fp64"][1]["total_mass"] - 1) < 1e-8


def test_config3_1000_steps_l2_error(capsys):
    """The precision configuration at its stated size: 256x256x128 MHD, noise
    1e-2, 1000 steps with FP32 storage against the FP64 fused path (itself
    within 1e-12 of the oracle per step); every field within 1e-5 relative
    L2, and the total mass of both within 1e-8."""
    from mhd_gb300.case import config3
    case = config3()
    st = initial_state(case)
    res = {}
    for prec in ("fp64", "fp32"):
        sim = Simulation(case, precision=prec)
        sim.upload_state(st)
        sim.communicate()
        sim.steps(1000, case.dt)
        res[prec] = (sim.download_state(), sim.diagnostics())
        sim.close()
    errs = {k: l2_rel(res["fp32"][0][k], res["fp64"][0][k]) for k in STATE_FIELDS}
    with capsys.disabled():
        print("\nFP32-storage vs FP64, 256x256x128, 1000 steps, relative L2:", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, v in errs.items():
        assert v <= 1e-5, (k, v)
    assert abs(res["fp32"][1]["total_mass"] / res["fp64"][1]["total_mass"] - 1) < 1e-8


def test_cfl_and_diagnostics_fp32():
    case = small_cases()["mhd_fixedT"]
    st = initial_state(case)
    sims = {p: Simulation(case, precision=p) for p in ("fp64", "fp32")}
    out = {}
    for p, sim in sims.items():
        sim.upload_state(st)
        sim.communicate()
        out[p] = (sim.cfl_dt(), sim.diagnostics())
        sim.close()
    assert abs(out["fp32"][0][0] / out["fp64"][0][0] - 1) < 1e-6
    for k in ("total_mass", "total_energy"):
        assert abs(out["fp32"][1][k] / out["fp64"][1][k] - 1) < 1e-7, k
    assert out["fp32"][1]["flags"] == 0


def test_unfused_calls_rejected_for_fp32():
    from mhd_gb300.abi import MhdError
    case = small_cases()["mhd_fixedT"]
    sim = Simulation(case, precision="fp32")
    with pytest.raises(MhdError):
        sim.fluxes()
    sim.close()


def test_integer_pipe_conversions_match_hardware():
    """The FP32-storage kernels widen and narrow with integer operations
    (mhd_convert.cuh) to keep conversions off the FP64 pipe; on 2^24 test
    patterns (random bits, rounding ties, the float range edges, subnormals)
    they equal cvt.f64.f32 and cvt.rn.f32.f64 bit for bit."""
    L = abi.load()
    n = C.c_longlong(-1)
    abi.check(L.mhd_selftest_convert(1 << 24, 20261203, C.byref(n)))
    assert n.value == 0


def test_device_initial_state_fp32():
    """FP32-storage contexts generate their initial state on the device too:
    the FP64 state in the RK register, plane-mean profiles, FP32 deviations;
    it matches the host mirror of the generator to the FP32 rounding."""
    from mhd_gb300.case import device_initial_state
    case = small_cases()["mhd_rot_shr"].replace(nPx=24, nPy=10, nPz=8, seed=4321)
    sim = Simulation(case, precision="fp32")
    sim.init_on_device()
    got = sim.download_state()
    want = device_initial_state(case)
    for k in STATE_FIELDS:
        scale = max(np.abs(want[k]).max(), 1e-300)
        assert np.abs(got[k] - want[k]).max() / scale <= 1e-6, k
    sim.communicate()
    sim.step(case.dt)
    assert sim.diagnostics()["nit"] == 1
    sim.close()
