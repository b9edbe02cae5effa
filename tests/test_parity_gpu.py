"""The unfused GPU path (-fmad=false kernels) against the reference's own
outputs (golden fixtures) and the oracle: bit-exact."""
import numpy as np
import pytest

from conftest import golden_case_names, load_golden
from gpu_util import oracle_for, sim_from_fixture
from mhd_gb300.case import FLUX_FIELDS, STATE_FIELDS, config0, initial_state
from mhd_gb300.sim import Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_case_names())
def test_fluxes_bit_exact_vs_reference(name):
    case, g = load_golden(name)
    sim = sim_from_fixture(case, g, "parity")
    sim.fluxes()
    for k in (FLUX_FIELDS if case.lMag else FLUX_FIELDS[:5]):
        got = sim.download(k)[1:-1, 1:-1, 1:-1]
        assert np.array_equal(got, g["flux_" + k]), (k, np.abs(got - g["flux_" + k]).max())
    sim.close()


@pytest.mark.parametrize("name", golden_case_names())
def test_three_steps_bit_exact_vs_reference(name):
    case, g = load_golden(name)
    sim = sim_from_fixture(case, g, "parity")
    for _ in range(3):
        sim.step(case.dt)
    for k in STATE_FIELDS[:case.nfields]:
        got = sim.download(k)
        assert np.array_equal(got, g["steps3_" + k]), (k, np.abs(got - g["steps3_" + k]).max())
    sim.close()


@pytest.mark.parametrize("name", ["mhd_fixedT", "hydro_default_bc"])
def test_cfl_steps_bit_exact_vs_reference(name):
    case, g = load_golden(name)
    sim = sim_from_fixture(case, g, "parity")
    dts = [sim.step(0.0)["dt"] for _ in range(2)]
    assert np.array_equal(np.array(dts), g["cfl2_dt"])
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(sim.download(k), g["cfl2_" + k]), k
    sim.close()


def test_unfused_abi_sequence_matches_oracle_calls():
    """One substage driven call by call (ZETA0, fluxes, GAM, BCON, communicate)."""
    case, g = load_golden("mhd_rot_shr")
    sim = sim_from_fixture(case, g, "parity")
    st = {k: g["in_" + k] for k in STATE_FIELDS}
    o = oracle_for(case, st)
    for m in (sim, o):
        m.step_block_ZETA0()
        m.fluxes()
        m.step_block_GAM(0.5 * case.dt)
        m.BCON(0.0)
        m.communicate()
    for k in STATE_FIELDS:
        assert np.array_equal(sim.download(k), o.arr[k]), k
    sim.close()


def test_config0_parity_100_steps_bit_exact():
    """64x64x32 MHD, 100 fixed-dt steps through the unfused GPU path equal
    the oracle bit for bit (the oracle equals the reference, see the CPU tests)."""
    case = config0()
    st = initial_state(case)
    sim = Simulation(case, path="parity")
    sim.upload_state(st)
    sim.communicate()
    sim.steps(100, case.dt)
    o = oracle_for(case, st, nthreads=16)
    o.steps(100)
    for k in STATE_FIELDS:
        assert np.array_equal(sim.download(k), o.arr[k]), k
    sim.close()


def test_config1_physics_parity_20_steps_bit_exact():
    """The benchmark's physics (lMag, lRot 0.1 about z, lShr) at 64x64x32:
    20 steps through the unfused GPU path equal the oracle (whose digest
    equals the reference's) bit for bit."""
    from mhd_gb300.case import config1
    case = config1().replace(nPx=64, nPy=64, nPz=32, nPEy=2, nPEz=2)
    st = initial_state(case)
    sim = Simulation(case, path="parity")
    sim.upload_state(st)
    sim.communicate()
    sim.steps(20, case.dt)
    o = oracle_for(case, st, nthreads=16)
    o.steps(20)
    for k in STATE_FIELDS:
        assert np.array_equal(sim.download(k), o.arr[k]), k
    sim.close()
