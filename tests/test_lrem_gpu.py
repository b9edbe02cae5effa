"""lRem, the Rempel relaxation (3dmhdparam.h:14): conduction of T minus its
horizontal mean plus the mean profile's HRAD (3dmhdsub.h:297-313), the RO
wall-ghost copy (3dmhdsub.h:229-238), TU / DZTU / DZTB wall temperatures
(3dmhdsub.h:783-802,852-854) and the CFL conduction limit with 1 + RKAPA
(3dmhdsub.h:79-83).  Fixtures come from the reference on one y rank."""
import numpy as np
import pytest

from conftest import load_golden, lrem_case_names
from gpu_util import rel_err, sim_from_fixture
from mhd_gb300 import abi
from mhd_gb300.case import FLUX_FIELDS, STATE_FIELDS
from mhd_gb300.sim import Batch, Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", lrem_case_names())
def test_parity_fluxes_steps_cfl_bit_exact(name):
    case, g = load_golden(name)
    sim = sim_from_fixture(case, g, "parity")
    sim.fluxes()
    for k in (FLUX_FIELDS if case.lMag else FLUX_FIELDS[:5]):
        assert np.array_equal(sim.download(k)[1:-1, 1:-1, 1:-1], g["flux_" + k]), k
    sim.close()
    sim = sim_from_fixture(case, g, "parity")
    for _ in range(3):
        sim.step(case.dt)
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(sim.download(k), g["steps3_" + k]), k
    sim.close()
    sim = sim_from_fixture(case, g, "parity")
    dts = [sim.step(0.0)["dt"] for _ in range(2)]
    assert np.array_equal(np.array(dts), g["cfl2_dt"])
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(sim.download(k), g["cfl2_" + k]), k
    sim.close()


@pytest.mark.parametrize("name", lrem_case_names())
def test_fused_within_tolerance(name):
    case, g = load_golden(name)
    sim = sim_from_fixture(case, g, "fused")
    for _ in range(3):
        sim.step(case.dt)
    got = sim.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert rel_err(got[k], g["steps3_" + k]) <= 3e-12, k
    sim.close()
    sim = sim_from_fixture(case, g, "fused")
    _, d = sim.steps_cfl(1)
    assert d["dt"] == g["cfl2_dt"][0]
    sim.close()


def test_lrem_batches_rejected():
    case, g = load_golden("lrem_fixedT")
    sim = sim_from_fixture(case, g, "fused")
    with pytest.raises(abi.MhdError):
        Batch([sim])
    sim.close()
