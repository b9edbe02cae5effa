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


@pytest.mark.parametrize("name", lrem_case_names())
def test_fp32_storage_within_precision_tolerance(name):
    """lRem with FP32 field storage (FP64 plane means, RK register and
    equation of state): 3 steps against the reference's fixture within the
    precision form's 1e-5 (relative L2 and max-norm), and its first CFL dt
    within 1e-6 of the reference's."""
    from gpu_util import METRIC_NAMES
    case, g = load_golden(name)
    mo = {n: g["in_" + n] for n in METRIC_NAMES}

    def fresh():
        s = Simulation(case, path="fused", precision="fp32", metric_override=mo)
        s.upload_state({k: g["in_" + k] for k in STATE_FIELDS})
        s.communicate()
        return s
    sim = fresh()
    for _ in range(3):
        sim.step(case.dt)
    got = sim.download_state()
    sim.close()
    for k in STATE_FIELDS[:case.nfields]:
        a, b = got[k][1:-1, 1:-1, 1:-1], g["steps3_" + k][1:-1, 1:-1, 1:-1]
        nb = np.linalg.norm(b)
        l2 = np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)
        assert l2 <= 1e-5 and rel_err(got[k], g["steps3_" + k]) <= 1e-5, (k, l2)
    sim = fresh()
    _, d = sim.steps_cfl(1)
    assert abs(d["dt"] / g["cfl2_dt"][0] - 1.0) <= 1e-6
    sim.close()
