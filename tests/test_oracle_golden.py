"""The CPU oracle (oracle/mhd_oracle.c) against fixtures produced by the
reference 3dmhd code itself (tests/golden/make_golden.py): bit-exact."""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN, golden_case_names, load_golden, lrem_case_names, plume_case_names
from mhd_gb300.case import FLUX_FIELDS, STATE_FIELDS, config0, initial_state

import oracle

METRIC_NAMES = ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")


def oracle_from_fixture(case, g):
    sim = oracle.OracleSim(case)
    # replay the fixture's own metric arrays and input state
    for n, a in zip(METRIC_NAMES, sim._metric_arrays):
        a[...] = g["in_" + n]
    sim.load({k: g["in_" + k] for k in STATE_FIELDS})
    sim.communicate()
    return sim


@pytest.mark.parametrize("name", golden_case_names() + plume_case_names() + lrem_case_names())
def test_fluxes_bit_exact(name):
    case, g = load_golden(name)
    sim = oracle_from_fixture(case, g)
    sim.fluxes()
    names = FLUX_FIELDS if case.lMag else FLUX_FIELDS[:5]
    for k in names:
        got = sim.arr[k][1:-1, 1:-1, 1:-1]
        assert np.array_equal(got, g["flux_" + k]), k


@pytest.mark.parametrize("name", golden_case_names() + plume_case_names() + lrem_case_names())
def test_three_steps_bit_exact(name):
    case, g = load_golden(name)
    sim = oracle_from_fixture(case, g)
    sim.steps(3)
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(sim.arr[k], g["steps3_" + k]), k


@pytest.mark.parametrize("name", ["mhd_fixedT", "hydro_default_bc", "lrem_fixedT", "lrem_flux"])
def test_cfl_steps_bit_exact(name):
    case, g = load_golden(name)
    sim = oracle_from_fixture(case, g)
    dts = sim.steps(2, dt=0.0)
    assert np.array_equal(dts, g["cfl2_dt"])
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(sim.arr[k], g["cfl2_" + k]), k


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def test_config0_100_steps_digest():
    """64x64x32 MHD, 100 fixed-dt steps: the oracle's final state hashes to
    the reference's (4 ranks)."""
    d = json.loads((GOLDEN / "config0_digest.json").read_text())
    case = config0()
    st = initial_state(case)
    if any(_sha(st[k]) != d["input_sha256"][k] for k in STATE_FIELDS):
        pytest.skip("this host's libm generates a different seeded input; digest not comparable")
    sim = oracle.OracleSim(case, st, nthreads=8)
    sim.communicate()
    sim.steps(d["steps"])
    for k in STATE_FIELDS:
        assert _sha(sim.arr[k]) == d["output_sha256"][k], k


def test_unsupported_wall_condition_is_rejected():
    case, g = load_golden("mhd_fixedT")
    sim = oracle_from_fixture(case.replace(iTCon=3), g)
    with pytest.raises(ValueError):
        sim.BCON()


@pytest.mark.parametrize("name", ["mhd_fixedT", "hydro_default_bc"])
def test_dat0_writer_matches_reference_dump(name, tmp_path):
    """mhd_write_dat0 (host code of the library) writes the same bytes as the
    reference's dumpData for the same state (3 steps of the golden case, 2x2 ranks)."""
    import ctypes as C
    from mhd_gb300 import abi
    import sys
    sys.path.insert(0, str(GOLDEN.parent.parent / "rast-3dmhd-cpp_gb300"))
    import build as mhd_build
    mhd_build.build()
    L = abi.load()
    case, g = load_golden(name)
    nf = case.nfields
    state = np.ascontiguousarray(np.stack([g["steps3_" + k] for k in STATE_FIELDS[:nf]]))
    prefix = str(tmp_path / "mine")
    rc = L.mhd_write_dat0(prefix.encode(), case.nPx, case.nPy, case.nPz, nf,
                          state.ctypes.data_as(C.POINTER(C.c_double)), case.nPEy, case.nPEz, 0)
    assert rc == 0
    for rank in range(case.nPEy * case.nPEz):
        ref = (GOLDEN / f"dat0_{name}" / f"test.dat0.{rank:04d}").read_bytes()
        mine = (tmp_path / f"mine.dat0.{rank:04d}").read_bytes()
        assert mine == ref, rank
    # read it back (a later record keeps the first one)
    rc = L.mhd_write_dat0(prefix.encode(), case.nPx, case.nPy, case.nPz, nf,
                          state.ctypes.data_as(C.POINTER(C.c_double)), case.nPEy, case.nPEz, 1)
    back = np.zeros_like(state)
    assert L.mhd_read_dat0(prefix.encode(), case.nPx, case.nPy, case.nPz, nf,
                           back.ctypes.data_as(C.POINTER(C.c_double)), case.nPEy, case.nPEz, 0) == 0
    I = np.s_[:, 1:-1, 1:-1, 1:-1]
    assert np.array_equal(back[I], state[I])


def test_config1_physics_64x64x32_20_steps_digest():
    """lMag + lRot (0.1 about z) + lShr at 64x64x32: the oracle's state after
    20 steps hashes to the reference's (4 ranks)."""
    from mhd_gb300.case import config1
    d = json.loads((GOLDEN / "config1_64x64x32_digest.json").read_text())
    case = config1().replace(nPx=64, nPy=64, nPz=32, nPEy=2, nPEz=2, name="config1_physics_64x64x32")
    st = initial_state(case)
    if any(_sha(st[k]) != d["input_sha256"][k] for k in STATE_FIELDS):
        pytest.skip("this host's libm generates a different seeded input; digest not comparable")
    sim = oracle.OracleSim(case, st, nthreads=8)
    sim.communicate()
    sim.steps(d["steps"])
    for k in STATE_FIELDS:
        assert _sha(sim.arr[k]) == d["output_sha256"][k], k


def test_threaded_cfl_reduction_equals_the_serial_one():
    """The plane-parallel CFL reduction used by the CPU baseline's adaptive-dt
    leg gives the serial (reference-order) DT and UMACH bit for bit on a
    finite state."""
    import oracle
    from mhd_gb300.case import initial_state, small_cases
    case = small_cases()["mhd_fixedT"]
    st = initial_state(case)
    o = oracle.OracleSim(case, st, nthreads=4)
    o.communicate()
    o.steps(2)
    serial = o.cfl_dt()
    o.p.cfl_parallel = 1
    threaded = o.cfl_dt()
    o.p.cfl_parallel = 0
    assert serial == threaded
