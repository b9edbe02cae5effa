"""The plume terms (3dmhd.cpp:413-426): the cooling spot on the top wall
(TP != 0 with iTCon 0 or 1, 3dmhdsub.h:750-778, time-dependent through TC)
and the internal heat sink of iTCon 2 (3dmhdsub.h:443-459, time-dependent
through TC and QFH).  The oracle is pinned to the reference on these cases
(tests/test_oracle_golden.py); here the GPU paths are compared with the
oracle run on the same host (the Gaussian factors come from the host's
libm on both sides)."""
import ctypes as C

import numpy as np
import pytest

from gpu_util import oracle_for, rel_err
from mhd_gb300 import abi
from mhd_gb300.case import FLUX_FIELDS, STATE_FIELDS, initial_state, plume_cases
from mhd_gb300.sim import Batch, Simulation, params_for

pytestmark = pytest.mark.gpu
NAMES = sorted(plume_cases())


def _start(case, path="fused", precision="fp64"):
    st = initial_state(case)
    sim = Simulation(case, path=path, precision=precision)
    sim.upload_state(st)
    sim.communicate()
    return sim, st


@pytest.mark.parametrize("name", NAMES)
def test_parity_path_bit_exact(name):
    case = plume_cases()[name]
    sim, st = _start(case, path="parity")
    o = oracle_for(case, st)
    sim.fluxes()
    o.fluxes()
    for k in FLUX_FIELDS[:5]:
        assert np.array_equal(sim.download(k)[1:-1, 1:-1, 1:-1], o.arr[k][1:-1, 1:-1, 1:-1]), k
    sim.close()
    sim, st = _start(case, path="parity")
    o = oracle_for(case, st)
    for _ in range(3):
        sim.step(case.dt)
    o.steps(3)
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(sim.download(k), o.arr[k]), k
    sim.close()


@pytest.mark.parametrize("name", NAMES)
def test_fused_path_within_tolerance(name):
    case = plume_cases()[name]
    sim, st = _start(case)
    o = oracle_for(case, st)
    for _ in range(3):
        sim.step(case.dt)
    o.steps(3)
    got = sim.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert rel_err(got[k], o.arr[k]) <= 3e-12, k
    sim.close()


@pytest.mark.parametrize("name", NAMES)
def test_fp32_storage_close_to_fp64(name):
    case = plume_cases()[name]
    s64, st = _start(case)
    s32, _ = _start(case, precision="fp32")
    for _ in range(3):
        s64.step(case.dt)
        s32.step(case.dt)
    a, b = s64.download_state(), s32.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert rel_err(b[k], a[k]) <= 1e-5, k
    s64.close()
    s32.close()


@pytest.mark.parametrize("name", NAMES)
def test_plume_term_acts(name):
    """The plume term changes the state (TP = 0 gives a different result)."""
    case = plume_cases()[name]
    s1, _ = _start(case)
    s0, _ = _start(case.replace(TP=0.0))
    for _ in range(2):
        s1.step(case.dt)
        s0.step(case.dt)
    assert not np.array_equal(s1.download("TT"), s0.download("TT"))
    s1.close()
    s0.close()


def test_adaptive_cfl_with_time_dependent_plume():
    """mhd_steps_cfl takes the per-step host path when the plume depends on
    TIMT; it equals steps of mhd_step(dt <= 0)."""
    case = plume_cases()["plume_top0"]
    a, _ = _start(case)
    b, _ = _start(case)
    _, da = a.steps_cfl(4)
    for _ in range(4):
        db = b.step(0.0)
    assert da["timt"] == db["timt"] and da["nit"] == 4
    ga, gb = a.download_state(), b.download_state()
    for k in STATE_FIELDS[:case.nfields]:
        assert np.array_equal(ga[k], gb[k]), k
    a.close()
    b.close()


def test_batches_need_time_independent_plume():
    dep = plume_cases()["plume_top0"]                 # TC != 0
    ind = plume_cases()["plume_top1"]                 # TC == 0
    s, _ = _start(dep)
    with pytest.raises(abi.MhdError):
        Batch([s])
    s.close()
    sims = [_start(ind.replace(seed=7 + i))[0] for i in range(2)]
    alone = [_start(ind.replace(seed=7 + i))[0] for i in range(2)]
    b = Batch(sims)
    b.set_tile(0)
    b.steps(3)
    b.sync()
    for x, y in zip(sims, alone):
        for _ in range(3):
            y.step(ind.dt)
        gx, gy = x.download_state(), y.download_state()
        for k in STATE_FIELDS[:ind.nfields]:
            assert rel_err(gx[k], gy[k]) <= 1e-12, k
    b.close()
    for x in sims + alone:
        x.close()


def test_step_without_plume_parameters_is_rejected():
    case = plume_cases()["plume_src2"]
    L = abi.load()
    p, keep = params_for(case)
    ctx = C.c_void_p()
    abi.check(L.mhd_create(C.byref(p), None, C.byref(ctx)))
    st = initial_state(case)
    flat = np.ascontiguousarray(np.stack([st[k] for k in STATE_FIELDS[:case.nfields]]))
    abi.check(L.mhd_upload_state(ctx, flat.ctypes.data_as(C.POINTER(C.c_double))))
    assert L.mhd_step(ctx, case.dt, None) == -1
    L.mhd_destroy(ctx)
