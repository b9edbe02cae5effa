"""mhd_step_host: one fused step from a host state to a host state, the
interior cut into z slabs whose upload, substages and download overlap on
three streams.  The result must equal upload + mhd_step + download bit for
bit (the same per-cell arithmetic), for pinned and pageable buffers, aliased
or separate, with the persistent FT of lShr carried across steps."""
import ctypes as C

import numpy as np
import pytest

from mhd_gb300 import abi
from mhd_gb300.case import STATE_FIELDS, Case, initial_state
from mhd_gb300.sim import Simulation

pytestmark = pytest.mark.gpu


def _flat(case, st):
    return np.ascontiguousarray(np.stack([st[k] for k in STATE_FIELDS[:case.nfields]]), dtype=np.float64)


class Pinned:
    def __init__(self, n):
        self.L = abi.load()
        self.p = C.c_void_p()
        abi.check(self.L.mhd_host_alloc(n * 8, C.byref(self.p)))
        self.a = np.ctypeslib.as_array(C.cast(self.p, C.POINTER(C.c_double)), shape=(n,))

    def free(self):
        self.L.mhd_host_free(self.p)


def _reference_steps(case, st, n):
    sim = Simulation(case)
    sim.upload_state(st)
    sim.communicate()
    for _ in range(n):
        sim.step(case.dt)
    out = _flat(case, sim.download_state())
    sim.close()
    return out


# nPy = 48: the isotropic instantiation (equal x and y spacings), 40: the uniform one
@pytest.mark.parametrize("mag,shr,npz,npy", [(True, True, 100, 40), (True, False, 96, 40), (False, True, 130, 40),
                                             (True, True, 40, 40), (True, True, 100, 48)])
@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_equals_device_step(mag, shr, npz, npy, pinned):
    case = Case(nPx=48, nPy=npy, nPz=npz, lMag=mag, lRot=True, lShr=shr, seed=21, name="pipe")
    st = initial_state(case)
    # ghosts as communicate() leaves them, so both paths start from the same arrays
    s0 = Simulation(case)
    s0.upload_state(st)
    s0.communicate()
    st = s0.download_state()
    s0.close()
    want = _reference_steps(case, st, 3)

    flat = _flat(case, st)
    sim = Simulation(case)
    if pinned:
        buf = Pinned(flat.size)
        buf.a[:] = flat.ravel()
        arr = buf.a
    else:
        arr = flat.ravel().copy()
    for _ in range(3):                        # aliased in/out, FT kept on the device
        sim.step_host(arr, arr)
    got = arr.reshape(flat.shape).copy()
    assert sim.diagnostics()["nit"] == 3
    sim.close()
    if pinned:
        buf.free()
    for f, k in enumerate(STATE_FIELDS[:case.nfields]):
        assert np.array_equal(got[f], want[f]), k


def test_step_host_separate_buffers_and_device_input():
    case = Case(nPx=40, nPy=32, nPz=128, lMag=True, seed=22, name="pipe2")
    st = initial_state(case)
    s0 = Simulation(case)
    s0.upload_state(st)
    s0.communicate()
    st = s0.download_state()
    s0.close()
    want2 = _reference_steps(case, st, 2)
    flat = _flat(case, st).ravel()
    out = np.empty_like(flat)
    sim = Simulation(case)
    sim.step_host(flat, out)                  # host -> host
    assert np.array_equal(flat, _flat(case, st).ravel())   # the input is left alone
    sim.step_host(None, out)                  # device state -> host
    sim.close()
    assert np.array_equal(out.reshape(want2.shape), want2)


# nPz = 40: too thin to pipeline, the steps run as upload + step + download one after another
@pytest.mark.parametrize("mag,shr,npz,npy", [(True, True, 100, 48), (True, False, 130, 40), (False, True, 96, 40),
                                             (True, True, 40, 40)])
def test_steps_host_chained_equals_device_steps(mag, shr, npz, npy):
    """mhd_steps_host: n host-to-host steps enqueued back to back (each step's
    upload of slab j waits only for the previous step's download of slab j+1)
    give the device steps bit for bit; the input buffer is left alone."""
    case = Case(nPx=48, nPy=npy, nPz=npz, lMag=mag, lRot=True, lShr=shr, seed=23, name="chain")
    st = initial_state(case)
    s0 = Simulation(case)
    s0.upload_state(st)
    s0.communicate()
    st = s0.download_state()
    s0.close()
    want = _reference_steps(case, st, 4)
    flat = _flat(case, st)
    src = flat.ravel().copy()
    buf = Pinned(flat.size)
    sim = Simulation(case)
    sim.steps_host(4, src, buf.a)             # separate in / out, pinned out
    got = buf.a.reshape(flat.shape).copy()
    assert np.array_equal(src, flat.ravel())
    assert sim.diagnostics()["nit"] == 4
    # aliased in / out on pageable memory, continuing from the pinned result
    arr = got.ravel().copy()
    sim.steps_host(2, arr, arr)
    sim.close()
    buf.free()
    for f, k in enumerate(STATE_FIELDS[:case.nfields]):
        assert np.array_equal(got[f], want[f]), k
    want6 = _reference_steps(case, st, 6)
    assert np.array_equal(arr.reshape(flat.shape), want6)


def test_steps_host_without_downloads_then_device_state():
    """out = NULL: step 0 uploads, later steps start from the device state
    (each substage 1 of slab j waits for the previous substage 3 of slab j+1)."""
    case = Case(nPx=40, nPy=40, nPz=128, lMag=True, lShr=True, seed=24, name="chain2")
    st = initial_state(case)
    s0 = Simulation(case)
    s0.upload_state(st)
    s0.communicate()
    st = s0.download_state()
    s0.close()
    want = _reference_steps(case, st, 3)
    sim = Simulation(case)
    sim.steps_host(3, _flat(case, st).ravel(), None)
    sim.sync()
    got = _flat(case, sim.download_state())
    sim.close()
    assert np.array_equal(got, want)
