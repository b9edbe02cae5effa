"""mhd_fluxes_noalloc, the entry point for callers that cannot call
cudaMalloc (HBM reserved up front in the caller's own pool, or a loop that
must not hit cudaMalloc's implicit device synchronisation).

The test owns the device buffers (allocated here with torch, as such a
caller's pool would hand them out), calls the entry point through the C ABI
twice in a row on different states, and compares each result with the
context-based mhd_fluxes.  Both run the same -fmad=false kernels, so the
tolerance is the one the parity tests use: bit-exact.  The second call also
shows that the scratch left behind by the first call does not leak into the
next result.
"""
import ctypes as C

import numpy as np
import pytest

from mhd_gb300 import abi
from mhd_gb300.case import FLUX_FIELDS, STATE_FIELDS, initial_state, metrics, small_cases
from mhd_gb300.sim import Simulation

pytestmark = pytest.mark.gpu

METRIC_NAMES = ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")


def _reference_fluxes(case, st, ft0):
    sim = Simulation(case, path="parity")
    sim.upload_state(st)
    sim.upload("FT", ft0)
    sim.communicate()
    sim.fluxes()
    out = {k: sim.download(k) for k in FLUX_FIELDS}
    sim.close()
    return out


def _noalloc_fluxes(torch, case, st, ft0):
    L = abi.load()
    dev = torch.device("cuda:0")
    keep = []

    def d(a):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        keep.append(t)
        return t.data_ptr()

    a = abi.MhdFluxesNoallocArgs()
    a.nPx, a.nPy, a.nPz = case.nPx, case.nPy, case.nPz
    a.switches = (abi.SW_LROT if case.lRot else 0) | (abi.SW_LMAG if case.lMag else 0) | \
                 (abi.SW_LSHR if case.lShr else 0)
    a.izCon, a.iTCon, a.iBCon = case.izCon, case.iTCon, case.iBCon
    for k in ("RE", "PR", "THETA", "GRAV", "RY", "ANG", "RM", "BETA", "TP", "GAMMA", "SFF"):
        setattr(a, k, float(getattr(case, k)))
    a.TB = case.tb
    for n, arr in zip(METRIC_NAMES, metrics(case).arrays()):
        setattr(a, n, d(arr))
    for f, k in enumerate(STATE_FIELDS):
        a.state[f] = d(st[k])
    outs = []
    for f, k in enumerate(FLUX_FIELDS):
        t = torch.zeros(case.shape, dtype=torch.float64, device=dev)
        if k == "FT":
            t.copy_(torch.from_numpy(ft0))
        outs.append(t)
        a.flux[f] = t.data_ptr()
    torch.cuda.synchronize()
    st_before = {k: st[k].copy() for k in STATE_FIELDS}
    rc = L.mhd_fluxes_noalloc(C.byref(a), None)
    assert rc == abi.MHD_OK
    torch.cuda.synchronize()
    for f, k in enumerate(STATE_FIELDS):
        assert np.array_equal(keep[len(METRIC_NAMES) + f].cpu().numpy(), st_before[k]), "input modified: " + k
    return {k: outs[f].cpu().numpy() for f, k in enumerate(FLUX_FIELDS)}


@pytest.mark.parametrize("name", ["mhd_rot_shr", "hydro_default_bc"])
def test_noalloc_matches_mhd_fluxes_on_two_calls(name):
    torch = pytest.importorskip("torch")
    base = small_cases()[name].replace(nPx=20, nPy=12, nPz=10)
    names = FLUX_FIELDS if base.lMag else FLUX_FIELDS[:5]
    for call, seed in enumerate((11, 12)):
        case = base.replace(seed=seed)
        st = initial_state(case)
        ft0 = np.random.default_rng(100 + seed).standard_normal(case.shape) * 1e-3
        want = _reference_fluxes(case, st, ft0)
        got = _noalloc_fluxes(torch, case, st, ft0)
        for k in names:
            a, b = got[k][1:-1, 1:-1, 1:-1], want[k][1:-1, 1:-1, 1:-1]
            assert np.array_equal(a, b), (call, k, float(np.abs(a - b).max()))


def test_noalloc_call_takes_no_device_memory():
    """After a first call on the device (which loads the module and with it
    the scratch array), a further call leaves the device's free memory and
    torch's allocation count unchanged."""
    torch = pytest.importorskip("torch")
    case = small_cases()["mhd_rot_shr"].replace(nPx=20, nPy=12, nPz=10, seed=21)
    st = initial_state(case)
    ft0 = np.zeros(case.shape)
    _noalloc_fluxes(torch, case, st, ft0)  # the first call on this device
    L = abi.load()
    dev = torch.device("cuda:0")
    a = abi.MhdFluxesNoallocArgs()
    a.nPx, a.nPy, a.nPz = case.nPx, case.nPy, case.nPz
    a.switches = abi.SW_LROT | abi.SW_LMAG | abi.SW_LSHR
    a.izCon, a.iTCon, a.iBCon = case.izCon, case.iTCon, case.iBCon
    for k in ("RE", "PR", "THETA", "GRAV", "RY", "ANG", "RM", "BETA", "TP", "GAMMA", "SFF"):
        setattr(a, k, float(getattr(case, k)))
    a.TB = case.tb
    keep = [torch.from_numpy(np.ascontiguousarray(m, dtype=np.float64)).to(dev) for m in metrics(case).arrays()]
    for n, t in zip(METRIC_NAMES, keep):
        setattr(a, n, t.data_ptr())
    for f, k in enumerate(STATE_FIELDS):
        t = torch.from_numpy(st[k]).to(dev)
        keep.append(t)
        a.state[f] = t.data_ptr()
    for f in range(8):
        t = torch.zeros(case.shape, dtype=torch.float64, device=dev)
        keep.append(t)
        a.flux[f] = t.data_ptr()
    torch.cuda.synchronize()
    free0, used0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for _ in range(2):
        assert L.mhd_fluxes_noalloc(C.byref(a), None) == abi.MHD_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == used0


def test_noalloc_rejects_grids_beyond_its_scratch():
    L = abi.load()
    a = abi.MhdFluxesNoallocArgs()
    a.nPx, a.nPy, a.nPz = 128, 128, 32  # 130*130*34 = 574,600 cells > MHD_NOALLOC_MAX_CELLS
    assert (a.nPx + 2) * (a.nPy + 2) * (a.nPz + 2) > abi.NOALLOC_MAX_CELLS
    assert L.mhd_fluxes_noalloc(C.byref(a), None) == -1
