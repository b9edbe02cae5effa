"""C-ABI checks that need no GPU: the library loads, exports every entry
point include/*.h declares, rejects unsupported configurations before any
CUDA call, and derives the reference's float-rounded constants bit for bit."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import REPO
from mhd_gb300 import abi
from mhd_gb300.case import small_cases
from mhd_gb300.sim import params_for

import oracle


@pytest.fixture(scope="module")
def lib():
    import sys
    sys.path.insert(0, str(REPO / "rast-3dmhd-cpp_gb300"))
    import build as mhd_build
    mhd_build.build()
    return abi.load()


def declared_symbols():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(mhd_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(abi.SIGNATURES), set(syms) - set(abi.SIGNATURES)


def test_status_strings(lib):
    assert lib.mhd_status_string(0) == b"ok"
    assert lib.mhd_status_string(-2) == b"unsupported configuration"


@pytest.mark.parametrize("change, status", [
    (dict(nPz=3), -1),
    (dict(izCon=2), -2),
    (dict(iTCon=3), -2),
    (dict(iBCon=1), -2),
    (dict(RE=0.0), -1),
])
def test_invalid_configs_rejected_without_gpu(lib, change, status):
    case = small_cases()["mhd_fixedT"].replace(**change)
    p, keep = params_for(case)
    ctx = C.c_void_p()
    assert lib.mhd_create(C.byref(p), None, C.byref(ctx)) == status
    assert not ctx.value


def test_lrem_and_nonperiodic_rejected(lib):
    """lRem with lShr (the reference then reads unfilled arrays) is rejected,
    as are non-periodic horizontal walls."""
    case = small_cases()["mhd_rot_shr"].replace(lRem=True)
    p, keep = params_for(case)
    ctx = C.c_void_p()
    assert lib.mhd_create(C.byref(p), None, C.byref(ctx)) == -2
    case = small_cases()["mhd_fixedT"]
    p, keep = params_for(case)
    p.ixCon = 1
    assert lib.mhd_create(C.byref(p), None, C.byref(ctx)) == -2


@pytest.mark.parametrize("name", sorted(small_cases()))
def test_constants_match_oracle_bit_exact(lib, name):
    case = small_cases()[name]
    p, keep = params_for(case)
    k = abi.MhdConstants()
    assert lib.mhd_compute_constants(C.byref(p), C.byref(k)) == 0
    o = oracle.OracleSim(case).p
    for f, _ in k._fields_:
        assert getattr(k, f) == getattr(o, f), f
