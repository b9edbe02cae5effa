"""Shared test set-up: the ``gpu`` marker, import paths and fixture loaders."""
import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
GOLDEN = REPO / "tests" / "golden"
for p in (REPO / "rast-3dmhd-cpp_gb300" / "python", REPO / "oracle", REPO):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


def golden_case_names():
    """The small switch-coverage cases (GPU tests replay their fixtures)."""
    return sorted(k for k in json.loads((GOLDEN / "cases.json").read_text())
                  if not k.startswith("plume_") and not k.startswith("lrem_"))


def lrem_case_names():
    """The lRem cases (Rempel relaxation, one y rank)."""
    return sorted(k for k in json.loads((GOLDEN / "cases.json").read_text()) if k.startswith("lrem_"))


def plume_case_names():
    """The plume cases: their Gaussian factors come from the host's libm, so
    GPU tests compare them with the oracle run on the same host, and only the
    CPU tests replay their fixtures."""
    return sorted(k for k in json.loads((GOLDEN / "cases.json").read_text()) if k.startswith("plume_"))


def load_golden(name):
    from mhd_gb300.case import Case
    d = json.loads((GOLDEN / "cases.json").read_text())[name]
    case = Case(**d)
    z = np.load(GOLDEN / f"{name}.npz")
    return case, {k: z[k] for k in z.files}
