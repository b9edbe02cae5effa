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
    return sorted(json.loads((GOLDEN / "cases.json").read_text()).keys())


def load_golden(name):
    from mhd_gb300.case import Case
    d = json.loads((GOLDEN / "cases.json").read_text())[name]
    case = Case(**d)
    z = np.load(GOLDEN / f"{name}.npz")
    return case, {k: z[k] for k in z.files}
