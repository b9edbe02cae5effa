"""Helpers shared by the GPU tests."""
import numpy as np

from mhd_gb300.case import STATE_FIELDS, Case, initial_state, metrics
from mhd_gb300.sim import Simulation

import oracle

METRIC_NAMES = ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")


def sim_from_fixture(case, g, path):
    mo = {n: g["in_" + n] for n in METRIC_NAMES}
    sim = Simulation(case, path=path, metric_override=mo)
    sim.upload_state({k: g["in_" + k] for k in STATE_FIELDS})
    sim.communicate()
    return sim


def oracle_for(case, state, nthreads=8):
    o = oracle.OracleSim(case, state, nthreads=nthreads)
    o.communicate()
    return o


def rel_err(got, ref, sl=np.s_[1:-1]):
    """max |got - ref| over the selection, relative to max |ref| there."""
    a, b = got[sl], ref[sl]
    scale = np.abs(b).max()
    d = np.abs(a - b).max()
    return d / scale if scale > 0 else d
