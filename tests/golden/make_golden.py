"""Generate the golden fixtures from the reference 3dmhd code itself.

Run where the reference sources are at hand (MHD_REFERENCE_DIR, else a
"reference" directory beside this repository):

    python tests/golden/make_golden.py

For every small switch-coverage case (mhd_gb300.case.small_cases, the
plume cases of mhd_gb300.case.plume_cases and the lRem cases of
mhd_gb300.case.lrem_cases) it builds
the reference with oracle/refcase.py (2 x 2 forked MPI ranks), feeds it the
seeded initial state and stores, as <case>.npz:
  in_*      the input state and metric arrays (so the fixture does not depend
            on this host's libm when it is replayed elsewhere)
  flux_*    the right-hand sides after one fluxes() call (interior only)
  steps3_*  the full state (ghosts included) after 3 fixed-dt RK3 steps
  cfl2_*    the state after 2 steps of the reference step() with its CFL dt,
            and cfl2_dt the two time steps (two cases only)
plus config0_digest.json: SHA-256 digests of the 64x64x32 MHD run of the
plain-method configuration after 100 fixed-dt steps (too large to store),
and for every fresh-start case of mhd_gb300.case.static_cases the state the
reference's Static() and communicate() build (<case>.npz, all fields,
ghosts included, with the z coordinates it was given).

    python tests/golden/make_golden.py --only static   # just the Static() fixtures
"""
from __future__ import annotations

import argparse
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "oracle"))
sys.path.insert(0, str(REPO / "rast-3dmhd-cpp_gb300" / "python"))

import refcase  # noqa: E402
from mhd_gb300.case import (FLUX_FIELDS, STATE_FIELDS, config0, config1, coordinates, initial_state,  # noqa: E402
                            lrem_cases, metrics, plume_cases, small_cases, static_cases)

METRIC_NAMES = ("dxxdx", "d2xxdx2", "DDX", "dyydy", "d2yydy2", "DDY", "dzzdz", "d2zzdz2", "DDZ", "RKAPA", "DKAPA")
CFL_CASES = ("mhd_fixedT", "hydro_default_bc", "lrem_fixedT", "lrem_flux")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def static_fixtures() -> None:
    """Static() + communicate() of every fresh-start case (harness mode 5);
    the input state is zero, as the reference's arrays are at a fresh start."""
    manifest = {}
    for name, case in static_cases().items():
        zero = {k: np.zeros(case.shape) for k in STATE_FIELDS}
        r = refcase.run(case, zero, "static", 0)
        out = {"ZEE": coordinates(case)[2]}
        for k in STATE_FIELDS[:case.nfields]:
            out["static_" + k] = r[k]
        if case.lRem:  # the harness returns RKAPA / DKAPA in the FU / FV slots
            out["static_RKAPA"] = r["FU"][:, 1, 1].copy()
            out["static_DKAPA"] = r["FV"][:, 1, 1].copy()
            out["static_walls"] = np.array([r["TU"], r["DZTU"], r["DZTB"]])
        np.savez_compressed(HERE / f"{name}.npz", **out)
        manifest[name] = case.to_dict()
        print("wrote", name)
    (HERE / "static_cases.json").write_text(json.dumps(manifest, indent=1, sort_keys=True))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=("all", "static"), default="all")
    args = ap.parse_args()
    if not refcase.reference_available():
        raise SystemExit(f"reference sources not found under {refcase.REF_DIR}")
    static_fixtures()
    if args.only == "static":
        return
    manifest = {}
    for name, case in list(small_cases().items()) + list(plume_cases().items()) + list(lrem_cases().items()):
        st = initial_state(case)
        m = metrics(case)
        out = {}
        for k in STATE_FIELDS:
            out["in_" + k] = st[k]
        for k, a in zip(METRIC_NAMES, m.arrays()):
            out["in_" + k] = a
        r = refcase.run(case, st, "fluxes", 0)
        for k in FLUX_FIELDS:
            out["flux_" + k] = r[k][1:-1, 1:-1, 1:-1]
        r = refcase.run(case, st, "steps", 3)
        for k in STATE_FIELDS:
            out["steps3_" + k] = r[k]
        if name in CFL_CASES:
            r = refcase.run(case, st, "cfl", 2)
            for k in STATE_FIELDS:
                out["cfl2_" + k] = r[k]
            out["cfl2_dt"] = r["dt_hist"]
        np.savez_compressed(HERE / f"{name}.npz", **out)
        manifest[name] = case.to_dict()
        print("wrote", name)
    (HERE / "cases.json").write_text(json.dumps(manifest, indent=1, sort_keys=True))

    # the reference's own dump files (dumpData) of two cases after 3 steps
    for name in ("mhd_fixedT", "hydro_default_bc"):
        case = small_cases()[name]
        d = HERE / f"dat0_{name}"
        d.mkdir(exist_ok=True)
        refcase.run(case, initial_state(case), "dump", 3, dump_prefix=str((d / "test").resolve()))
        print("wrote", d)

    c0 = config0()
    st = initial_state(c0)
    r = refcase.run(c0, st, "steps", 100)
    digest = {
        "case": c0.to_dict(),
        "steps": 100,
        "reference_ranks": c0.nPEy * c0.nPEz,
        "input_sha256": {k: sha(st[k]) for k in STATE_FIELDS},
        "output_sha256": {k: sha(r[k]) for k in STATE_FIELDS},
        "output_interior_absmax": {k: float(np.abs(r[k][1:-1, 1:-1, 1:-1]).max()) for k in STATE_FIELDS},
        "TIMT": r["TIMT"],
    }
    (HERE / "config0_digest.json").write_text(json.dumps(digest, indent=1, sort_keys=True))
    print("wrote config0_digest.json")

    # the 512x512x256 benchmark's physics (lMag, lRot 0.1 about z, lShr) at 64x64x32, 20 steps
    c1 = config1().replace(nPx=64, nPy=64, nPz=32, nPEy=2, nPEz=2, name="config1_physics_64x64x32")
    st = initial_state(c1)
    r = refcase.run(c1, st, "steps", 20)
    digest = {
        "case": c1.to_dict(),
        "steps": 20,
        "reference_ranks": 4,
        "input_sha256": {k: sha(st[k]) for k in STATE_FIELDS},
        "output_sha256": {k: sha(r[k]) for k in STATE_FIELDS},
        "output_interior_absmax": {k: float(np.abs(r[k][1:-1, 1:-1, 1:-1]).max()) for k in STATE_FIELDS},
    }
    (HERE / "config1_64x64x32_digest.json").write_text(json.dumps(digest, indent=1, sort_keys=True))
    print("wrote config1_64x64x32_digest.json")


if __name__ == "__main__":
    main()
