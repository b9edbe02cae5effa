"""Build and run the reference 3dmhd code as the parity oracle.

TEST INFRASTRUCTURE ONLY.  Nothing on the product path imports this module:
only tests/, the golden-fixture script and bench.py's CPU-baseline leg do.

Recipe (no reference sources are copied):
  * generate a 3dmhdparam.h (grid sizes, switches, decomposition) and a
    3dmhdset.h (the ``par[]`` run table, exact hex-float literals) for the case
    into ``oracle/_ref/<key>/``;
  * compile oracle/ref_harness.cpp, which #includes the reference's own
    3dmhd.cpp, with ``g++ -O2 -std=c++20 -ffp-contract=off`` and the include
    order ``-I <key dir> -I- -I <reference> -I oracle/mpishim`` so that the
    generated headers shadow the reference's copies (the reference includes
    them with quotes from its own directory);
  * link oracle/mpishim/mpishim.c (forked ranks over shared memory).
The reference tree is only needed to BUILD; the binaries land in
``oracle/_ref/`` (git-ignored).
"""
from __future__ import annotations

import fcntl
import hashlib
import os
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(REPO / "rast-3dmhd-cpp_gb300" / "python"))
from mhd_gb300.case import Case, STATE_FIELDS, FLUX_FIELDS, ZFIELDS, coordinates, metrics  # noqa: E402

# the reference checkout: MHD_REFERENCE_DIR, else a "reference" directory beside
# this repository
REF_DIR = Path(os.environ.get("MHD_REFERENCE_DIR", str(REPO.parent / "reference")))
OUT_DIR = HERE / "_ref"
MAGIC = 0x3344484D


def reference_available() -> bool:
    return (REF_DIR / "3dmhd.cpp").is_file()


def _hexf(v: float) -> str:
    return float(v).hex()


def _b(v: bool) -> str:
    return "true" if v else "false"


def param_header(case: Case) -> str:
    """3dmhdparam.h for one case: the same symbol set the reference declares
    (3dmhdparam.h:1-124), with this case's sizes and switches."""
    if case.nPy % case.nPEy or case.nPz % case.nPEz:
        raise ValueError("grid not divisible by the rank grid")
    if case.nPEz < 2:
        raise ValueError("the reference needs nPEz >= 2 (3dmhdparam.h:20)")
    return f"""#pragma once
#include <string>
#include <sys/stat.h>
const std::string outputDir = "output/";
const std::string fInp = outputDir + "test";
const std::string fOut = outputDir + "test";
#define lRot {_b(case.lRot)}
#define lMag {_b(case.lMag)}
#define lPot false
#define lRem {_b(case.lRem)}
#define lShr {_b(case.lShr)}
const int nPEy = {case.nPEy};
const int nPEz = {case.nPEz};
const int nPE = nPEy * nPEz;
const int nPx = {case.nPx};
const int nPy = {case.nPy};
const int nPz = {case.nPz};
const int nRy = nPy / nPEy;
const int nRz = nPz / nPEz;
const int nCore = nPx * nRy * nRz;
const int ix = 2;
const int iy = 2;
const int iz = 2;
const int IPAD = 0;
const int ny = nRy + iy;
const int nz = nRz + iz;
const int nx = nPx + ix;
#define nGrid 0
const double XX1 = 0, XX2 = 0;
const double YY1 = 0, YY2 = 0;
const double ZZ1 = 0, ZZ2 = 0;
const double XA = 0, XB = 0, XC = 0, XD = 0;
const double YA = 0, YB = 0, YC = 0, YD = 0;
const double ZA = 0, ZB = 0, ZC = 0, ZD = 0;
#define ixCon 0
#define iyCon 0
#define izCon {case.izCon}
#define iTCon {case.iTCon}
#define iBCon {case.iBCon}
const double SFF = {_hexf(case.SFF)};
#define iD 0
const double DH = 0, DV = 0;
const int iWord = 8;
const int nCol = 0, nRow = 0, nTubes = nCol * nRow;
#define nTube {case.nTube}
"""


def set_header(case: Case) -> str:
    """3dmhdset.h for one case: setup() fills ipar/par like 3dmhdset.h:7-24."""
    par = {0: case.RE, 1: case.PR, 2: case.THETA, 3: case.GRAV, 4: case.RY, 5: case.ANG,
           6: case.RM, 7: case.BETA, 11: case.TP, 12: case.TC, 13: case.XP, 14: case.YP, 15: case.ZP,
           16: case.xMax, 17: case.yMax, 18: case.zMax, 52: case.QFH, 53: case.GAMMA, 54: case.HH}
    # Static()'s model (3dmhd.cpp:409-423), written only when set so that the
    # headers of the other cases stay as they were
    for k, v in ((8, case.PZP), (9, case.SIGMA), (10, case.POLYS), (19, case.AMPT), (20, case.AMPB),
                 (21, case.BFH), (22, case.BZP), (34, case.XCENT), (35, case.ZCENT), (36, case.R_MAX),
                 (37, case.C_MT), (38, case.A_TUBE)):
        if v != 0.0:
            par[k] = v
    lines = "\n".join(f"    par[{k}] = {_hexf(v)};" for k, v in sorted(par.items()))
    return f"""#ifndef _3DMHD_SET_H_
#define _3DMHD_SET_H_
#include <cmath>
#include <string>
void setup(int ipar[32], double par[64]) {{
    for (int i = 0; i < 32; i++) ipar[i] = 0;
    for (int i = 0; i < 64; i++) par[i] = 0;
    ipar[0] = 1;
    ipar[1] = 1;
    ipar[2] = 10;
    ipar[3] = 1;
{lines}
}}
#endif
"""


def build_key(case: Case) -> str:
    h = hashlib.sha1((param_header(case) + set_header(case)).encode()).hexdigest()[:12]
    return f"p{case.nPx}x{case.nPy}x{case.nPz}_r{case.nPEy}x{case.nPEz}_{h}"


def _shim_object() -> Path:
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    obj = OUT_DIR / "mpishim.o"
    src = HERE / "mpishim" / "mpishim.c"
    if not obj.exists() or obj.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-std=gnu11", "-c", str(src), "-o", str(obj)], check=True)
    return obj


def build(case: Case) -> Path:
    """Compile the reference harness for ``case``; returns the binary path."""
    if not reference_available():
        raise FileNotFoundError(f"reference sources not found under {REF_DIR}")
    key = build_key(case)
    d = OUT_DIR / key
    exe = d / "ref_harness"
    harness = HERE / "ref_harness.cpp"
    d.mkdir(parents=True, exist_ok=True)
    # one build per key at a time: concurrent builds would rewrite the
    # generated headers under each other's compiler
    with open(d / ".lock", "w") as lk:
        fcntl.flock(lk, fcntl.LOCK_EX)
        if exe.exists() and exe.stat().st_mtime >= harness.stat().st_mtime:
            return exe
        (d / "3dmhdparam.h").write_text(param_header(case))
        (d / "3dmhdset.h").write_text(set_header(case))
        shim = _shim_object()
        tmp = d / f"ref_harness.{os.getpid()}.tmp"
        cmd = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-w",
               "-I", str(d), "-I-", "-I", str(REF_DIR), "-I", str(HERE / "mpishim"),
               str(harness), str(shim), "-o", str(tmp)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + r.stderr[-4000:])
        os.replace(tmp, exe)
    return exe


# ---------------------------------------------------------------------------
# harness input / output files
# ---------------------------------------------------------------------------
MODES = {"fluxes": 0, "steps": 1, "cfl": 2, "substage": 3, "dump": 4, "static": 5}


def write_input(path: Path, case: Case, state: dict, mode: str, nsteps: int,
                FT: np.ndarray | None = None, timt0: float = 0.0) -> None:
    m = metrics(case)
    # version 2: the coordinate arrays EXX, WYY, ZEE follow the nine fields
    hdr = struct.pack("<8i8i", MAGIC, 2, case.nPx, case.nPy, case.nPz, int(case.lMag), MODES[mode], nsteps,
                      *([0] * 8))
    # reserved doubles 0-2: the lRem wall values TU, DZTU, DZTB
    hdr += struct.pack("<16d", case.dt, case.tb, timt0, case.TU, case.DZTU, case.DZTB, *([0.0] * 10))
    with open(path, "wb") as f:
        f.write(hdr)
        for a in m.arrays():
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        for k in STATE_FIELDS:
            f.write(np.ascontiguousarray(state[k], dtype=np.float64).tobytes())
        ft = np.zeros(case.shape) if FT is None else FT
        f.write(np.ascontiguousarray(ft, dtype=np.float64).tobytes())
        for a in coordinates(case):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())


def read_output(path: Path, case: Case, nsteps: int) -> dict:
    n = int(np.prod(case.shape))
    raw = np.fromfile(path, dtype=np.float64)
    out = {}
    names = list(STATE_FIELDS) + list(FLUX_FIELDS) + list(ZFIELDS)
    for i, k in enumerate(names):
        out[k] = raw[i * n:(i + 1) * n].reshape(case.shape).copy()
    tr = raw[24 * n:]
    out["TIMT"] = float(tr[0])
    out["UMACH"] = float(tr[1])
    out["seconds"] = float(tr[2])
    out["DT"] = float(tr[4])
    out["dt_hist"] = tr[16:16 + nsteps].copy()
    # mode "static" with lRem: the wall values Static() derived
    out["TU"], out["DZTU"], out["DZTB"] = float(tr[5]), float(tr[6]), float(tr[7])
    return out


def run(case: Case, state: dict, mode: str = "steps", nsteps: int = 1,
        FT: np.ndarray | None = None, timt0: float = 0.0, timeout: float = 1800.0,
        dump_prefix: str | None = None) -> dict:
    """Run the reference on ``state`` and return the gathered global arrays.
    mode "dump" also has the reference write its own dump files at dump_prefix."""
    exe = build(case)
    with tempfile.TemporaryDirectory(prefix="mhdref_") as td:
        fin = Path(td) / "in.bin"
        fout = Path(td) / "out.bin"
        write_input(fin, case, state, mode, nsteps, FT=FT, timt0=timt0)
        cmd = [str(exe), str(fin), str(fout)] + ([dump_prefix] if dump_prefix else [])
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=td)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}):\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        return read_output(fout, case, nsteps)
