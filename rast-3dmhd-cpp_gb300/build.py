"""Build the in-tree CUDA library libmhd_gb300.so for sm_103a.

Each .cu translation unit is compiled by nvcc in parallel, then linked into
one shared library with the C ABI of include/mhd_gb300.h.  The parity TU is
compiled with -fmad=false (no FMA contraction, so it reproduces the CPU
reference bit for bit); the other kernels keep FMA contraction on.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
LIB = OUT / "libmhd_gb300.so"
OBJ = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++20", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", str(PKG.parent / "include")]
# (source, object name, extra flags)
UNITS = [
    ("mhd_abi.cu", "mhd_abi", []),
    ("mhd_parity.cu", "mhd_parity", ["-fmad=false"]),
    ("mhd_fused.cu", "mhd_fused", []),
    ("mhd_fused.cu", "mhd_fused_xp", ["-DMHD_FUSED_XP=1"]),
    ("mhd_fused_batch.cu", "mhd_fused_batch_uxy", ["-DMHD_BATCH_UXY=1"]),
    ("mhd_fused_batch.cu", "mhd_fused_batch_gen", ["-DMHD_BATCH_UXY=0"]),
    ("mhd_diag.cu", "mhd_diag", []),
    ("mhd_noalloc.cu", "mhd_noalloc", []),
    ("mhd_fp32.cu", "mhd_fp32", []),
    ("mhd_batch.cu", "mhd_batch", []),
    ("mhd_io.cu", "mhd_io", []),
    ("mhd_init.cu", "mhd_init", []),
    ("mhd_pipeline.cu", "mhd_pipeline", []),
    ("mhd_selftest.cu", "mhd_selftest", []),
    ("mhd_static.cu", "mhd_static", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (cand == "nvcc" or Path(cand).exists()):
            return cand
    return "nvcc"


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    OUT.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "mhd_gb300.h"]
    jobs = []
    for src, oname, extra in UNITS:
        s = CSRC / src
        o = OBJ / (oname + ".o")
        if _stale(o, [s] + headers) or ptxas_info:
            cmd = [nvcc()] + ARCH + COMMON + extra + (["-Xptxas", "-v"] if ptxas_info else []) + \
                  ["-c", str(s), "-o", str(o)]
            jobs.append((oname, cmd))

    def run(job):
        name, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return name, r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for name, r in ex.map(run, jobs):
                if verbose or ptxas_info:
                    sys.stderr.write(r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr[-6000:]}")
    objs = [OBJ / (oname + ".o") for _, oname, _ in UNITS]
    if _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
