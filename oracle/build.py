"""Builds the test harness that runs the reference's own driver and CUDA
graph backend on the GPU host (oracle/ref_gpu.cu).

TEST INFRASTRUCTURE ONLY.  It needs oracle/_ref/cuminlp_ref_gpu.cuh, which
oracle/build_ref.sh writes from the reference tree where that is mounted; the
header travels with the working tree, so the harness can be compiled on any
machine with nvcc.  Without the header nothing is built and the tests that
need the harness skip.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF_OUT = HERE / "_ref"
HEADER = REF_OUT / "cuminlp_ref_gpu.cuh"
GAMS_SRC = REF_OUT / "cuminlp_ref_gams.cpp"
GAMS_OBJ = REF_OUT / "ref_gams_frontend.o"
OBJ = REF_OUT / "ref_gpu.o"
EXE = REF_OUT / "ref_gpu"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: Path, deps: list[Path]) -> bool:
    return not target.exists() or any(d.stat().st_mtime > target.stat().st_mtime for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def available() -> bool:
    return HEADER.exists()


def compile_ref_gpu(force: bool = False) -> Path | None:
    """Compiles ref_gpu.cu, and the reference's GAMS frontend beside it, to
    objects (no library needed yet)."""
    if not available():
        return None
    if GAMS_SRC.exists() and (force or _stale(GAMS_OBJ, [GAMS_SRC])):
        # plain IEEE arithmetic in the frontend's constant folding, as the
        # reference builds it
        _run([os.environ.get("CXX", "g++"), "-std=c++20", "-O2", "-ffp-contract=off", "-fPIC",
              f"-I{HERE / 'ref_shim_gpu'}", "-c", "-x", "c++", str(GAMS_SRC), "-o", str(GAMS_OBJ)])
    deps = [HEADER, HERE / "ref_gpu.cu", ROOT / "include" / "cuminlp_gb300.h",
            ROOT / "include" / "cuminlp_gb300" / "region_backend.hpp",
            ROOT / "include" / "cuminlp_gb300" / "aggregate_backend.hpp",
            HERE / "ref_shim_gpu" / "cuinterval" / "cuinterval.h", HERE / "ref_shim_gpu" / "cuinterval" / "interval.h",
            HERE / "oracle.h", HERE / "ref_oracle_roles.hpp"]
    if force or _stale(OBJ, deps):
        _run([_nvcc(), "-std=c++20", "-O2", ARCH, "--expt-relaxed-constexpr", "-w",
              f"-I{REF_OUT}", f"-I{HERE / 'ref_shim_gpu'}", f"-I{ROOT / 'include'}",
              "-c", str(HERE / "ref_gpu.cu"), "-o", str(OBJ)])
    return OBJ


def link_ref_gpu(lib: Path, force: bool = False) -> Path | None:
    """Links the harness against the library built in place, and against
    the oracle (its "oracle" backend: the reference driver over the CPU
    oracle's roles)."""
    if not available() or not OBJ.exists():
        return None
    from cuminlp_gb300 import build as b
    orc = b.build_oracle()
    objs = [OBJ] + ([GAMS_OBJ] if GAMS_OBJ.exists() else [])
    if force or _stale(EXE, objs + [lib, orc]):
        _run([_nvcc(), ARCH, *map(str, objs), "-o", str(EXE), f"-L{lib.parent}", "-lcuminlp_gb300",
              f"-L{orc.parent}", "-loracle", "-Xlinker", "-rpath", "-Xlinker", str(lib.parent),
              "-Xlinker", "-rpath", "-Xlinker", str(orc.parent)])
    return EXE
