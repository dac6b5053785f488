"""Builds the native parts in place.

``build_library()`` compiles the CUDA sources under ``csrc/`` for sm_103a
into ``libcuminlp_gb300.so`` next to this file; each translation unit is
compiled in parallel, then linked.  ``build_oracle()`` compiles the CPU
oracle (test infrastructure) into ``oracle/liboracle.so``.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcuminlp_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    "-O3", "-std=c++17", ARCH, "-lineinfo", "--fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-frounding-math",
    "--expt-relaxed-constexpr", "-DNDEBUG",
]
SOURCES = ["program.cpp", "eval_kernels.cu", "search_kernels.cu", "batch_kernels.cu", "capi.cu", "batch.cu",
           "server.cpp", "noalloc.cu", "emu_check.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build cuminlp_gb300")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh"))
    headers.append(ROOT / "include" / "cuminlp_gb300.h")
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
            jobs.append([nvcc, *NVCC_FLAGS, *lang, "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lpthread"])
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(force: bool = False) -> Path:
    srcs = [ORACLE_DIR / "oracle.c", ORACLE_DIR / "oracle.h", ORACLE_DIR / "oracle_interval.inc",
            ROOT / "include" / "cuminlp_gb300.h"]
    if force or _stale(ORACLE_LIB, srcs):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-frounding-math", "-fPIC", "-shared",
              str(ORACLE_DIR / "oracle.c"), "-o", str(ORACLE_LIB), "-lm", "-lpthread"])
    return ORACLE_LIB


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("ok")
