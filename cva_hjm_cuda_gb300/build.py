"""Build recipe of libhjmcva.so (in-tree, sm_103a only).

    python -m cva_hjm_cuda_gb300.build

Every CUDA translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` in parallel, the C++
drop-in by g++, and the shared library is linked with the static CUDA runtime
into ``cva_hjm_cuda_gb300/lib/libhjmcva.so``.  Object files go to
``cva_hjm_cuda_gb300/_build/``.  No cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libhjmcva.so"

CUDA_SOURCES = ["hjm_forward.cu", "hjm_eresp.cu", "hjm_mresp.cu", "hjm_adjoint.cu", "hjm_pc.cu", "hjm_mlmc.cu", "hjm_capi.cu", "hjm_static.cu", "peak_fma.cu"]
CXX_SOURCES = ["hjm_dropin.cpp", "hjm_calib.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parents[1]
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", str(INCLUDE), "-c", str(s), "-o", str(o)])
    for src in CXX_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-I", str(INCLUDE), "-I", str(cuda / "include"),
                         "-c", str(s), "-o", str(o)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
