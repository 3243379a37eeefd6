"""In-tree build of libfvgb.so (the sm_103a CUDA library and its C ABI).

Every translation unit is compiled in parallel with nvcc for sm_103a only and
linked into ``foamadapter_gb300/_lib/libfvgb.so`` (static CUDA runtime).  The
finite-volume kernels are compiled with ``-fmad=false`` so that no
multiply-add is contracted: their results are bit-identical to the serial CPU
face loops they restate.  Host C++ is compiled with ``-ffp-contract=off`` so
x86-64 and aarch64 hosts produce the same mesh geometry.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
OBJ_DIR = OUT_DIR / "obj"
LIB = OUT_DIR / "libfvgb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               f"-I{INCLUDE}", f"-I{CSRC}"] + ARCH
# translation unit -> extra flags
CU_UNITS = {
    "mesh.cu": [],
    "explicit_ops.cu": ["-fmad=false"],
    "assembly.cu": ["-fmad=false"],
    "solver.cu": ["-fmad=false"],
    "piso.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "boxmesh.cu": ["-fmad=false"],
    "serve.cu": [],
    "amg.cu": [],
    "ilu.cu": ["-fmad=false"],
}
CPP_UNITS = ["common.cpp", "meshgen.cpp", "foamio.cpp", "foamdict.cpp", "tunecache.cpp"]
HEADERS = [INCLUDE / "fvgb.h", CSRC / "internal.cuh", CSRC / "fvgb_host_common.h", CSRC / "json_min.h", CSRC / "tunecache.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfvgb")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile (if stale) and link libfvgb.so; returns its path."""
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for unit, extra in CU_UNITS.items():
        src = CSRC / unit
        obj = OBJ_DIR / (unit + ".o")
        if ptxas_info or _stale(obj, [src, *HEADERS, Path(__file__)]):
            cmd = [nvcc, "-c", str(src), "-o", str(obj), *NVCC_COMMON, *extra]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for unit in CPP_UNITS:
        src = CSRC / unit
        obj = OBJ_DIR / (unit + ".o")
        if _stale(obj, [src, *HEADERS, Path(__file__)]):
            jobs.append(["g++", "-c", str(src), "-o", str(obj), "-O2", "-std=c++17", "-fPIC",
                         "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    objs = [OBJ_DIR / (u + ".o") for u in list(CU_UNITS) + CPP_UNITS]
    if jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, LIB)
    if verbose or ptxas_info:
        for log in logs:
            if log.strip():
                print(log)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
