"""Build recipe of the CPU oracle (test infrastructure only).

Compiles ``oracle/fvoracle.c`` and ``oracle/boxmesh.c`` into ``oracle/_build/libfvoracle.so`` with
``-ffp-contract=off`` (no contraction of a*b+c into a fused multiply-add; the
algorithm calls fma() explicitly where it wants one) and OpenMP for the timed
multi-core CPU baseline.  The reference implementation (FoamAdapter + NeoN +
Kokkos + Ginkgo + OpenFOAM) cannot be compiled here, so there is no
``oracle/_ref`` build; the oracle is this restatement.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "fvoracle.c"
SRCS = [SRC, HERE / "boxmesh.c"]
HDR = HERE / "fvoracle.h"
OUT = HERE / "_build" / "libfvoracle.so"


def build() -> Path:
    OUT.parent.mkdir(parents=True, exist_ok=True)
    deps = [*SRCS, HDR, Path(__file__)]
    if OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", *map(str, SRCS), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build())
