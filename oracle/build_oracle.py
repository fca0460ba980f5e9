"""Build recipe of the CPU oracle (test infrastructure only).

Compiles ``oracle/sbm_oracle.c`` into ``oracle/build/libsbm_oracle.so`` with
``-O2 -ffp-contract=off`` (no fused multiply-add, so the Fortran evaluation
order is kept exactly) and OpenMP.  The reference itself (Fortran + MPI) has
no compiler in this image, so there is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "sbm_oracle.c"
HDRS = [HERE / "sbm_oracle.h", HERE.parent / "include" / "sbm_capi.h"]
LIB = HERE / "build" / "libsbm_oracle.so"

CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
          "-std=c11", "-Wall"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(
            p.stat().st_mtime <= LIB.stat().st_mtime for p in [SRC, *HDRS]):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CC", "gcc"), *CFLAGS, "-o", str(tmp), str(SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
