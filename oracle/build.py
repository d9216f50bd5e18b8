"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/mft_oracle.c into oracle/_build/libmft_oracle.so with FMA
contraction disabled, so its rounding follows Julia code outside @muladd.
"""
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libmft_oracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "mft_oracle.c"
    hdr = HERE / "mft_oracle.h"
    if (not force and OUT.exists() and OUT.stat().st_mtime >= src.stat().st_mtime
            and OUT.stat().st_mtime >= hdr.stat().st_mtime):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp%d" % os.getpid())
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-Wall", "-Wno-unused-variable", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
