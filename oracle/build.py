"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/mft_oracle.c twice:
  _build/libmft_oracle.so        the parity build: FMA contraction disabled, so its
                                 rounding follows Julia code outside @muladd;
  _build/libmft_oracle_speed.so  the timing build of the CPU baseline: -O3 with FMA
                                 contraction and loop unrolling allowed.  No -march /
                                 -mcpu=native: the same recipe runs on x86_64 and on the
                                 aarch64 GPU hosts, whose baseline ISA already has FMA and
                                 128-bit SIMD.
"""
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libmft_oracle.so"
OUT_SPEED = HERE / "_build" / "libmft_oracle_speed.so"

_COMMON = ["-std=c11", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", "-Wall",
           "-Wno-unused-variable"]
FLAGS = {"parity": ["-O2", "-ffp-contract=off"],
         "speed": ["-O3", "-ffp-contract=fast", "-funroll-loops"]}


def _one(out: Path, flags, force: bool) -> Path:
    src = HERE / "mft_oracle.c"
    hdr = HERE / "mft_oracle.h"
    if (not force and out.exists() and out.stat().st_mtime >= src.stat().st_mtime
            and out.stat().st_mtime >= hdr.stat().st_mtime
            and out.stat().st_mtime >= Path(__file__).stat().st_mtime):
        return out
    out.parent.mkdir(parents=True, exist_ok=True)
    tmp = out.with_suffix(".so.tmp%d" % os.getpid())
    cmd = ["gcc"] + flags + _COMMON + ["-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


def build(force: bool = False, variant: str = "parity") -> Path:
    """Builds both variants (they compile in parallel); returns the requested one."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(2) as ex:
        futs = {v: ex.submit(_one, o, FLAGS[v], force)
                for v, o in (("parity", OUT), ("speed", OUT_SPEED))}
        paths = {v: f.result() for v, f in futs.items()}
    return paths[variant]


def flags(variant: str) -> str:
    return " ".join(["gcc"] + FLAGS[variant] + _COMMON)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
