"""The integer float <-> double conversions of the double-word epilogues
(meshfreetrixi.jl_gb300/csrc/mft_fpbits.h), compiled for the host with g++ and checked
against the host's IEEE conversions: float -> double over all 2^32 float patterns,
double -> float (round to nearest, ties to even) over every exponent and sign with random
significands and the exact ties.  The device code calls the same functions."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_integer_conversions_match_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "fpbits_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", str(ROOT / "meshfreetrixi.jl_gb300" / "csrc"),
                    str(ROOT / "tests" / "fpbits_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "1"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:]
    assert out.stdout.startswith("ok f2d 4261412866 ")
