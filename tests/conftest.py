import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG_DIR = ROOT / "meshfreetrixi.jl_gb300"
for p in (str(ROOT), str(PKG_DIR)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def cyl():
    """Reference fixture test/data/cyl_0_05 (2154 nodes) as committed golden data."""
    import numpy as np
    d = np.load(GOLDEN / "cyl_0_05.npz")
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; on a GPU run it must load."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("mft_build", PKG_DIR / "build.py")
    libbuild = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(libbuild)
    libbuild.build()
    import meshfree_gb300 as m
    m.load()
    return m
