"""The C-ABI library builds, loads and exports every entry point of the header
(CPU only: no CUDA work is issued)."""
import ctypes as C
import re
from pathlib import Path

from conftest import ROOT


def _declared():
    text = (ROOT / "include" / "meshfree_gb300.h").read_text()
    decl = re.findall(r"^(?:mft_status|const char\*)\s+(mft_[a-z0-9_]+)\s*\(", text, re.M)
    return sorted(set(decl))


def test_header_and_binding_agree(gpu_lib):
    from meshfree_gb300._lib import SIGNATURES
    assert sorted(SIGNATURES) == _declared()


def test_library_exports_every_declared_symbol(gpu_lib):
    from meshfree_gb300._lib import LIB_PATH
    lib = C.CDLL(str(LIB_PATH))
    for name in _declared():
        assert hasattr(lib, name), name


def test_version_and_null_handling(gpu_lib):
    lib = gpu_lib.load()
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    assert lib.mft_version(C.byref(a), C.byref(b), C.byref(c)) == 0
    assert (a.value, b.value) >= (0, 1)
    # NULL handle / NULL output pointer are rejected with MFT_ERR_ARG, no abort
    assert lib.mft_ctx_create(None, 0, 0) == 1
    assert lib.mft_sync(None) == 1
    assert lib.mft_last_error(None) == b"null context"


def test_product_path_has_no_oracle_dependency():
    """The shipped package never imports the checker."""
    pkg = ROOT / "meshfreetrixi.jl_gb300"
    for p in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")):
        text = p.read_text()
        assert "oracle" not in text.replace("Oracle", "").lower() or p.name == "workloads.py", p
