"""The C-ABI library loads (no GPU needed) and exports every function that
include/ubr.h declares; the ctypes mirror matches the header."""
import re
from pathlib import Path

from umbreon_gb300 import abi, build

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "ubr.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ubr_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    build.build_ubr()
    names = declared_functions()
    assert len(names) >= 10
    L = abi.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(abi.SIGNATURES), "ctypes signatures out of sync with include/ubr.h"


def test_status_strings_and_version():
    L = abi.lib()
    assert L.ubr_abi_version() == abi.ABI_VERSION
    for code in abi.STATUS:
        assert L.ubr_status_string(code)


def test_context_creation_without_gpu_reports_no_device():
    import ctypes as C
    import torch
    if torch.cuda.is_available():
        return
    h = C.c_void_p()
    assert abi.lib().ubr_context_create(C.byref(h), None) == abi.UBR_NO_DEVICE
