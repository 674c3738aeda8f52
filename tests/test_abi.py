"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
entry point include/*.h declares (no compute calls: CPU only)."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(mcd_[a-z0-9_]+)\s*\(",
                             text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("mcd_create", "mcd_destroy", "mcd_last_error", "mcd_price_european",
                     "mcd_price_batch", "mcd_philox", "mcd_draws"):
        assert required in names


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = C.CDLL(gpu_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_create_without_gpu_fails_cleanly(gpu_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(gpu_lib.McdError):
        gpu_lib.Engine(0)


def test_abi_version_and_layouts(gpu_lib):
    lib = gpu_lib.lib()
    assert lib.mcd_abi_version() == 1
    assert gpu_lib.CONTRACT_DTYPE.itemsize == 128
    assert C.sizeof(gpu_lib.McResult) == 24
    assert C.sizeof(gpu_lib.McOptions) == 8

