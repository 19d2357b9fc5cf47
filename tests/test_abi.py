"""The C ABI library: it loads and exports every symbol include/dim3gpu.h
declares (no compute calls -- this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "dim3gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dim3g_\w+)\s*\(", src)))


def test_header_declares_the_expected_api():
    names = declared_functions()
    import dim3gpu
    assert sorted(dim3gpu.EXPORTS) == names


def test_library_exports_every_declared_symbol(built):
    import dim3gpu
    lib = ctypes.CDLL(dim3gpu.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import dim3gpu
    with pytest.raises(dim3gpu.Dim3GError):
        dim3gpu.Context(0)
