"""The C-ABI library builds, loads and exports every entry point its header declares."""
import ctypes
import os
import subprocess

import pytest

from shci_gb300 import _lib


@pytest.fixture(scope="module")
def lib():
    from shci_gb300 import build
    build.build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_exports_every_declared_symbol(lib):
    names = _lib.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_header_is_plain_c():
    """The boundary header compiles as C (no C++ or torch types in the signatures)."""
    r = subprocess.run(["gcc", "-x", "c", "-std=c99", "-fsyntax-only", "-Wall", "-Werror",
                        os.path.abspath(_lib.HEADER)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_create_reports_missing_gpu_cleanly(lib):
    """Without a visible GPU the context cannot be created: a status, not a crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    h = ctypes.c_void_p()
    lib.shci_create.restype = ctypes.c_int
    st = lib.shci_create(ctypes.byref(h), 0, ctypes.c_size_t(0))
    assert st != 0
    assert not h.value
    with pytest.raises(_lib.ShciError):
        _lib.Context()
