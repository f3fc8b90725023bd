"""The C ABI library builds, loads without a GPU and exports every function
include/twochnrg_gb300.h declares (no compute calls here)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "twochnrg_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nrg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from twochnrg_gb300 import build
    path = build.build()
    return ctypes.CDLL(path), path


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("nrg_create", "nrg_sweep_run", "nrg_diag_blocks", "nrg_diag_block_noalloc"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    L, path = lib
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"not exported: {missing}"
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (nrg_[a-z0-9_]+)", out))
    assert set(declared_functions()) <= exported


def test_status_strings_without_a_device(lib):
    L, _ = lib
    L.nrg_status_string.restype = ctypes.c_char_p
    assert L.nrg_status_string(0) == b"ok"
    assert L.nrg_status_string(5) == b"size limit exceeded"


def test_create_fails_loudly_without_a_gb300(lib):
    """No CPU fallback: on a host without an sm_103 device nrg_create refuses."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L, _ = lib
    h = ctypes.c_void_p()
    assert L.nrg_create(0, ctypes.byref(h)) != 0
    assert not h.value


def test_noalloc_size_check_is_host_side(lib):
    """Sizes above NRG_NOALLOC_MAX_N are refused before any device access."""
    L, _ = lib
    L.nrg_diag_block_noalloc.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4
    dummy = ctypes.c_void_p(16)
    assert L.nrg_diag_block_noalloc(257, dummy, dummy, dummy, None) == 5
    assert L.nrg_diag_block_noalloc(0, dummy, dummy, dummy, None) == 1
