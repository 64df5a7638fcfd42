"""CPU checks of the drop-in boundary: libcmdg.so builds, loads, and exports
every entry point that include/cmdg.h declares (no GPU call is made)."""
import ctypes
import os
import re

import pytest

from conftest import REPO

from cmdg import _lib

HEADER = os.path.join(REPO, "include", "cmdg.h")


def header_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(cmdg_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g

    g.build_library()
    return _lib.load()


def test_header_declares_the_python_binding():
    assert header_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_version_and_error_path_without_gpu(lib):
    assert b"sm_103a" in lib.cmdg_version()
    out = ctypes.c_void_p()
    # NULL descriptor: rejected before any CUDA call
    rc = lib.cmdg_mesh_create_brick(None, ctypes.byref(out))
    assert rc == 1 and out.value is None
    assert b"NULL" in lib.cmdg_last_error()
    d = _lib.BrickDesc()
    d.N = 9
    rc = lib.cmdg_mesh_create_brick(ctypes.byref(d), ctypes.byref(out))
    assert rc == 1 and b"polynomial order" in lib.cmdg_last_error()


def test_null_model_is_an_argument_error(lib):
    rc = lib.cmdg_tendency(None, None, None, 0.0, 1.0, 0.0, None)
    assert rc == 1
