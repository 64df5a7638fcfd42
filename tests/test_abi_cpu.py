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


STRUCTS = [("cmdg_brick_desc", "BrickDesc"), ("cmdg_shell_desc", "ShellDesc"), ("cmdg_atmos_params", "AtmosParams"),
           ("cmdg_grid_arrays", "GridArrays")]


def test_struct_layouts_match_the_header(tmp_path):
    """sizeof/offsetof of every descriptor struct, compiled from the header
    with the host C compiler, equals the ctypes layout of the binding."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "cmdg.h"', "int main(void) {"]
    for cname, pyname in STRUCTS:
        lines.append(f'printf("{pyname} size %zu\\n", sizeof({cname}));')
        for field, _ in getattr(_lib, pyname)._fields_:
            lines.append(f'printf("{pyname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    import subprocess

    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for _, pyname in STRUCTS:
        cls = getattr(_lib, pyname)
        assert got[(pyname, "size")] == ctypes.sizeof(cls), pyname
        for field, _ in cls._fields_:
            assert got[(pyname, field)] == getattr(cls, field).offset, (pyname, field)


JULIA_TYPES = {"Cint": ctypes.c_int, "Cdouble": ctypes.c_double, "Int64": ctypes.c_int64}


def julia_struct(text, name):
    body = re.search(rf"^struct {name}\n(.*?)^end", text, flags=re.M | re.S).group(1)
    return [re.match(r"\s*(\w+)::([^#]+?)\s*(?:#|$)", l).groups() for l in body.split("\n") if "::" in l]


def test_julia_shim_structs_match_the_binding():
    """The Julia ccall structs declare the same fields, in the same order and
    of the same C types, as the ctypes binding (and so as the header)."""
    text = open(os.path.join(REPO, "climatemachine.jl_gb300", "julia", "CMDG.jl")).read()
    for jname, pyname in [("Brick", "BrickDesc"), ("AtmosParams", "AtmosParams"), ("GridArrays", "GridArrays")]:
        jf = julia_struct(text, jname)
        pf = getattr(_lib, pyname)._fields_
        assert [f for f, _ in jf] == [f for f, _ in pf], jname
        for (f, jt), (_, ct) in zip(jf, pf):
            m = re.match(r"NTuple\{(\d+), (\w+)\}", jt)
            if m:
                assert ct._type_ == JULIA_TYPES[m.group(2)] and ct._length_ == int(m.group(1)), (jname, f)
            elif jt.startswith("Ptr"):
                assert ct == ctypes.c_void_p, (jname, f)
            else:
                assert ct == JULIA_TYPES[jt], (jname, f)
