"""The C-ABI library builds, loads and exports every entry point of include/fdmgpu.h."""
import os
import re
import ctypes as C

import pytest

from conftest import ROOT


@pytest.fixture(scope="session")
def lib_path():
    from fdmnes_gb300 import build
    return build.build()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fdmgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fdmgpu_[a-z_0-9]+)\s*\(", src)))


def test_exports_every_declared_symbol(lib_path):
    lib = C.CDLL(lib_path)
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n


def test_host_only_entry_points(lib_path):
    lib = C.CDLL(lib_path)
    lib.fdmgpu_version.restype = C.c_char_p
    assert b"sm_103a" in lib.fdmgpu_version()
    n = C.c_int32(0)
    buf = C.create_string_buffer(6)
    lib.fdmgpu_get_solver_params(C.byref(n), buf)
    assert n.value == 1 and buf.value.startswith(b"GPU")
    # argument checks happen before any device work
    assert lib.fdmgpu_create(None, None) == 1
    lib.fdmgpu_last_error.restype = C.c_char_p
    assert lib.fdmgpu_last_error()


def test_solver_module_fails_loudly_without_library(tmp_path):
    from fdmnes_gb300 import solver
    with pytest.raises(RuntimeError):
        solver.load_library(str(tmp_path / "missing.so"))
