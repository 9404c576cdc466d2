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


def test_create_rejects_bad_grids_before_device_work(lib_path):
    """fdmgpu_create checks nspino (1, or 2 with spin-orbit) and the grid sizes
    before it touches a device, so the checks run on a host without a GPU."""
    from fdmnes_gb300 import abi, cluster as CL
    lib = C.CDLL(lib_path)
    lib.fdmgpu_create.argtypes = [C.c_void_p, C.c_void_p]
    lib.fdmgpu_create.restype = C.c_int
    d = abi.grid_dict(CL.small_cu_structure())
    h = C.c_void_p()
    for bad in ({"nspino": 3}, {"nspino": 0}, {"npoint": 0}, {"ngrph": 0}):
        ga = abi.GridArgs(dict(d, **bad))
        assert lib.fdmgpu_create(C.addressof(ga.s), C.byref(h)) == 1, bad
        assert not h.value
