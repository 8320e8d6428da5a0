"""The C ABI: libraries load, export every declared entry point, and reject
bad configurations without touching a GPU."""
import ctypes as C
import os
import re

import pytest

from fv_140823_gb300 import abi
from fv_140823_gb300._native import lib_path, load_gpu_lib, load_mesh_lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header, prefix):
    src = open(os.path.join(REPO, "include", header)).read()
    return sorted(set(re.findall(r"\b(?:int|void|const char \*)\s*(" + prefix + r"\w+)\s*\(", src)))


@pytest.mark.parametrize("header,lib,prefix", [("fvgpu.h", "libfvgpu.so", "fvgpu_"),
                                               ("fvmesh.h", "libfvmesh.so", "fvmesh_")])
def test_every_declared_symbol_is_exported(header, lib, prefix):
    names = declared(header, prefix)
    assert len(names) >= 9
    dll = C.CDLL(lib_path(lib))
    missing = [n for n in names if not hasattr(dll, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from fv_140823_gb300._native import gpu_symbols
    assert sorted(gpu_symbols()) == declared("fvgpu.h", "fvgpu_")


def _create(**kw):
    lib = load_gpu_lib()
    cfg = abi.SolverConfig(**kw).to_c()
    ctx = C.c_void_p()
    rc = lib.fvgpu_create(C.byref(cfg), C.byref(ctx))
    if rc == 0:
        lib.fvgpu_destroy(ctx)
    return rc


@pytest.mark.parametrize("kw,rc", [(dict(model=4), abi.ERR_UNSUPPORTED), (dict(iprimtv=1), abi.ERR_UNSUPPORTED),
                                   (dict(ischeme=3), abi.ERR_ARG), (dict(precision=7), abi.ERR_ARG),
                                   (dict(gamma=1.0), abi.ERR_ARG)])
def test_config_validation_before_device(kw, rc):
    assert _create(**kw) == rc


def test_no_device_is_reported():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert _create() == abi.ERR_NODEVICE


def test_mesh_lib_errors():
    lib = load_mesh_lib()
    h = C.c_void_p()
    lo = (C.c_double * 3)(0, 0, 0)
    ln = (C.c_double * 3)(1, 1, 1)
    per = (C.c_int * 3)(0, 0, 0)
    bc = (C.c_int * 6)(2, 2, 2, 2, 2, 2)
    assert lib.fvmesh_create_uniform(lo, ln, 0, per, bc, C.byref(h)) == -3
    bad = (C.c_int * 6)(2, 2, 9, 2, 2, 2)
    assert lib.fvmesh_create_uniform(lo, ln, 2, per, bad, C.byref(h)) == -1
