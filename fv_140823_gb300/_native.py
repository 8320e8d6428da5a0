"""Loading of the in-tree native libraries (ctypes).

A missing library is an error: there is no Python or CPU fallback for any
entry point of the package.  Build with ``__graft_entry__.build()`` or
``python -m fv_140823_gb300._build``.
"""
from __future__ import annotations

import ctypes as C
import os

_LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
_cache: dict[str, C.CDLL] = {}


def lib_path(name: str) -> str:
    return os.path.join(_LIB_DIR, name)


def _load(name: str) -> C.CDLL:
    if name in _cache:
        return _cache[name]
    path = lib_path(name)
    if not os.path.isfile(path):
        raise RuntimeError(f"{name} is not built ({path} missing); run __graft_entry__.build()")
    lib = C.CDLL(path)
    _cache[name] = lib
    return lib


def load_mesh_lib() -> C.CDLL:
    lib = _load("libfvmesh.so")
    if not getattr(lib, "_fv_typed", False):
        vp, i64p = C.c_void_p, C.POINTER(C.c_int64)
        lib.fvmesh_create_uniform.argtypes = [vp, vp, C.c_int, vp, vp, C.POINTER(C.c_void_p)]
        lib.fvmesh_create_uniform.restype = C.c_int
        lib.fvmesh_destroy.argtypes = [vp]
        lib.fvmesh_destroy.restype = None
        lib.fvmesh_sizes.argtypes = [vp, i64p, i64p]
        lib.fvmesh_leaves.argtypes = [vp, vp, vp]
        lib.fvmesh_refine.argtypes = [vp, vp, C.c_int]
        lib.fvmesh_flatten.argtypes = [vp, vp]
        lib.fvmesh_cell_nodes.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]
        lib.fvmesh_domain.argtypes = [vp, vp, vp, vp, vp]
        lib.fvmesh_last_error.argtypes = []
        lib.fvmesh_last_error.restype = C.c_char_p
        lib._fv_typed = True
    return lib
