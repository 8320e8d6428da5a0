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
        lib.fvmesh_leaf_cells.argtypes = [vp, vp, vp]
        lib.fvmesh_refine.argtypes = [vp, vp, C.c_int]
        lib.fvmesh_adapt.argtypes = [vp, vp, C.c_int, C.c_int]
        lib.fvmesh_transfer.argtypes = [vp, C.c_int, C.c_int64, vp, vp]
        lib.fvmesh_flatten.argtypes = [vp, vp]
        lib.fvmesh_cell_nodes.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]
        lib.fvmesh_domain.argtypes = [vp, vp, vp, vp, vp]
        lib.fvmesh_last_error.argtypes = []
        lib.fvmesh_last_error.restype = C.c_char_p
        lib.fvmesh_export_tecplot.argtypes = [vp, C.c_int64, vp, vp, vp, vp, C.c_int64, vp, vp, vp, vp,
                                              C.c_char_p]
        lib.fvmesh_export_tecplot.restype = C.c_int
        lib.fvmesh_export_last_error.argtypes = []
        lib.fvmesh_export_last_error.restype = C.c_char_p
        lib._fv_typed = True
    return lib


# Every entry point declared in include/fvgpu.h, with its ctypes signature.
_GPU_SIGS = {
    "fvgpu_create": ([C.c_void_p, C.POINTER(C.c_void_p)], C.c_int),
    "fvgpu_destroy": ([C.c_void_p], C.c_int),
    "fvgpu_set_precision": ([C.c_void_p, C.c_int], C.c_int),
    "fvgpu_upload_mesh": ([C.c_void_p, C.c_void_p], C.c_int),
    "fvgpu_upload_state": ([C.c_void_p, C.c_void_p, C.c_int64], C.c_int),
    "fvgpu_download_state": ([C.c_void_p, C.c_void_p, C.c_int64], C.c_int),
    "fvgpu_download": ([C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "fvgpu_faceinterp": ([C.c_void_p], C.c_int),
    "fvgpu_gradcalc": ([C.c_void_p], C.c_int),
    "fvgpu_rhs": ([C.c_void_p], C.c_int),
    "fvgpu_set_inner": ([C.c_void_p, C.c_void_p], C.c_int),
    "fvgpu_rhs_nb": ([C.c_void_p, C.c_int], C.c_int),
    "fvgpu_rk": ([C.c_void_p, C.c_int, C.c_double], C.c_int),
    "fvgpu_step": ([C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int], C.c_int),
    "fvgpu_compute_dt": ([C.c_void_p, C.c_double, C.POINTER(C.c_double)], C.c_int),
    "fvgpu_conservation": ([C.c_void_p, C.c_void_p], C.c_int),
    "fvgpu_residual_vjp": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64], C.c_int),
    "fvgpu_upload_leaves": ([C.c_void_p, C.c_void_p], C.c_int),
    "fvgpu_checkpoint_save": ([C.c_void_p, C.c_char_p, C.c_double, C.c_int64], C.c_int),
    "fvgpu_checkpoint_load": ([C.c_void_p, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)], C.c_int),
    "fvgpu_checkpoint_write": ([C.c_char_p, C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double, C.c_int64],
                               C.c_int),
    "fvgpu_checkpoint_read": ([C.c_char_p, C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.POINTER(C.c_double),
                               C.POINTER(C.c_int64)], C.c_int),
    "fvgpu_mesh_signature": ([C.c_void_p, C.POINTER(C.c_uint64)], C.c_int),
    "fvgpu_criterion": ([C.c_void_p, C.c_int, C.c_double, C.c_int32, C.c_void_p], C.c_int),
    "fvgpu_measure_fp64": ([C.c_int, C.POINTER(C.c_double)], C.c_int),
    "fvgpu_halo_set": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64], C.c_int),
    "fvgpu_halo_pack": ([C.c_void_p, C.c_void_p], C.c_int),
    "fvgpu_halo_unpack": ([C.c_void_p, C.c_void_p], C.c_int),
    "fvgpu_residual_vjp_device": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "fvgpu_adjoint_steps": ([C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_int64],
                            C.c_int),
    "fvgpu_profile_adjoint": ([C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "fvgpu_last_error": ([C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int64), C.c_char_p, C.c_int],
                         C.c_int),
    "fvgpu_neq": ([C.c_void_p], C.c_int),
    "fvgpu_synchronize": ([C.c_void_p], C.c_int),
    "fvgpu_profile_step": ([C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p],
                           C.c_int),
    "fvgpu_get_stream": ([C.c_void_p, C.POINTER(C.c_void_p)], C.c_int),
    "fvgpu_conservation_noalloc": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p],
                                   C.c_int),
}


def gpu_symbols() -> list[str]:
    return list(_GPU_SIGS)


def load_gpu_lib() -> C.CDLL:
    lib = _load("libfvgpu.so")
    if not getattr(lib, "_fv_typed", False):
        for name, (args, res) in _GPU_SIGS.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = res
        lib._fv_typed = True
    return lib
