"""Tecplot export of the leaf field, as the reference writes it.

The reference's time loop exports every ``exstep`` steps with ``gradcalc``
followed by ``exportfield_linked_V3`` (loop.c:50-55): one FEPOINT zone of
BRICK elements whose points are node links shared between leaves, carrying
link means of the conserved variables, the pressure and four gradient
magnitudes (exportfield_linked_V3.c:19-572).  Here the field lives on the
GPU: :func:`export_solver` runs the gradients on the device
(``fvgpu_gradcalc``), downloads the state and the gradients, and hands them to
the host writer in libfvmesh (``fvmesh_export_tecplot``), which forms the
links in the reference's order and prints with its formats, so the file has
the reference's bytes for the same leaves and field.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._native import load_mesh_lib


class _TecplotCfg(C.Structure):
    _fields_ = [("model", C.c_int), ("neq", C.c_int), ("root_level", C.c_int), ("pad", C.c_int),
                ("gamma", C.c_double), ("pinf", C.c_double)]


def file_name(tstep: int) -> str:
    """The reference's file name for step `tstep` (rank 0 writes for all)."""
    return "field_linked%08dprt%02d.dat" % (int(tstep), 0)


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def write_field_linked(path: str, tables, S: np.ndarray, SG: np.ndarray | None, *, model: int, gamma: float,
                       pinf: float, root_level: int | None = None) -> str:
    """Write the file for leaf field S [neq][n] and gradients SG [neq+1][3][n]
    (None: zero gradients) on the flattened mesh `tables`.  The trees of the
    "iel" column are the cells of level `root_level` (default: the coarsest
    leaf level) in Morton order."""
    lib = load_mesh_lib()
    n = int(tables.ncells)
    neq = 4 if model == 2 else 5
    S = np.ascontiguousarray(S, dtype=np.float64)
    if S.shape != (neq, n):
        raise ValueError(f"S must be ({neq}, {n})")
    if SG is not None:
        SG = np.ascontiguousarray(SG, dtype=np.float64)
        if SG.shape != (neq + 1, 3, n):
            raise ValueError(f"SG must be ({neq + 1}, 3, {n})")
    level = np.ascontiguousarray(tables.level, dtype=np.int32)
    rl = int(level.min()) if root_level is None else int(root_level)
    cfg = _TecplotCfg(int(model), neq, rl, 0, float(gamma), float(pinf))
    ijk = np.ascontiguousarray(tables.ijk, dtype=np.int32)
    nbr = np.ascontiguousarray(tables.nbr, dtype=np.int32)
    nh = int(tables.nhang)
    hang = np.ascontiguousarray(tables.hang_nbr if nh else np.zeros((1, 4)), dtype=np.int32)
    lo = np.ascontiguousarray(tables.lo, dtype=np.float64)
    ln = np.ascontiguousarray(tables.length, dtype=np.float64)
    rc = lib.fvmesh_export_tecplot(C.byref(cfg), n, _ptr(level), _ptr(ijk), _ptr(nbr), _ptr(hang), nh, _ptr(lo),
                                   _ptr(ln), _ptr(S), _ptr(SG) if SG is not None else None,
                                   os.fsencode(path))
    if rc != 0:
        raise RuntimeError(f"fvmesh_export_tecplot: {lib.fvmesh_export_last_error().decode()}")
    return path


def export_solver(solver, tables, directory: str, tstep: int, root_level: int | None = None) -> str:
    """loop.c:50-55 on a device-resident run: gradients of the current state
    on the GPU, state and gradients downloaded, file written on the host as
    `directory`/field_linked<tstep>prt00.dat."""
    solver.gradcalc()
    S = solver.state()
    SG = solver.sg()
    cfg = solver.cfg
    return write_field_linked(os.path.join(directory, file_name(tstep)), tables, S, SG, model=cfg.model,
                              gamma=cfg.gamma, pinf=cfg.pinf, root_level=root_level)
