"""Python view of the host octree mesh builder (``include/fvmesh.h``).

The reference's host keeps its forest of octrees and, in the GB300 design,
flattens the leaves after every adaptation into structure-of-arrays tables
that stay resident on the device.  :class:`OctreeMesh` drives the C++
builder; :meth:`OctreeMesh.flatten` returns those tables as numpy arrays
(:class:`MeshTables`), which is exactly what ``fvgpu_upload_mesh`` takes.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._native import load_mesh_lib

BC_INFLOW = 1
BC_TRANSMISSIVE = 2
BC_REFLECTIVE = 3
BC_NOSLIP = 4
HANG0 = -16
# face f: 0=-y 1=+x 2=+y 3=-x 4=-z 5=+z ; opposite face of f
FACE_AXIS = (1, 0, 1, 0, 2, 2)
FACE_SIGN = (-1, 1, 1, -1, -1, 1)
FACE_OPP = (2, 3, 0, 1, 5, 4)


class _Tables(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "level", "ijk", "nbr", "nbr_face", "area", "dcf", "dcc", "vol", "centroid",
        "hang_nbr", "hang_area", "hang_cell", "hang_face", "frames")]


@dataclass
class MeshTables:
    """Flattened mesh: ``[face][cell]`` arrays are shaped ``(6, ncells)``."""

    ncells: int
    nhang: int
    level: np.ndarray      # (n,) int32
    ijk: np.ndarray        # (3, n) int32
    nbr: np.ndarray        # (6, n) int32 neighbour code
    nbr_face: np.ndarray   # (6, n) int32
    area: np.ndarray       # (6, n) f64
    dcf: np.ndarray        # (6, n) f64
    dcc: np.ndarray        # (6, n) f64
    vol: np.ndarray        # (n,) f64
    centroid: np.ndarray   # (3, n) f64
    hang_nbr: np.ndarray   # (nhang, 4) int32
    hang_area: np.ndarray  # (nhang, 4) f64
    hang_cell: np.ndarray  # (nhang,) int32
    hang_face: np.ndarray  # (nhang,) int32
    frames: np.ndarray     # (6, 9) f64
    lo: tuple
    length: tuple
    periodic: tuple
    side_bc: tuple


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class OctreeMesh:
    """Axis-aligned 2:1-balanced octree over a box, leaves in Morton order."""

    def __init__(self, lo=(0.0, 0.0, 0.0), length=(1.0, 1.0, 1.0), base_level: int = 3,
                 periodic=(0, 0, 0), side_bc=(BC_TRANSMISSIVE,) * 6):
        self._lib = load_mesh_lib()
        self._h = C.c_void_p()
        lo_a = (C.c_double * 3)(*lo)
        len_a = (C.c_double * 3)(*length)
        per_a = (C.c_int * 3)(*[int(bool(p)) for p in periodic])
        bc_a = (C.c_int * 6)(*side_bc)
        rc = self._lib.fvmesh_create_uniform(lo_a, len_a, int(base_level), per_a, bc_a,
                                             C.byref(self._h))
        self._check(rc)
        self.lo = tuple(float(x) for x in lo)
        self.length = tuple(float(x) for x in length)
        self.periodic = tuple(int(bool(p)) for p in periodic)
        self.side_bc = tuple(int(b) for b in side_bc)

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise RuntimeError(f"fvmesh error {rc}: {self._lib.fvmesh_last_error().decode()}")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.fvmesh_destroy(h)
            self._h = C.c_void_p()

    def sizes(self) -> tuple[int, int]:
        n = C.c_int64()
        nh = C.c_int64()
        self._check(self._lib.fvmesh_sizes(self._h, C.byref(n), C.byref(nh)))
        return n.value, nh.value

    @property
    def ncells(self) -> int:
        return self.sizes()[0]

    def leaves(self) -> tuple[np.ndarray, np.ndarray]:
        n, _ = self.sizes()
        level = np.empty(n, np.int32)
        cen = np.empty((3, n), np.float64)
        self._check(self._lib.fvmesh_leaves(self._h, C.c_void_p(_p(level)), C.c_void_p(_p(cen))))
        return level, cen

    def leaf_cells(self) -> tuple[np.ndarray, np.ndarray]:
        """Leaf levels (n,) and lattice positions (3, n), Morton order: the
        leaf list :meth:`Solver.upload_leaves` flattens on the device."""
        n, _ = self.sizes()
        level = np.empty(n, np.int32)
        ijk = np.empty((3, n), np.int32)
        self._check(self._lib.fvmesh_leaf_cells(self._h, C.c_void_p(_p(level)), C.c_void_p(_p(ijk))))
        return level, ijk

    def refine(self, flags, max_level: int) -> None:
        f = np.ascontiguousarray(np.asarray(flags, dtype=np.uint8))
        if f.shape != (self.ncells,):
            raise ValueError("flags must have one entry per leaf")
        self._check(self._lib.fvmesh_refine(self._h, C.c_void_p(_p(f)), int(max_level)))

    def adapt(self, split, min_level: int, max_level: int) -> None:
        """One adaptation pass toward the per-leaf target levels `split`
        (``fvmesh_adapt``: one level per pass, sibling merges, 2:1 balance)."""
        sp = np.ascontiguousarray(np.asarray(split, dtype=np.int32))
        if sp.shape != (self.ncells,):
            raise ValueError("split must have one entry per leaf")
        self._check(self._lib.fvmesh_adapt(self._h, C.c_void_p(_p(sp)), int(min_level), int(max_level)))

    def transfer(self, S_old: np.ndarray) -> np.ndarray:
        """State [neq][n_old] on the leaves before the last :meth:`adapt` ->
        state on the current leaves (children inherit, merged parents average)."""
        S_old = np.ascontiguousarray(S_old, dtype=np.float64)
        neq, n_old = S_old.shape
        S_new = np.empty((neq, self.ncells))
        self._check(self._lib.fvmesh_transfer(self._h, int(neq), C.c_int64(n_old), C.c_void_p(_p(S_old)),
                                              C.c_void_p(_p(S_new))))
        return S_new

    def cell_nodes(self, level: int, i: int, j: int, k: int) -> np.ndarray:
        out = np.empty((8, 3), np.float64)
        self._check(self._lib.fvmesh_cell_nodes(self._h, level, i, j, k, C.c_void_p(_p(out))))
        return out

    def flatten(self) -> MeshTables:
        n, nh = self.sizes()
        t = MeshTables(
            ncells=n, nhang=nh,
            level=np.empty(n, np.int32), ijk=np.empty((3, n), np.int32),
            nbr=np.empty((6, n), np.int32), nbr_face=np.empty((6, n), np.int32),
            area=np.empty((6, n)), dcf=np.empty((6, n)), dcc=np.empty((6, n)),
            vol=np.empty(n), centroid=np.empty((3, n)),
            hang_nbr=np.empty((max(nh, 1), 4), np.int32)[:nh],
            hang_area=np.empty((max(nh, 1), 4))[:nh],
            hang_cell=np.empty(max(nh, 1), np.int32)[:nh],
            hang_face=np.empty(max(nh, 1), np.int32)[:nh],
            frames=np.empty((6, 9)),
            lo=self.lo, length=self.length, periodic=self.periodic, side_bc=self.side_bc)
        ct = _Tables(*[C.c_void_p(_p(getattr(t, name))) for name, _ in _Tables._fields_])
        self._check(self._lib.fvmesh_flatten(self._h, C.byref(ct)))
        return t


def uniform_mesh(level: int, lo=(0.0, 0.0, 0.0), length=(1.0, 1.0, 1.0), periodic=(0, 0, 0),
                 side_bc=(BC_TRANSMISSIVE,) * 6) -> OctreeMesh:
    return OctreeMesh(lo, length, level, periodic, side_bc)


def refine_by(mesh: OctreeMesh, predicate, max_level: int, passes: int | None = None) -> OctreeMesh:
    """Refine repeatedly: each pass flags leaves where predicate(level, centroid)
    is true (vectorised over leaves), until max_level or no flags remain."""
    for _ in range(passes if passes is not None else 32):
        level, cen = mesh.leaves()
        flags = np.asarray(predicate(level, cen), dtype=bool) & (level < max_level)
        if not flags.any():
            break
        mesh.refine(flags.astype(np.uint8), max_level)
    return mesh


__all__ = ["OctreeMesh", "MeshTables", "uniform_mesh", "refine_by", "BC_INFLOW",
           "BC_TRANSMISSIVE", "BC_REFLECTIVE", "BC_NOSLIP", "HANG0", "FACE_AXIS", "FACE_SIGN",
           "FACE_OPP"]
