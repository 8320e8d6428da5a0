"""ctypes mirrors of the structs and constants of ``include/fvgpu.h``."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

OK = 0
ERR_ARG = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_STATE = -4
ERR_NONFINITE = -5
ERR_EOS = -6
ERR_UNSUPPORTED = -7
ERR_MESH = -8
ERR_NODEVICE = -9
ERR_TIMEOUT = -10
ERROR_NAMES = {
    ERR_ARG: "FVGPU_ERR_ARG", ERR_CUDA: "FVGPU_ERR_CUDA", ERR_NOMEM: "FVGPU_ERR_NOMEM",
    ERR_STATE: "FVGPU_ERR_STATE", ERR_NONFINITE: "FVGPU_ERR_NONFINITE", ERR_EOS: "FVGPU_ERR_EOS",
    ERR_UNSUPPORTED: "FVGPU_ERR_UNSUPPORTED", ERR_MESH: "FVGPU_ERR_MESH",
    ERR_NODEVICE: "FVGPU_ERR_NODEVICE", ERR_TIMEOUT: "FVGPU_ERR_TIMEOUT",
}

FP64 = 0
MIXED = 1
FLAG_NO_BRICKS = 1
SCHEME_EULER = 1
SCHEME_SSPRK2 = 2
SCHEME_SSPRK3 = 3
SCHEMES = {"euler": SCHEME_EULER, "ssprk2": SCHEME_SSPRK2, "ssprk3": SCHEME_SSPRK3}
STAGES = {SCHEME_EULER: (1,), SCHEME_SSPRK2: (1, 4), SCHEME_SSPRK3: (1, 2, 3)}

FIELD_S = 0
FIELD_SN = 1
FIELD_RHS = 2
FIELD_SF = 3
FIELD_SG = 4
HANG0 = -16
KIND_NAMES = ("faceinterp", "gradcalc", "residual", "rk", "dt", "mixed_stage", "mixed_aux", "adjoint")
NKINDS = 8


class FvConfig(C.Structure):
    _fields_ = [("model", C.c_int), ("ns", C.c_int), ("ischeme", C.c_int), ("iprimtv", C.c_int),
                ("eos", C.c_int), ("precision", C.c_int), ("device", C.c_int),
                ("flags", C.c_int), ("gamma", C.c_double), ("pinf", C.c_double),
                ("visc", C.c_double), ("ymin", C.c_double), ("inflow", C.c_double * 8),
                ("reserved", C.c_double * 4)]


class FvMeshSoa(C.Structure):
    _fields_ = [("ncells", C.c_int64), ("nhang", C.c_int64)] + [
        (n, C.c_void_p) for n in ("nbr", "nbr_face", "area", "dcf", "dcc", "vol", "hang_nbr",
                                  "hang_area", "frames", "level")]


@dataclass
class SolverConfig:
    """Python form of ``fvgpu_config`` (CON / PAR fields the path reads)."""

    model: int = 1
    ns: int = 0
    ischeme: int = 2
    iprimtv: int = 0
    eos: int = 0
    precision: int = FP64
    device: int = 0
    flags: int = 0
    gamma: float = 1.4
    pinf: float = 0.0
    visc: float = 0.0
    ymin: float = 0.0
    inflow: tuple = field(default_factory=lambda: (0.0,) * 8)

    @property
    def neq(self) -> int:
        return 4 if self.model == 2 else 5

    def to_c(self) -> FvConfig:
        c = FvConfig()
        for n in ("model", "ns", "ischeme", "iprimtv", "eos", "precision", "device", "flags"):
            setattr(c, n, int(getattr(self, n)))
        for n in ("gamma", "pinf", "visc", "ymin"):
            setattr(c, n, float(getattr(self, n)))
        inflow = list(self.inflow) + [0.0] * (8 - len(self.inflow))
        for i in range(8):
            c.inflow[i] = float(inflow[i])
        return c


class MeshSoaHolder:
    """Keeps contiguous copies of a MeshTables alive behind an FvMeshSoa."""

    def __init__(self, t):
        def cont(a, dt):
            return np.ascontiguousarray(a, dtype=dt)

        self.arrays = {
            "nbr": cont(t.nbr, np.int32), "nbr_face": cont(t.nbr_face, np.int32),
            "area": cont(t.area, np.float64), "dcf": cont(t.dcf, np.float64),
            "dcc": cont(t.dcc, np.float64), "vol": cont(t.vol, np.float64),
            "hang_nbr": cont(t.hang_nbr if t.nhang else np.zeros((1, 4)), np.int32),
            "hang_area": cont(t.hang_area if t.nhang else np.zeros((1, 4)), np.float64),
            "frames": cont(t.frames, np.float64), "level": cont(t.level, np.int32),
        }
        self.soa = FvMeshSoa()
        self.soa.ncells = int(t.ncells)
        self.soa.nhang = int(t.nhang)
        for k, a in self.arrays.items():
            setattr(self.soa, k, a.ctypes.data)
        self.ncells = int(t.ncells)

# fvgpu_criterion kinds (criterionsplt.c)
CRIT_GRAD_RHO = 0
CRIT_RHO_BELOW = 1
CRIT_GRAD_RHO_H = 2


class FvLeaves(C.Structure):
    """fvgpu_leaves (include/fvgpu.h)."""
    _fields_ = [("ncells", C.c_int64), ("level", C.c_void_p), ("ijk", C.c_void_p), ("lo", C.c_double * 3),
                ("len", C.c_double * 3), ("periodic", C.c_int * 3), ("side_bc", C.c_int * 6)]
