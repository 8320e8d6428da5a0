"""ctypes front-ends for the oracle libraries (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()``, ``bench.py``'s CPU-baseline and
reference arms, and ``tests/golden/make_golden.py`` import this module.  The
product path (``fv_140823_gb300``) never does.

* :class:`RefHarness` drives ``oracle/_ref/libfvref.so``: the reference's own
  C sources, compiled unchanged, on BRANCH/CELL/LEAF objects built from the
  flattened tables (see ``oracle/ref_harness.c``).
* :class:`Oracle` drives ``oracle/_build/liboracle.so``: the C restatement of
  the same path on the flattened tables (``oracle/fvoracle.c``).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libfvref.so")
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
ORACLE_AD_LIB = os.path.join(HERE, "_build", "liboracle_ad.so")

# stage lists of the reference's RK(irk) cases (RK.c:16-47)
SCHEMES = {"ssprk3": (1, 2, 3), "ssprk2": (1, 4), "euler": (1,)}


@dataclass
class PhysConfig:
    """The CON / PAR fields the residual path reads (inputset.c:39-110)."""

    model: int = 1        # 1 ideal/stiffened gas, 2 barotropic liquid, 3 two-phase mixture
    ns: int = 0           # 1 = viscous fluxes
    ischeme: int = 2      # 1 first order, 2 MUSCL/minmod
    iprimtv: int = 0      # 1 = reconstruct primitive variables
    eos: int = 0          # 1 = viscous work term in the energy equation
    i_case: int = 0       # selects the inflow state of bc code 1 (bc_inlet.c)
    gamma: float = 1.4
    pinf: float = 0.0
    visc: float = 0.0
    ymin: float = 0.0
    dt: float = 1e-3

    @property
    def neq(self) -> int:
        return 4 if self.model == 2 else 5


class _RefCfg(C.Structure):
    _fields_ = [("model", C.c_int), ("ns", C.c_int), ("ischeme", C.c_int), ("iprimtv", C.c_int),
                ("neq", C.c_int), ("eos", C.c_int), ("i_case", C.c_int), ("pad", C.c_int),
                ("gamma", C.c_double), ("pinf", C.c_double), ("visc", C.c_double),
                ("ymin", C.c_double), ("dt", C.c_double)]


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def ref_available() -> bool:
    return os.path.isfile(REF_LIB)


class RefHarness:
    """The reference's own residual / RK code on a flattened mesh."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.isfile(REF_LIB):
                raise RuntimeError("oracle/_ref/libfvref.so is not built (reference tree absent?)")
            L = C.CDLL(REF_LIB)
            vp = C.c_void_p
            L.refh_create.restype = vp
            L.refh_create.argtypes = [vp, C.c_int64] + [vp] * 13
            L.refh_destroy.argtypes = [vp]
            L.refh_set_dt.argtypes = [vp, C.c_double]
            L.refh_set_state.argtypes = [vp, vp]
            L.refh_get.argtypes = [vp, C.c_int, vp]
            for n in ("refh_faceinterp", "refh_gradcalc", "refh_rhs"):
                getattr(L, n).argtypes = [vp]
            L.refh_rk.argtypes = [vp, C.c_int]
            L.refh_step.argtypes = [vp, vp, C.c_int]
            L.refh_conservation.argtypes = [vp, vp]
            L.refh_criterion.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
            L.refh_export.argtypes = [vp, C.c_int, C.c_int]
            L.refh_export.restype = C.c_int
            L.refh_geometry.argtypes = [vp, vp, vp, vp]
            cls._lib = L
        return cls._lib

    def __init__(self, tables, cfg: PhysConfig):
        L = self.lib()
        self.t = tables
        self.cfg = cfg
        self.n = tables.ncells
        self.neq = cfg.neq
        rc = _RefCfg(cfg.model, cfg.ns, cfg.ischeme, cfg.iprimtv, cfg.neq, cfg.eos, cfg.i_case, 0,
                     cfg.gamma, cfg.pinf, cfg.visc, cfg.ymin, cfg.dt)
        self._keep = [np.ascontiguousarray(x) for x in (
            tables.level, tables.ijk, tables.nbr, tables.nbr_face, tables.area, tables.vol,
            tables.centroid, tables.hang_nbr if tables.nhang else np.zeros((1, 4), np.int32),
            tables.hang_area if tables.nhang else np.zeros((1, 4)), tables.frames)]
        lo = (C.c_double * 3)(*tables.lo)
        ln = (C.c_double * 3)(*tables.length)
        per = (C.c_int * 3)(*tables.periodic)
        self._h = L.refh_create(C.byref(rc), self.n, *[_ptr(a) for a in self._keep], lo, ln, per)
        if not self._h:
            raise RuntimeError("refh_create failed")

    def close(self):
        if getattr(self, "_h", None):
            self.lib().refh_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_dt(self, dt: float):
        self.lib().refh_set_dt(self._h, float(dt))

    def set_state(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.shape == (self.neq, self.n)
        self.lib().refh_set_state(self._h, _ptr(U))

    def _get(self, which: int, shape) -> np.ndarray:
        out = np.empty(shape)
        self.lib().refh_get(self._h, which, _ptr(out))
        return out

    def state(self):
        return self._get(0, (self.neq, self.n))

    def state_n(self):
        return self._get(1, (self.neq, self.n))

    def rhs_array(self):
        return self._get(2, (self.neq, self.n))

    def sf(self):
        return self._get(3, (6, self.neq, self.n))

    def sg(self):
        return self._get(4, (self.neq + 1, 3, self.n))

    def faceinterp(self):
        self.lib().refh_faceinterp(self._h)

    def gradcalc(self):
        self.lib().refh_gradcalc(self._h)

    def rhs(self):
        self.lib().refh_rhs(self._h)

    def rk(self, irk: int):
        self.lib().refh_rk(self._h, int(irk))

    def residual(self, U: np.ndarray) -> np.ndarray:
        """RHS of the reference for state U (faceinterp / gradcalc as configured)."""
        self.set_state(U)
        if self.cfg.ischeme == 2:
            self.faceinterp()
        if self.cfg.ns == 1:
            self.gradcalc()
        self.rhs()
        return self.rhs_array()

    def step(self, scheme: str = "ssprk3", nsteps: int = 1):
        st = (C.c_int * len(SCHEMES[scheme]))(*SCHEMES[scheme])
        for _ in range(nsteps):
            self.lib().refh_step(self._h, st, len(SCHEMES[scheme]))

    def conservation(self) -> np.ndarray:
        out = np.empty(self.neq + 1)
        self.lib().refh_conservation(self._h, _ptr(out))
        return out

    def geometry(self):
        """The reference's own volume, face / sub-face areas and face frames of
        every leaf (meshproperties.c, normalvector.c, tagvector.c): vol [n],
        area [6][4][n], frames [6][9][n]."""
        vol = np.empty(self.n)
        area = np.empty((6, 4, self.n))
        frames = np.empty((6, 9, self.n))
        self.lib().refh_geometry(self._h, _ptr(vol), _ptr(area), _ptr(frames))
        return vol, area, frames

    def export(self, root_level: int, tstep: int, directory: str) -> str:
        """gradcalc + the reference's Tecplot writer (loop.c:50-55) on the
        current state; returns the path of field_linked<tstep>prt00.dat,
        written in `directory`."""
        cwd = os.getcwd()
        os.chdir(directory)
        try:
            rc = self.lib().refh_export(self._h, int(root_level), int(tstep))
        finally:
            os.chdir(cwd)
        if rc != 0:
            raise ValueError("a leaf is coarser than root_level")
        return os.path.join(directory, "field_linked%08dprt%02d.dat" % (tstep, 0))

    def criterion(self, i_case: int, level: int, geo_adapth: int = 0) -> np.ndarray:
        """criterionsplt.c flags of the leaves (gradients from the last gradcalc)."""
        out = np.empty(self.n, np.int32)
        self.lib().refh_criterion(self._h, int(i_case), int(geo_adapth), int(level), _ptr(out))
        return out


class Oracle:
    """The C restatement (oracle/fvoracle.c) on the flattened tables.

    Arrays are numpy, layouts U [neq][n], SF [6][neq][n], SG [neq+1][3][n]."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.isfile(ORACLE_LIB):
                raise RuntimeError("oracle/_build/liboracle.so is not built")
            L = C.CDLL(ORACLE_LIB)
            vp = C.c_void_p
            L.fvo_faceinterp.argtypes = [vp, vp, vp, vp]
            L.fvo_gradcalc.argtypes = [vp, vp, vp, vp]
            L.fvo_rhs.argtypes = [vp, vp, vp, vp, vp, vp]
            L.fvo_rhs_nb.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int]
            L.fvo_rk.argtypes = [C.c_int, C.c_double, C.c_int, vp, vp, vp, vp]
            L.fvo_step.argtypes = [vp, vp, vp, C.c_int, C.c_double, vp, vp, vp, vp, vp]
            L.fvo_conservation.argtypes = [C.c_int, vp, vp, vp]
            L.fvo_cell_lambda.argtypes = [vp, vp, vp, C.c_int64]
            L.fvo_cell_lambda.restype = C.c_double
            L.fvo_max_lambda.argtypes = [vp, vp, vp]
            L.fvo_max_lambda.restype = C.c_double
            L.fvo_error.argtypes = [C.POINTER(C.c_int64)]
            L.fvo_error.restype = C.c_int
            L.fvo_clear_error.argtypes = []
            L.fvo_set_threads.argtypes = [C.c_int]
            L.fvo_get_threads.restype = C.c_int
            cls._lib = L
        return cls._lib

    def __init__(self, tables, cfg):
        from fv_140823_gb300.abi import MeshSoaHolder
        self.L = self.lib()
        self.cfg = cfg
        self.ccfg = cfg.to_c()
        self.mesh = MeshSoaHolder(tables)
        self.n = tables.ncells
        self.neq = cfg.neq

    def _m(self):
        return C.byref(self.mesh.soa)

    def _c(self):
        return C.byref(self.ccfg)

    @classmethod
    def set_threads(cls, n: int):
        cls.lib().fvo_set_threads(int(n))

    @classmethod
    def threads(cls) -> int:
        return cls.lib().fvo_get_threads()

    def error(self):
        cell = C.c_int64()
        code = self.L.fvo_error(C.byref(cell))
        self.L.fvo_clear_error()
        return code, cell.value

    def faceinterp(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        SF = np.zeros((6, self.neq, self.n))
        self.L.fvo_faceinterp(self._c(), self._m(), _ptr(U), _ptr(SF))
        return SF

    def gradcalc(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        SG = np.zeros((self.neq + 1, 3, self.n))
        self.L.fvo_gradcalc(self._c(), self._m(), _ptr(U), _ptr(SG))
        return SG

    def rhs(self, U, SF=None, SG=None, inner=None, inner_outer=0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        SF = np.zeros((6, self.neq, self.n)) if SF is None else np.ascontiguousarray(SF)
        SG = np.zeros((self.neq + 1, 3, self.n)) if SG is None else np.ascontiguousarray(SG)
        R = np.zeros((self.neq, self.n))
        if inner is None:
            self.L.fvo_rhs(self._c(), self._m(), _ptr(U), _ptr(SF), _ptr(SG), _ptr(R))
        else:
            inner = np.ascontiguousarray(inner, dtype=np.int32)
            self.L.fvo_rhs_nb(self._c(), self._m(), _ptr(U), _ptr(SF), _ptr(SG), _ptr(R),
                              _ptr(inner), int(inner_outer))
        return R

    def residual(self, U):
        """faceinterp / gradcalc as configured, then RHS."""
        SF = self.faceinterp(U) if self.cfg.ischeme == 2 else None
        SG = self.gradcalc(U) if self.cfg.ns == 1 else None
        return self.rhs(U, SF, SG)

    def step(self, U, dt, scheme="ssprk3", nsteps=1):
        S = np.array(U, dtype=np.float64, copy=True, order="C")
        SN = np.zeros_like(S)
        SF = np.zeros((6, self.neq, self.n))
        SG = np.zeros((self.neq + 1, 3, self.n))
        R = np.zeros_like(S)
        st = (C.c_int * len(SCHEMES[scheme]))(*SCHEMES[scheme])
        for _ in range(nsteps):
            self.L.fvo_step(self._c(), self._m(), st, len(SCHEMES[scheme]), float(dt), _ptr(S),
                            _ptr(SN), _ptr(SF), _ptr(SG), _ptr(R))
        return S

    def rk(self, irk, dt, S, SN, R):
        """In-place RK(irk) on numpy arrays S, SN given RHS R."""
        self.L.fvo_rk(int(irk), float(dt), self.neq, self._m(), _ptr(S), _ptr(SN), _ptr(R))

    def conservation(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        out = np.empty(self.neq + 1)
        self.L.fvo_conservation(self.neq, self._m(), _ptr(U), _ptr(out))
        return out

    def max_lambda(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        return self.L.fvo_max_lambda(self._c(), self._m(), _ptr(U))

    def cfl_dt(self, U, cfl):
        return cfl / self.max_lambda(U)


class OracleAD:
    """Forward-mode (dual number) restatement: exact JVPs of the residual and
    of RK steps (oracle/fvoracle_ad.cpp), model 1, inviscid."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.isfile(ORACLE_AD_LIB):
                raise RuntimeError("oracle/_build/liboracle_ad.so is not built")
            L = C.CDLL(ORACLE_AD_LIB)
            vp = C.c_void_p
            L.fvo_ad_residual.argtypes = [vp, vp, vp, vp]
            L.fvo_ad_jvp.argtypes = [vp, vp, vp, vp, vp, vp]
            L.fvo_ad_steps_jvp.argtypes = [vp, vp, vp, C.c_int, C.c_double, C.c_int, vp, vp, vp, vp]
            L.fvo_ad_count_steps.argtypes = [vp, vp, vp, C.c_int, C.c_double, C.c_int, vp, vp]
            L.fvo_ad_count_stage.argtypes = [vp, vp, C.c_int, C.c_double, vp, vp]
            cls._lib = L
        return cls._lib

    def __init__(self, tables, cfg):
        from fv_140823_gb300.abi import MeshSoaHolder
        self.L = self.lib()
        self.cfg = cfg
        self.ccfg = cfg.to_c()
        self.mesh = MeshSoaHolder(tables)
        self.n = tables.ncells

    def residual(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty_like(U)
        assert self.L.fvo_ad_residual(C.byref(self.ccfg), C.byref(self.mesh.soa), _ptr(U), _ptr(R)) == 0
        return R

    def jvp(self, U, V):
        U = np.ascontiguousarray(U, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        R = np.empty_like(U)
        JV = np.empty_like(U)
        assert self.L.fvo_ad_jvp(C.byref(self.ccfg), C.byref(self.mesh.soa), _ptr(U), _ptr(V), _ptr(R),
                                 _ptr(JV)) == 0
        return R, JV

    def steps_jvp(self, U, V, dt, scheme="ssprk3", nsteps=1):
        U = np.ascontiguousarray(U, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        S = np.empty_like(U)
        JV = np.empty_like(U)
        st = (C.c_int * len(SCHEMES[scheme]))(*SCHEMES[scheme])
        assert self.L.fvo_ad_steps_jvp(C.byref(self.ccfg), C.byref(self.mesh.soa), st, len(SCHEMES[scheme]),
                                       float(dt), int(nsteps), _ptr(U), _ptr(V), _ptr(S), _ptr(JV)) == 0
        return S, JV

    def count_steps(self, U, dt, scheme="ssprk3", nsteps=1):
        """FP64 operations of nsteps steps: (add/sub, mul, div, sqrt)."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        out = np.zeros(4, np.uint64)
        st = (C.c_int * len(SCHEMES[scheme]))(*SCHEMES[scheme])
        assert self.L.fvo_ad_count_steps(C.byref(self.ccfg), C.byref(self.mesh.soa), st, len(SCHEMES[scheme]),
                                         float(dt), int(nsteps), _ptr(U), out.ctypes.data) == 0
        return out

    def count_stage(self, U, irk, dt):
        """FP64 operations of one stage: (faceinterp, residual + RK(irk)),
        each (add/sub, mul, div, sqrt)."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        out = np.zeros(8, np.uint64)
        assert self.L.fvo_ad_count_stage(C.byref(self.ccfg), C.byref(self.mesh.soa), int(irk), float(dt), _ptr(U),
                                         out.ctypes.data) == 0
        return out[:4], out[4:]


def criterion(U, SG, vol, kind, threshold, level_hi):
    """Refinement flags, criterionsplt.c:24-86 (restated; i_case 204 is
    |grad rho| > threshold, i_case 2500 is rho < threshold; kind 2 scales
    |grad rho| by the cell size V^(1/3)).  SG: gradcalc output [neq+1][3][n]."""
    g = SG[0]
    mag = np.sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2])
    if kind == 1:
        hit = U[0] < threshold
    else:
        if kind == 2:
            mag = mag * np.cbrt(vol)
        hit = mag > threshold
    return np.where(hit, level_hi, 1).astype(np.int32)
