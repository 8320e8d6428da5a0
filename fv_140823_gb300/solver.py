"""Host-side mirror of the reference's residual / RK interface over libfvgpu.

The reference drives the hot path with ``void`` calls on its global run
structure (``RHS(run)``, ``RHS_nb(run, inner)``, ``RK(irk, run)``,
``faceinterp(run)``, ``gradcalc(run)``; strdata.h:642-656).  :class:`Solver`
keeps those names and their meaning on a device-resident state:

    s = Solver(tables, SolverConfig(...))
    s.set_state(U)            # LEAF.S of every leaf
    s.faceinterp(); s.rhs()   # faceinterp(run); RHS(run)
    s.rk(1, dt)               # RK(1, run)
    s.step("ssprk3", dt=dt, nsteps=100)   # the missing advancetimeexplicit

Where the reference prints a message and calls ``exit(0)`` (a NaN residual,
an EOS without a root, HLLC wave speeds that are not finite), these methods
raise :class:`FvGpuError` carrying the library's error code and offending cell.
There is no CPU fallback: without the CUDA library or a GPU every call fails.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._native import load_gpu_lib


class FvGpuError(RuntimeError):
    def __init__(self, code: int, cell: int, msg: str):
        super().__init__(f"{abi.ERROR_NAMES.get(code, code)}: {msg}" + (f" (cell {cell})" if cell >= 0 else ""))
        self.code = code
        self.cell = cell


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Solver:
    """One libfvgpu context with a resident mesh."""

    def __init__(self, tables, cfg: abi.SolverConfig | None = None):
        self.lib = load_gpu_lib()
        self.cfg = cfg or abi.SolverConfig()
        self._ccfg = self.cfg.to_c()
        self._ctx = C.c_void_p()
        rc = self.lib.fvgpu_create(C.byref(self._ccfg), C.byref(self._ctx))
        if rc != 0:
            self._raise(rc, ctx=None)
        self.neq = self.lib.fvgpu_neq(self._ctx)
        self.n = 0
        if tables is not None:
            self.upload_mesh(tables)

    # -- plumbing ---------------------------------------------------------
    def _raise(self, rc: int, ctx="self"):
        code = C.c_int()
        cell = C.c_int64()
        buf = C.create_string_buffer(512)
        self.lib.fvgpu_last_error(self._ctx if ctx == "self" else None, C.byref(code), C.byref(cell), buf, 512)
        raise FvGpuError(rc, cell.value, buf.value.decode(errors="replace"))

    def _call(self, name: str, *args):
        rc = getattr(self.lib, name)(self._ctx, *args)
        if rc != 0:
            self._raise(rc)
        return rc

    def close(self):
        if getattr(self, "_ctx", None) is not None and self._ctx.value:
            self.lib.fvgpu_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- data --------------------------------------------------------------
    def upload_mesh(self, tables):
        self._mesh = abi.MeshSoaHolder(tables)
        self._call("fvgpu_upload_mesh", C.byref(self._mesh.soa))
        self.n = tables.ncells

    def set_precision(self, precision: int):
        self._call("fvgpu_set_precision", int(precision))
        self.cfg.precision = int(precision)

    def set_state(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != (self.neq, self.n):
            raise ValueError(f"state must be ({self.neq}, {self.n})")
        self._call("fvgpu_upload_state", _ptr(U), C.c_int64(self.n))
        self.synchronize()

    def state(self) -> np.ndarray:
        out = np.empty((self.neq, self.n))
        self._call("fvgpu_download_state", _ptr(out), C.c_int64(self.n))
        return out

    def download(self, field: int) -> np.ndarray:
        shapes = {abi.FIELD_S: (self.neq, self.n), abi.FIELD_SN: (self.neq, self.n),
                  abi.FIELD_RHS: (self.neq, self.n), abi.FIELD_SF: (6, self.neq, self.n),
                  abi.FIELD_SG: (self.neq + 1, 3, self.n)}
        out = np.empty(shapes[field])
        self._call("fvgpu_download", int(field), _ptr(out))
        return out

    def rhs_array(self) -> np.ndarray:
        return self.download(abi.FIELD_RHS)

    def sf(self) -> np.ndarray:
        return self.download(abi.FIELD_SF)

    def sg(self) -> np.ndarray:
        return self.download(abi.FIELD_SG)

    def state_n(self) -> np.ndarray:
        return self.download(abi.FIELD_SN)

    # -- the reference's calls ------------------------------------------
    def faceinterp(self):
        self._call("fvgpu_faceinterp")

    def gradcalc(self):
        self._call("fvgpu_gradcalc")

    def rhs(self):
        self._call("fvgpu_rhs")

    def set_inner(self, inner):
        inner = np.ascontiguousarray(inner, dtype=np.int32)
        self._call("fvgpu_set_inner", _ptr(inner))

    def rhs_nb(self, inner_outer: int):
        self._call("fvgpu_rhs_nb", int(inner_outer))

    def rk(self, irk: int, dt: float):
        self._call("fvgpu_rk", int(irk), float(dt))

    def residual(self, U: np.ndarray | None = None) -> np.ndarray:
        """faceinterp / gradcalc as configured, RHS, and download."""
        if U is not None:
            self.set_state(U)
        if self.cfg.ischeme == 2:
            self.faceinterp()
        if self.cfg.ns == 1:
            self.gradcalc()
        self.rhs()
        return self.rhs_array()

    # -- time stepping and reductions --------------------------------------
    def step(self, scheme="ssprk3", dt: float = 0.0, cfl: float = 0.0, nsteps: int = 1):
        sc = abi.SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        self._call("fvgpu_step", sc, float(dt), float(cfl), int(nsteps))

    def compute_dt(self, cfl: float) -> float:
        out = C.c_double()
        self._call("fvgpu_compute_dt", float(cfl), C.byref(out))
        return out.value

    def conservation(self) -> np.ndarray:
        out = np.empty(self.neq + 1)
        self._call("fvgpu_conservation", _ptr(out))
        return out

    def upload_leaves(self, level: np.ndarray, ijk: np.ndarray, lo, length, periodic, side_bc):
        """Build the mesh tables on the GPU from the Morton-sorted leaf list
        (fvgpu_upload_leaves): bit-identical to the host flattener's tables."""
        self._leaf_level = np.ascontiguousarray(level, dtype=np.int32)
        self._leaf_ijk = np.ascontiguousarray(ijk, dtype=np.int32)
        lv = abi.FvLeaves(self._leaf_level.size, _ptr(self._leaf_level).value, _ptr(self._leaf_ijk).value,
                          (C.c_double * 3)(*lo), (C.c_double * 3)(*length), (C.c_int * 3)(*periodic),
                          (C.c_int * 6)(*side_bc))
        self._call("fvgpu_upload_leaves", C.byref(lv))
        self.n = int(self._leaf_level.size)

    @classmethod
    def from_leaves(cls, tables, cfg: abi.SolverConfig | None = None) -> "Solver":
        """A context whose tables are flattened on the device from `tables`'
        leaf list (level, ijk and the box)."""
        s = cls(None, cfg)
        s.upload_leaves(tables.level, tables.ijk, tables.lo, tables.length, tables.periodic, tables.side_bc)
        return s

    # -- restart and adaptation helpers ------------------------------------------
    def checkpoint_save(self, path: str, time: float = 0.0, step: int = 0):
        """Bit-exact binary restart file of the state (fvgpu_checkpoint_save)."""
        self._call("fvgpu_checkpoint_save", str(path).encode(), float(time), C.c_int64(step))

    def checkpoint_load(self, path: str) -> tuple[float, int]:
        t, st = C.c_double(), C.c_int64()
        self._call("fvgpu_checkpoint_load", str(path).encode(), C.byref(t), C.byref(st))
        return t.value, st.value

    def mesh_signature(self) -> int:
        out = C.c_uint64()
        self._call("fvgpu_mesh_signature", C.byref(out))
        return out.value

    def criterion(self, kind: int, threshold: float, level_hi: int) -> np.ndarray:
        """Refinement flags of criterionsplt.c (abi.CRIT_*)."""
        out = np.empty(self.n, np.int32)
        self._call("fvgpu_criterion", int(kind), float(threshold), C.c_int32(level_hi), _ptr(out))
        return out

    # -- halo exchange -------------------------------------------------------
    def halo_set(self, send_cells: np.ndarray, recv_cells: np.ndarray):
        """Local cells this rank packs for others / receives into (ghosts)."""
        self._halo_send = np.ascontiguousarray(send_cells, dtype=np.int32)
        self._halo_recv = np.ascontiguousarray(recv_cells, dtype=np.int32)
        self._call("fvgpu_halo_set", _ptr(self._halo_send), C.c_int64(self._halo_send.size),
                   _ptr(self._halo_recv), C.c_int64(self._halo_recv.size))

    def halo_pack(self, send_ptr: int):
        """Gather the send cells' state into a device buffer [neq][nsend]."""
        self._call("fvgpu_halo_pack", C.c_void_p(send_ptr))

    def halo_unpack(self, recv_ptr: int):
        """Scatter a device buffer [neq][nrecv] into the ghost cells."""
        self._call("fvgpu_halo_unpack", C.c_void_p(recv_ptr))

    # -- adjoint -------------------------------------------------------------
    def residual_vjp(self, w: np.ndarray) -> np.ndarray:
        """(dR/dU)^T w at the current state (FP64 residual)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        if w.shape != (self.neq, self.n):
            raise ValueError(f"w must have shape {(self.neq, self.n)}")
        out = np.empty((self.neq, self.n))
        self._call("fvgpu_residual_vjp", _ptr(w), _ptr(out), C.c_int64(self.n))
        return out

    def residual_vjp_device(self, w_ptr: int, out_ptr: int):
        """(dR/dU)^T w on caller-owned device arrays [neq][ncells], queued on
        the context's stream (:meth:`stream_handle`)."""
        self._call("fvgpu_residual_vjp_device", C.c_void_p(w_ptr), C.c_void_p(out_ptr))

    def adjoint_steps(self, gN: np.ndarray, dt: float, scheme="ssprk3", nsteps: int = 1) -> np.ndarray:
        """Advance the current state nsteps fixed-dt steps (checkpointing each
        step start) and return (dS_N/dS_0)^T gN."""
        sc = abi.SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        g = np.array(gN, dtype=np.float64, order="C", copy=True)
        if g.shape != (self.neq, self.n):
            raise ValueError(f"gN must have shape {(self.neq, self.n)}")
        self._call("fvgpu_adjoint_steps", sc, float(dt), int(nsteps), _ptr(g), _ptr(g), C.c_int64(self.n))
        return g

    def profile_adjoint(self, reps: int = 5) -> tuple[float, float]:
        """Mean device ms of one residual evaluation and of one adjoint."""
        a, b = C.c_double(), C.c_double()
        self._call("fvgpu_profile_adjoint", int(reps), C.byref(a), C.byref(b))
        return a.value, b.value

    def profile_step(self, scheme="ssprk3", dt: float = 0.0, cfl: float = 0.0, nsteps: int = 1):
        """Per-kernel-kind device time (ms) and launch counts of nsteps eager steps."""
        sc = abi.SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        ms = np.zeros(abi.NKINDS)
        launches = np.zeros(abi.NKINDS, np.int32)
        self._call("fvgpu_profile_step", sc, float(dt), float(cfl), int(nsteps), _ptr(ms), _ptr(launches))
        return ms, launches

    def stream_handle(self) -> int:
        """cudaStream_t of the context (e.g. for torch.cuda.ExternalStream)."""
        out = C.c_void_p()
        self._call("fvgpu_get_stream", C.byref(out))
        return int(out.value or 0)

    def synchronize(self):
        self._call("fvgpu_synchronize")


def checkpoint_write(path: str, U: np.ndarray, mesh_sig: int, time: float = 0.0, step: int = 0):
    """Write a restart file from a host array (no GPU needed)."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    rc = load_gpu_lib().fvgpu_checkpoint_write(str(path).encode(), _ptr(U), U.shape[0], C.c_int64(U.shape[1]),
                                               C.c_uint64(mesh_sig), float(time), C.c_int64(step))
    if rc != 0:
        raise FvGpuError(rc, -1, f"cannot write {path}")


def checkpoint_read(path: str, neq: int, ncells: int, mesh_sig: int):
    """Read a restart file into a host array: (U, time, step)."""
    U = np.empty((neq, ncells))
    t, st = C.c_double(), C.c_int64()
    rc = load_gpu_lib().fvgpu_checkpoint_read(str(path).encode(), _ptr(U), int(neq), C.c_int64(ncells),
                                              C.c_uint64(mesh_sig), C.byref(t), C.byref(st))
    if rc != 0:
        raise FvGpuError(rc, -1, f"{path}: not a restart file of this mesh, or damaged")
    return U, t.value, st.value
