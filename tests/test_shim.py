"""The link-time drop-in shim (fv_140823_gb300/csrc/shim/fvshim.c) inside the
reference's own host objects.

tests/shim/shimbuild.py links the reference's objects minus RHS, RHS_nb, RK,
faceinterp and gradcalc, the shim that replaces them, the table-driven RUN
builder of oracle/ref_harness.c, and a stand-in for libfvgpu that computes with
the oracle (tests/shim/fake_fvgpu.c).  The harness's calls RHS(run),
faceinterp(run), RK(irk, run) ... then resolve to the shim, which flattens the
leaf list with the host's own distance(), uploads it and keeps the state
"device"-side.  Every result is compared bit for bit with the unmodified
reference (oracle/_ref/libfvref.so) on the same mesh.  Runs where the
reference tree exists (CPU only).
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from fvtest import bits_equal, golden_names, load_golden

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "shim"))

pyoracle = pytest.importorskip("pyoracle")
if not pyoracle.ref_available():
    pytest.skip("reference tree absent: the shim links the reference's host objects", allow_module_level=True)

import shimbuild as shim_build  # noqa: E402  (tests/shim/shimbuild.py)

FVSHIM_S, FVSHIM_SN, FVSHIM_RHS, FVSHIM_SF, FVSHIM_SG = 1, 2, 4, 8, 16


@pytest.fixture(scope="module")
def shimlib():
    path = shim_build.build_shim_test()
    assert path is not None
    return path


def make_harness(shimlib):
    class ShimHarness(pyoracle.RefHarness):
        _lib = None

        @classmethod
        def lib(cls):
            if cls._lib is None:
                saved = pyoracle.REF_LIB
                pyoracle.REF_LIB = shimlib
                try:
                    cls._lib = None
                    L = pyoracle.RefHarness.lib.__func__(cls)
                finally:
                    pyoracle.REF_LIB = saved
                vp = C.c_void_p
                L.fvshim_sync_host.argtypes = [vp, C.c_int]
                L.fvshim_invalidate.argtypes = [vp]
                L.fvshim_set_scheme.argtypes = [C.c_int]
                L.fvshim_counters.argtypes = [C.POINTER(C.c_long), C.POINTER(C.c_long)]
                L.advancetimeexplicit.argtypes = [vp]
                L.fake_calls.argtypes = [C.c_int]
                L.fake_calls.restype = C.c_int
                cls._lib = L
            return cls._lib

        @property
        def run(self):  # struct refh begins with its RUN pointer
            return C.cast(self._h, C.POINTER(C.c_void_p))[0]

        def set_state(self, U):
            super().set_state(U)
            self.lib().fvshim_invalidate(self.run)

        def sync(self, fields):
            self.lib().fvshim_sync_host(self.run, fields)

        def close(self):
            if getattr(self, "_h", None):
                self.lib().fvshim_release()
            super().close()

    return ShimHarness


def phys(cfg, z, name):
    # the inflow fixture uses the reference's i_case 200 inflow state (tests/golden/make_golden.py)
    return pyoracle.PhysConfig(model=cfg.model, ns=cfg.ns, ischeme=cfg.ischeme, eos=cfg.eos, gamma=cfg.gamma,
                               pinf=cfg.pinf, visc=cfg.visc, ymin=cfg.ymin, dt=float(z["dt"]),
                               i_case=200 if name == "inflow_l3" else 0)


@pytest.mark.parametrize("name", golden_names())
def test_shim_reproduces_reference_calls(shimlib, name):
    t, cfg, z = load_golden(name)
    pc = phys(cfg, z, name)
    Shim = make_harness(shimlib)
    ref, sh = pyoracle.RefHarness(t, pc), Shim(t, pc)
    try:
        U = z["U"]
        for h in (ref, sh):
            h.set_state(U)
            if pc.ischeme == 2:
                h.faceinterp()
            if pc.ns == 1:
                h.gradcalc()
            h.rhs()
        sh.sync(FVSHIM_RHS | FVSHIM_SF | FVSHIM_SG)
        assert bits_equal(sh.rhs_array(), ref.rhs_array())
        if pc.ischeme == 2:
            assert bits_equal(sh.sf(), ref.sf())
        if pc.ns == 1:
            assert bits_equal(sh.sg(), ref.sg())
        # the stage sequence of a step through RK(0), faceinterp, gradcalc, RHS, RK(k)
        for h in (ref, sh):
            h.set_state(U)
            h.step(str(z["scheme"]), int(z["nsteps"]))
        sh.sync(FVSHIM_S | FVSHIM_SN)
        assert bits_equal(sh.state(), ref.state())
        assert bits_equal(sh.state_n(), ref.state_n())
    finally:
        sh.close()
        ref.close()


def test_shim_advancetimeexplicit_keeps_state_on_device(shimlib):
    t, cfg, z = load_golden("amr_periodic_muscl")
    pc = phys(cfg, z, "amr_periodic_muscl")
    Shim = make_harness(shimlib)
    ref, sh = pyoracle.RefHarness(t, pc), Shim(t, pc)
    try:
        U = z["U"]
        ref.set_state(U)
        ref.step("ssprk3", 4)
        sh.set_state(U)
        L = sh.lib()
        up0, sy0, up1, sy1 = C.c_long(), C.c_long(), C.c_long(), C.c_long()
        L.fvshim_counters(C.byref(up0), C.byref(sy0))
        for _ in range(4):
            L.advancetimeexplicit(sh.run)
        L.fvshim_counters(C.byref(up1), C.byref(sy1))
        # one flatten + upload, no host sync inside the time loop
        assert up1.value - up0.value == 1 and sy1.value == sy0.value
        assert L.fake_calls(8) == 0 and L.fake_calls(5) == 4
        assert not bits_equal(sh.state(), ref.state())  # leaves untouched until a sync point
        sh.sync(FVSHIM_S)
        assert bits_equal(sh.state(), ref.state())
        # the host's own gradcalc (the export point of the time loop) syncs S and SG
        sh.set_state(U)
        for _ in range(2):
            L.advancetimeexplicit(sh.run)
        sh.gradcalc()
        ref.set_state(U)
        ref.step("ssprk3", 2)
        ref.gradcalc()
        assert bits_equal(sh.state(), ref.state())
    finally:
        sh.close()
        ref.close()


def test_shim_exports_the_reference_symbols(shimlib):
    L = C.CDLL(shimlib)
    for sym in ("RHS", "RHS_nb", "RK", "faceinterp", "gradcalc", "advancetimeexplicit", "advancetimeexplicit_nb",
                "fvshim_sync_host", "fvshim_invalidate", "fvshim_set_scheme", "fvshim_set_precision",
                "fvshim_set_error_handler", "fvshim_release", "fvshim_counters"):
        assert hasattr(L, sym), sym
