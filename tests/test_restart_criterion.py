"""Bit-exact restart files and the refinement criterion.

* The restart format (fvgpu_checkpoint_write / _read, host code of libfvgpu)
  round-trips the FP64 state bit for bit and rejects damaged, truncated or
  foreign files; the reference's text restart (restart_save.c:41, "%15.10e")
  is shown to lose bits on the same state.
* The criterion restatement (pyoracle.criterion) equals the reference's own
  criterionsplt.c on its gradients (oracle/_ref); the GPU kernel equals the
  restatement (gpu marker).
* GPU: save after some steps, load into a fresh context, continue: bit-identical
  to the uninterrupted run.
"""
import os
import tempfile

import numpy as np
import pytest

from fv_140823_gb300 import abi, cases
from fvtest import bits_equal, load_golden
import pyoracle


def test_restart_file_round_trip_and_rejections():
    from fv_140823_gb300.solver import FvGpuError, checkpoint_read, checkpoint_write
    rng = np.random.default_rng(3)
    U = rng.standard_normal((5, 1000)) * 10.0 ** rng.integers(-300, 300, (5, 1000))
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "s.fvck")
        checkpoint_write(p, U, mesh_sig=1234, time=0.125, step=77)
        V, t, st = checkpoint_read(p, 5, 1000, 1234)
        assert bits_equal(V, U) and t == 0.125 and st == 77
        with pytest.raises(FvGpuError):
            checkpoint_read(p, 5, 1000, 1235)              # another mesh
        with pytest.raises(FvGpuError):
            checkpoint_read(p, 5, 999, 1234)               # another size
        raw = bytearray(open(p, "rb").read())
        raw[100] ^= 1
        q = os.path.join(d, "bad.fvck")
        open(q, "wb").write(bytes(raw))
        with pytest.raises(FvGpuError):
            checkpoint_read(q, 5, 1000, 1234)              # flipped bit: checksum
        open(q, "wb").write(bytes(raw[:-9]))
        with pytest.raises(FvGpuError):
            checkpoint_read(q, 5, 1000, 1234)              # truncated
    # the reference's text restart loses bits on the same numbers
    text = np.array([float(f"{x:15.10e}") for x in U.ravel()[:100]])
    assert not bits_equal(text, U.ravel()[:100])


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference tree absent")
@pytest.mark.parametrize("name", ["sod_l3", "amr_periodic_muscl", "tgv_l3"])
def test_criterion_restatement_matches_reference(name):
    t, cfg, z = load_golden(name)
    pc = pyoracle.PhysConfig(model=cfg.model, ns=cfg.ns, ischeme=cfg.ischeme, eos=cfg.eos, gamma=cfg.gamma,
                             pinf=cfg.pinf, visc=cfg.visc, ymin=cfg.ymin, dt=float(z["dt"]))
    ref = pyoracle.RefHarness(t, pc)
    try:
        U = z["U"]
        ref.set_state(U)
        ref.gradcalc()
        g = np.sqrt((ref.sg()[0] ** 2).sum(axis=0))
        for q in (0.5, 0.9):
            # the reference hard-codes |grad rho| > 100 (i_case 204): scale the
            # state (its density gradient scales with it) to put the threshold
            # at a quantile of the positive gradients
            scale = 100.0 / np.quantile(g[g > 0], q)
            ref.set_state(U * scale)
            ref.gradcalc()
            SG = ref.sg()
            want = ref.criterion(204, 7)
            got = pyoracle.criterion(U * scale, SG, t.vol, abi.CRIT_GRAD_RHO, 100.0, 7)
            assert np.array_equal(got, want) and 0 < np.sum(got == 7) < got.size
        # i_case 2500: rho < 50
        scale = 50.0 / np.quantile(U[0], 0.4)
        ref.set_state(U * scale)
        got = pyoracle.criterion(U * scale, SG, t.vol, abi.CRIT_RHO_BELOW, 50.0, 5)
        assert np.array_equal(got, ref.criterion(2500, 5))
    finally:
        ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sod_l3", "tgv_l3", "bubble_l3"])
def test_gpu_criterion_matches_restatement(name):
    from fv_140823_gb300.solver import Solver
    t, cfg, z = load_golden(name)
    U = z["U"]
    with Solver(t, cfg) as s:
        s.set_state(U)
        s.gradcalc()
        SG = s.sg()
        g = np.sqrt((SG[0] ** 2).sum(axis=0))

        def between(x, q):
            # a threshold halfway between two distinct data values near the
            # quantile: no cell sits within rounding of it (cbrt is not
            # correctly rounded on either side)
            u = np.unique(x)
            i = min(max(int(q * u.size), 1), u.size - 1)
            return 0.5 * (u[i - 1] + u[i])

        for kind, thr in ((abi.CRIT_GRAD_RHO, between(g, 0.7)), (abi.CRIT_RHO_BELOW, between(U[0], 0.3)),
                          (abi.CRIT_GRAD_RHO_H, between(g * np.cbrt(t.vol), 0.7))):
            got = s.criterion(kind, float(thr), 6)
            assert np.array_equal(got, pyoracle.criterion(U, SG, t.vol, kind, float(thr), 6)), kind


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_gpu_restart_continues_bit_identically(precision):
    from fv_140823_gb300.abi import SolverConfig
    from fv_140823_gb300.solver import Solver
    c = cases.periodic(level=4)
    cfg = SolverConfig(**{**c.cfg.__dict__, "precision": precision})
    with Solver(c.tables, cfg) as s:
        s.set_state(c.U)
        dt = s.compute_dt(0.5)
        s.step("ssprk3", dt=dt, nsteps=6)
        ref = s.state()
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "r.fvck")
        with Solver(c.tables, cfg) as s:
            s.set_state(c.U)
            s.step("ssprk3", dt=dt, nsteps=3)
            s.checkpoint_save(p, time=3 * dt, step=3)
        with Solver(c.tables, cfg) as s:
            t, st = s.checkpoint_load(p)
            assert st == 3 and t == 3 * dt
            s.step("ssprk3", dt=dt, nsteps=3)
            assert bits_equal(s.state(), ref)
