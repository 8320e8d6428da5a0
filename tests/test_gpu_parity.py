"""FP64 GPU path against the reference (golden fixtures) and the oracle.

Every comparison on the FP64 path is bit for bit: libfvgpu evaluates each
cell in the reference's order with IEEE division / square root and no fused
multiply-add, so its residuals, face values, gradients and RK states equal
the reference's C code exactly (models 1 and 3; model 2 uses CUDA's pow and
is held to 1e-12 relative).
"""
import numpy as np
import pytest

from fv_140823_gb300 import abi, cases
from fv_140823_gb300.abi import SolverConfig
from fv_140823_gb300.mesh import refine_by, uniform_mesh
from fvtest import bits_equal, golden_names, load_golden, max_rel, random_ideal_state
from pyoracle import Oracle

pytestmark = pytest.mark.gpu


def solver(t, cfg):
    from fv_140823_gb300.solver import Solver
    return Solver(t, cfg)


def amr_mesh(periodic, seed, base=2, maxl=4):
    rng = np.random.default_rng(seed)
    c0 = rng.uniform(0.3, 0.7, 3)
    m = uniform_mesh(base, periodic=periodic)
    refine_by(m, lambda l, c: ((c - c0[:, None]) ** 2).sum(0) < 0.06, maxl)
    return m.flatten()


@pytest.mark.parametrize("name", golden_names())
def test_gpu_matches_reference_golden(name):
    t, cfg, z = load_golden(name)
    U = z["U"]
    with solver(t, cfg) as s:
        s.set_state(U)
        if cfg.ischeme == 2:
            s.faceinterp()
            assert bits_equal(s.sf(), z["SF"])
        if cfg.ns == 1:
            s.gradcalc()
            assert bits_equal(s.sg(), z["SG"])
        s.rhs()
        assert bits_equal(s.rhs_array(), z["R"])
        s.set_state(U)
        s.step(str(z["scheme"]), dt=float(z["dt"]), nsteps=int(z["nsteps"]))
        assert bits_equal(s.state(), z["S_out"])


@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 1, 1)])
@pytest.mark.parametrize("ischeme", [1, 2])
@pytest.mark.parametrize("ns", [0, 1])
def test_residual_random_states_amr(periodic, ischeme, ns):
    t = amr_mesh(periodic, seed=3 + ischeme + 2 * ns, base=3, maxl=5)
    U = random_ideal_state(t.ncells, np.random.default_rng(7))
    cfg = SolverConfig(model=1, ischeme=ischeme, ns=ns, eos=ns, visc=0.01 * ns)
    orc = Oracle(t, cfg)
    with solver(t, cfg) as s:
        R = s.residual(U)
        assert bits_equal(R, orc.residual(U))
        if ischeme == 2:
            assert bits_equal(s.sf(), orc.faceinterp(U))
        if ns == 1:
            assert bits_equal(s.sg(), orc.gradcalc(U))


@pytest.mark.parametrize("ns", [0, 1])
def test_wall_boundaries_match_oracle(ns):
    """Slip (3) and no-slip (4) walls have no reference code; the oracle and
    the GPU share one definition (velocity and momentum mirrored as such)."""
    rng = np.random.default_rng(21)
    c0 = rng.uniform(0.3, 0.7, 3)
    m = uniform_mesh(3, side_bc=(3, 4, 3, 4, 3, 4))
    refine_by(m, lambda l, c: ((c - c0[:, None]) ** 2).sum(0) < 0.06, 5)
    t = m.flatten()
    U = random_ideal_state(t.ncells, np.random.default_rng(22))
    cfg = SolverConfig(model=1, ischeme=2, ns=ns, eos=ns, visc=0.01 * ns)
    orc = Oracle(t, cfg)
    with solver(t, cfg) as s:
        assert bits_equal(s.residual(U), orc.residual(U))
        assert bits_equal(s.sf(), orc.faceinterp(U))
        s.set_state(U)
        s.step("ssprk3", dt=1e-4, nsteps=2)
        assert bits_equal(s.state(), orc.step(U, 1e-4, "ssprk3", 2))


@pytest.mark.parametrize("scheme", ["euler", "ssprk2", "ssprk3"])
@pytest.mark.parametrize("ischeme", [1, 2])
def test_fixed_dt_steps(scheme, ischeme):
    t = amr_mesh((1, 0, 1), seed=11, base=3, maxl=5)
    U = random_ideal_state(t.ncells, np.random.default_rng(12))
    cfg = SolverConfig(model=1, ischeme=ischeme)
    orc = Oracle(t, cfg)
    with solver(t, cfg) as s:
        s.set_state(U)
        s.step(scheme, dt=1e-3, nsteps=4)
        assert bits_equal(s.state(), orc.step(U, 1e-3, scheme, 4))


def test_mixture_model3_bubble():
    c = cases.bubble(base_level=3, extra_levels=2)
    orc = Oracle(c.tables, c.cfg)
    with solver(c.tables, c.cfg) as s:
        assert bits_equal(s.residual(c.U), orc.residual(c.U))
        s.set_state(c.U)
        s.step("ssprk3", dt=2e-7, nsteps=3)
        assert bits_equal(s.state(), orc.step(c.U, 2e-7, "ssprk3", 3))


def test_barotropic_model2_tolerance():
    t = amr_mesh((0, 0, 0), seed=21)
    rng = np.random.default_rng(22)
    n = t.ncells
    U = np.zeros((4, n))
    U[0] = 998.2 + rng.uniform(-1.0, 1.0, n)
    U[1:4] = U[0] * 0.5 * rng.standard_normal((3, n))
    for ischeme in (1, 2):
        cfg = SolverConfig(model=2, ischeme=ischeme)
        with solver(t, cfg) as s:
            R = s.residual(U)
        Rr = Oracle(t, cfg).residual(U)
        assert max_rel(R, Rr) <= 1e-12


def test_cfl_steps_match_oracle_dt_sequence():
    c = cases.sod(level=4)
    orc = Oracle(c.tables, c.cfg)
    S = c.U.copy()
    for _ in range(3):
        dt = orc.cfl_dt(S, 0.5)
        S = orc.step(S, dt, "ssprk3", 1)
    with solver(c.tables, c.cfg) as s:
        s.set_state(c.U)
        assert s.compute_dt(0.5) == orc.cfl_dt(c.U, 0.5)
        s.step("ssprk3", cfl=0.5, nsteps=3)
        assert bits_equal(s.state(), S)


def test_rhs_nb_inner_outer_split():
    t = amr_mesh((0, 0, 0), seed=31)
    U = random_ideal_state(t.ncells, np.random.default_rng(32))
    cfg = SolverConfig(model=1, ischeme=2)
    orc = Oracle(t, cfg)
    inner = (np.arange(t.ncells) % 3 == 0).astype(np.int32)
    with solver(t, cfg) as s:
        s.set_state(U)
        s.faceinterp()
        s.set_inner(inner)
        s.rhs_nb(1)
        s.rhs_nb(0)
        assert bits_equal(s.rhs_array(), orc.residual(U))


def test_reference_call_sequence_rk_stages():
    """RK(0); per stage faceinterp, RHS, RK(k) through the individual calls."""
    t = amr_mesh((1, 1, 1), seed=41)
    U = random_ideal_state(t.ncells, np.random.default_rng(42))
    cfg = SolverConfig(model=1, ischeme=2)
    dt = 1.5e-3
    with solver(t, cfg) as s:
        s.set_state(U)
        s.rk(0, dt)
        for irk in (1, 2, 3):
            s.faceinterp()
            s.rhs()
            s.rk(irk, dt)
        assert bits_equal(s.state(), Oracle(t, cfg).step(U, dt, "ssprk3", 1))
        assert bits_equal(s.state_n(), U)


def test_conservation_sums():
    t = amr_mesh((1, 1, 1), seed=51, base=3, maxl=5)
    U = random_ideal_state(t.ncells, np.random.default_rng(52))
    cfg = SolverConfig()
    with solver(t, cfg) as s:
        s.set_state(U)
        sums = s.conservation()
        again = s.conservation()
    ref = Oracle(t, cfg).conservation(U)
    assert bits_equal(sums, again)  # fixed reduction order
    assert max_rel(sums, ref) <= 1e-13


def test_periodic_step_conserves_mass_and_energy():
    c = cases.periodic(level=4)
    with solver(c.tables, c.cfg) as s:
        s.set_state(c.U)
        before = s.conservation()
        s.step("ssprk3", cfl=0.5, nsteps=5)
        after = s.conservation()
    assert np.allclose(before[[0, 1, 2, 3, 4]], after[[0, 1, 2, 3, 4]], rtol=1e-12, atol=1e-13)


def test_deterministic_repeat():
    c = cases.periodic(level=4)
    outs = []
    for _ in range(2):
        with solver(c.tables, c.cfg) as s:
            s.set_state(c.U)
            s.step("ssprk3", cfl=0.5, nsteps=3)
            outs.append(s.state())
    assert bits_equal(outs[0], outs[1])


def test_nonfinite_state_reports_cell_and_context_recovers():
    from fv_140823_gb300.solver import FvGpuError
    c = cases.sod(level=3)
    U = c.U.copy()
    U[0, 77] = np.nan
    with solver(c.tables, c.cfg) as s:
        s.set_state(U)
        s.faceinterp()
        s.rhs()
        with pytest.raises(FvGpuError) as ei:
            s.synchronize()
        assert ei.value.code in (abi.ERR_NONFINITE, abi.ERR_EOS)
        assert ei.value.cell >= 0
        # the context stays usable
        assert bits_equal(s.residual(c.U), Oracle(c.tables, c.cfg).residual(c.U))


def test_mesh_validation_rejects_broken_tables():
    from fv_140823_gb300.solver import FvGpuError
    t = uniform_mesh(2).flatten()
    bad = uniform_mesh(2).flatten()
    bad.nbr = bad.nbr.copy()
    bad.nbr[1, 0] = 5  # cell 0 +x face pointing at a cell that does not link back
    with solver(t, SolverConfig()) as s:
        with pytest.raises(FvGpuError) as ei:
            s.upload_mesh(bad)
        assert ei.value.code == abi.ERR_MESH
        bad2 = uniform_mesh(2).flatten()
        bad2.vol = bad2.vol.copy()
        bad2.vol[3] = -1.0
        with pytest.raises(FvGpuError):
            s.upload_mesh(bad2)
