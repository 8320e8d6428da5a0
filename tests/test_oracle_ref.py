"""The C restatement (oracle/fvoracle.c) against the reference's own C code.

oracle/_ref/libfvref.so is the reference's hot-path sources compiled
unchanged with a harness that builds its BRANCH/CELL/LEAF objects from the
flattened tables.  Every comparison here is bit for bit.  Skipped where the
reference tree is absent (the GPU host); tests/test_golden_oracle.py covers
that case with stored reference outputs.
"""
import numpy as np
import pytest

from fv_140823_gb300 import cases
from fv_140823_gb300.abi import SolverConfig
from fv_140823_gb300.mesh import refine_by, uniform_mesh
from fvtest import bits_equal, random_ideal_state
from pyoracle import Oracle, PhysConfig, RefHarness, ref_available

pytestmark = pytest.mark.skipif(not ref_available(), reason="reference harness not built (no reference tree)")


def phys(cfg, dt=1e-3, i_case=0):
    return PhysConfig(model=cfg.model, ns=cfg.ns, ischeme=cfg.ischeme, eos=cfg.eos, i_case=i_case,
                      gamma=cfg.gamma, pinf=cfg.pinf, visc=cfg.visc, ymin=cfg.ymin, dt=dt)


def amr_mesh(periodic, seed):
    rng = np.random.default_rng(seed)
    c0 = rng.uniform(0.3, 0.7, 3)
    m = uniform_mesh(2, periodic=periodic)
    refine_by(m, lambda l, c: ((c - c0[:, None]) ** 2).sum(0) < 0.06, 4)
    return m.flatten()


@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 1, 1), (1, 0, 0)])
@pytest.mark.parametrize("ischeme", [1, 2])
def test_residual_ideal_gas_amr(periodic, ischeme):
    t = amr_mesh(periodic, seed=sum(periodic) + 10 * ischeme)
    rng = np.random.default_rng(3)
    U = random_ideal_state(t.ncells, rng)
    cfg = SolverConfig(model=1, ischeme=ischeme)
    ref, orc = RefHarness(t, phys(cfg)), Oracle(t, cfg)
    Rr = ref.residual(U)
    assert bits_equal(orc.residual(U), Rr)
    if ischeme == 2:
        assert bits_equal(orc.faceinterp(U), ref.sf())


@pytest.mark.parametrize("eos", [0, 1])
def test_viscous_and_gradients(eos):
    t = amr_mesh((1, 0, 1), seed=5)
    U = random_ideal_state(t.ncells, np.random.default_rng(4))
    cfg = SolverConfig(model=1, ischeme=2, ns=1, eos=eos, visc=0.01)
    ref, orc = RefHarness(t, phys(cfg)), Oracle(t, cfg)
    Rr = ref.residual(U)
    assert bits_equal(orc.gradcalc(U), ref.sg())
    assert bits_equal(orc.residual(U), Rr)


@pytest.mark.parametrize("ischeme", [1, 2])
def test_mixture_model3(ischeme):
    c = cases.bubble(base_level=3, extra_levels=1)
    cfg = SolverConfig(model=3, ischeme=ischeme, ymin=1e-6)
    ref, orc = RefHarness(c.tables, phys(cfg)), Oracle(c.tables, cfg)
    assert bits_equal(orc.residual(c.U), ref.residual(c.U))


def test_barotropic_model2_first_order():
    # model 2 with first-order face values (facevalues.c calls the EOS on the
    # right side); the MUSCL variant of the reference writes the EOS of both
    # sides into the own side (facercnstr.c:37) and is not compared.
    t = amr_mesh((0, 0, 0), seed=8)
    rng = np.random.default_rng(9)
    n = t.ncells
    U = np.zeros((4, n))
    U[0] = 998.2 + rng.uniform(-1.0, 1.0, n)
    U[1:4] = U[0] * 0.5 * rng.standard_normal((3, n))
    cfg = SolverConfig(model=2, ischeme=1)
    ref, orc = RefHarness(t, phys(cfg)), Oracle(t, cfg)
    assert bits_equal(orc.residual(U), ref.residual(U))


def test_inflow_boundary():
    m = uniform_mesh(3, side_bc=(2, 2, 2, 1, 2, 2))
    t = m.flatten()
    g, rho, u, p = 1.4, 1.4, 3.0, 1.0
    e = rho * ((p + g * 0.0) / (rho * (g - 1.0)) + 0.5 * (u * u + 0.0 * 0.0 + 0.0 * 0.0))
    cfg = SolverConfig(model=1, ischeme=2, inflow=(rho, rho * u, 0.0, 0.0, e))
    U = random_ideal_state(t.ncells, np.random.default_rng(11))
    ref, orc = RefHarness(t, phys(cfg, i_case=200)), Oracle(t, cfg)
    assert bits_equal(orc.residual(U), ref.residual(U))


@pytest.mark.parametrize("scheme", ["euler", "ssprk2", "ssprk3"])
def test_rk_steps(scheme):
    t = amr_mesh((1, 1, 1), seed=12)
    U = random_ideal_state(t.ncells, np.random.default_rng(13))
    cfg = SolverConfig(model=1, ischeme=2)
    ref, orc = RefHarness(t, phys(cfg, dt=2e-3)), Oracle(t, cfg)
    ref.set_state(U)
    ref.step(scheme, 3)
    assert bits_equal(orc.step(U, 2e-3, scheme, 3), ref.state())


def test_sod_full_size_steps():
    c = cases.sod(level=5)
    ref, orc = RefHarness(c.tables, phys(c.cfg, dt=1e-3)), Oracle(c.tables, c.cfg)
    ref.set_state(c.U)
    ref.step("ssprk3", 2)
    assert bits_equal(orc.step(c.U, 1e-3, "ssprk3", 2), ref.state())


def test_conservation_sums_sequential_order():
    t = amr_mesh((0, 0, 0), seed=14)
    U = random_ideal_state(t.ncells, np.random.default_rng(15))
    cfg = SolverConfig()
    ref, orc = RefHarness(t, phys(cfg)), Oracle(t, cfg)
    ref.set_state(U)
    assert bits_equal(orc.conservation(U), ref.conservation())


def _geometry_meshes():
    m = uniform_mesh(2, periodic=(1, 0, 1))
    refine_by(m, lambda l, c: ((c[0] - 0.6) ** 2 + (c[1] - 0.5) ** 2 + (c[2] - 0.45) ** 2) < 0.07, 4)
    return {"amr_unit": m.flatten(),
            "tgv_2pi": cases.tgv(base_level=3, extra_levels=2).tables,
            "bubble": cases.bubble(base_level=3, extra_levels=1).tables,
            "bump": cases.bump(base_level=3, extra_levels=2).tables}


@pytest.mark.parametrize("name", ["amr_unit", "tgv_2pi", "bubble", "bump"])
def test_geometry_equals_the_references_own(name):
    """Cell volumes, face and 1:4 sub-face areas and face frames of the mesh
    tables equal, bit for bit, what the reference's own meshproperties.c,
    normalvector.c and tagvector.c compute from the leaves' node coordinates
    (the 2*pi Taylor-Green box is the case where coordinates round)."""
    t = _geometry_meshes()[name]
    ref = RefHarness(t, PhysConfig(model=1, ns=0, ischeme=2, iprimtv=0, eos=0, i_case=0, gamma=1.4, pinf=0.0,
                                   visc=0.0, ymin=0.0, dt=1e-3))
    try:
        vol, area, frames = ref.geometry()
    finally:
        ref.close()
    n = t.ncells
    want = np.zeros((6, 4, n))
    for f in range(6):
        for c in range(n):
            code = int(t.nbr[f, c])
            if code <= -16:
                want[f, :, c] = t.hang_area[-16 - code]
            else:
                want[f, 0, c] = t.area[f, c]
    assert bits_equal(vol, t.vol)
    assert bits_equal(area, want)
    assert bits_equal(frames, np.repeat(np.asarray(t.frames).reshape(6, 9)[:, :, None], n, axis=2))
