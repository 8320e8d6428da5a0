"""FP32-mixed path against the FP64 path (which is bit-identical to the
reference).  Tolerance: relative L2 error per conserved field <= 1e-6 (the
accuracy budget) after the stated number of steps; the Sod tube and the
two-phase bubble are held to about 3x the errors they reach (Sod 2e-8 /
9.6e-8 / 2.4e-8 on rho / rho u / E; bubble 1.4e-14 on rho, 2.4e-7 on the
momentum, 5e-16 on rho Y), so that a regression shows."""
import numpy as np
import pytest

from fv_140823_gb300 import abi, cases
from fv_140823_gb300.abi import SolverConfig

pytestmark = pytest.mark.gpu


def solver(t, cfg):
    from fv_140823_gb300.solver import Solver
    return Solver(t, cfg)


def rel_l2_mom(a, b):
    """Relative L2 error per field with the three momentum components measured
    against the norm of the whole momentum (a component that is zero in exact
    arithmetic has only rounding noise and no relative error of its own)."""
    e = rel_l2(a, b)
    nm = max(np.linalg.norm(b[1:4]), 1e-300)
    e[1:4] = [np.linalg.norm(a[v] - b[v]) / nm for v in (1, 2, 3)]
    return e


def rel_l2(a, b):
    return np.array([np.linalg.norm(a[v] - b[v]) / max(np.linalg.norm(b[v]), 1e-300) for v in range(a.shape[0])])


def run(case, precision, nsteps, dt):
    cfg = SolverConfig(**{**case.cfg.__dict__, "precision": precision})
    with solver(case.tables, cfg) as s:
        s.set_state(case.U)
        s.step(case.scheme, dt=dt, nsteps=nsteps)
        return s.state()


def fixed_dt(case):
    cfg = SolverConfig(**{**case.cfg.__dict__, "precision": abi.FP64})
    with solver(case.tables, cfg) as s:
        s.set_state(case.U)
        return s.compute_dt(case.cfl)


@pytest.mark.parametrize("level,nsteps", [(5, 50), (6, 20)])
def test_periodic_smooth_flow_within_1e6(level, nsteps):
    c = cases.periodic(level=level)
    dt = fixed_dt(c)
    a = run(c, abi.MIXED, nsteps, dt)
    b = run(c, abi.FP64, nsteps, dt)
    err = rel_l2(a, b)
    assert np.all(err <= 1e-6), err


def test_sod_within_1e5():
    c = cases.sod(level=5)
    dt = fixed_dt(c)
    a, b = run(c, abi.MIXED, 20, dt), run(c, abi.FP64, 20, dt)
    err = rel_l2(a, b)
    assert err[0] <= 6e-8 and err[1] <= 2.9e-7 and err[4] <= 7e-8, err
    # momentum components normal to the tube stay exactly zero in both paths
    assert not np.any(a[2:4]) and not np.any(b[2:4])


@pytest.mark.parametrize("scheme", ["euler", "ssprk2", "ssprk3"])
def test_amr_bump_all_schemes(scheme):
    c = cases.bump(base_level=4, extra_levels=2)
    c.scheme = scheme
    dt = fixed_dt(c)
    err = rel_l2(run(c, abi.MIXED, 10, dt), run(c, abi.FP64, 10, dt))
    assert np.all(err[[0, 1, 4]] <= 1e-6), err


def test_mixture_bubble_model3():
    c = cases.bubble(base_level=3, extra_levels=2)
    dt = 2e-7
    err = rel_l2(run(c, abi.MIXED, 5, dt), run(c, abi.FP64, 5, dt))
    # the density and rho Y are paired FP32 words reconstructed in FP64, so
    # the FP64 pressure inversion sees both partial densities to FP64
    # rounding; the momentum carries the FP32 flux arithmetic
    assert err[0] <= 4e-14 and err[4] <= 1.5e-15, err
    assert np.all(err[1:4] <= 7e-7), err


def test_mixture_bubble_model3_viscous():
    """Model 3 with viscous fluxes: velocities (face fluxes, ghosts and the
    Green-Gauss gradients) divide by the density of the paired state words."""
    c = cases.bubble(base_level=3, extra_levels=2)
    cfg = SolverConfig(**{**c.cfg.__dict__, "ns": 1, "eos": 0, "visc": 1e-3})
    c = cases.Case("bubble_viscous", c.tables, c.U, cfg, cfl=0.5, nsteps=5)
    dt = 2e-7
    err = rel_l2(run(c, abi.MIXED, 5, dt), run(c, abi.FP64, 5, dt))
    assert err[0] <= 4e-14 and err[4] <= 1.5e-15 and np.all(err[1:4] <= 8e-7), err


@pytest.mark.parametrize("bc", [2, 3, 4])
def test_smooth_flow_next_to_domain_boundaries_within_1e6(bc):
    """A cell next to a domain boundary limits its slope on that axis as the
    reference does (a transmissive ghost gives sm = 0 * inf, NaN, and a zero
    slope); a one-sided slope there would show as a 1e-3-level error."""
    from fv_140823_gb300.mesh import uniform_mesh
    t = uniform_mesh(4, side_bc=(bc,) * 6).flatten()
    x, y, z = t.centroid
    s2 = lambda a: np.sin(2.0 * np.pi * a)
    rho = 1.0 + 0.2 * s2(x + 0.1) * s2(y + 0.3) * s2(z + 0.2)
    u, v, w = 0.2 * s2(y + 0.2), 0.1 * s2(z + 0.4), 0.15 * s2(x + 0.3)
    p = 1.0 + 0.1 * s2(x + 0.25) * s2(y + 0.15)
    c = cases.Case("boundary", t, cases.conservative_ideal(rho, u, v, w, p), SolverConfig(model=1, ischeme=2),
                   cfl=0.5, nsteps=10)
    dt = fixed_dt(c)
    err = rel_l2(run(c, abi.MIXED, 10, dt), run(c, abi.FP64, 10, dt))
    assert np.all(err <= 1e-6), err


@pytest.mark.parametrize("mesh", ["uniform", "amr"])
def test_mixed_conserves_and_is_deterministic(mesh):
    """Mass and energy on periodic meshes (the AMR one with 1:4 faces, 4x4x4
    bricks and general blocks on concurrent streams) drift only by the FP32
    rounding of the stage increments; repeated runs are bitwise equal."""
    if mesh == "uniform":
        c = cases.periodic(level=5)
    else:
        from fv_140823_gb300.mesh import refine_by, uniform_mesh
        m = uniform_mesh(4, periodic=(1, 1, 1))
        refine_by(m, lambda l, cen: ((cen - 0.5) ** 2).sum(0) < 0.04, 5)
        t = m.flatten()
        x, y, z = t.centroid
        s2 = lambda q: np.sin(2.0 * np.pi * q)
        rho = 1.0 + 0.1 * s2(x) * s2(y) * s2(z)
        U = cases.conservative_ideal(rho, 0.2 * s2(y), 0.1 * s2(z), 0.15 * s2(x), 1.0 + 0.05 * s2(x + y))
        c = cases.Case("amr", t, U, SolverConfig(model=1, ischeme=2), cfl=0.5, nsteps=7)
    cfg = SolverConfig(**{**c.cfg.__dict__, "precision": abi.MIXED})
    outs = []
    for _ in range(2):
        with solver(c.tables, cfg) as s:
            s.set_state(c.U)
            before = s.conservation()
            s.step("ssprk3", cfl=0.5, nsteps=7)
            after = s.conservation()
            outs.append(s.state())
        drift = np.abs(after - before)[[0, 4]] / np.abs(before[[0, 4]])
        assert np.all(drift <= 1e-9), drift
    assert np.array_equal(outs[0].view(np.int64), outs[1].view(np.int64))


def test_mixed_cfl_dt_tracks_fp64():
    c = cases.periodic(level=5)
    dts = {}
    for prec in (abi.MIXED, abi.FP64):
        cfg = SolverConfig(**{**c.cfg.__dict__, "precision": prec})
        with solver(c.tables, cfg) as s:
            s.set_state(c.U)
            s.step("ssprk3", cfl=0.5, nsteps=5)
            dts[prec] = s.compute_dt(0.5)
    assert abs(dts[abi.MIXED] - dts[abi.FP64]) <= 1e-6 * dts[abi.FP64]


def test_precision_switch_keeps_state():
    c = cases.periodic(level=4)
    with solver(c.tables, SolverConfig(**{**c.cfg.__dict__, "precision": abi.FP64})) as s:
        s.set_state(c.U)
        s.set_precision(abi.MIXED)
        s.step("ssprk3", cfl=0.5, nsteps=3)   # odd count: the state ends in the second buffer
        s.set_precision(abi.FP64)
        s.step("ssprk3", cfl=0.5, nsteps=1)
        S = s.state()
    assert np.all(np.isfinite(S))
    ref = run(c, abi.FP64, 0, 1.0)
    assert np.array_equal(ref, c.U)


@pytest.mark.parametrize("eos", [1, 0])
def test_mixed_viscous_taylor_green_within_1e6(eos):
    """Viscous fluxes in the mixed path (FP32 gradients and stress, general
    kernel) against the FP64 path on the Taylor-Green vortex with 1:4 faces,
    with and without the energy work term; viscosity raised so that the
    viscous terms shape the flow over the steps compared."""
    c = cases.tgv(base_level=3, extra_levels=1)
    base = {**c.cfg.__dict__, "eos": eos, "visc": 0.05}
    dt = fixed_dt(cases.Case(c.name, c.tables, c.U, SolverConfig(**base), cfl=c.cfl, nsteps=1))

    def run_p(precision):
        with solver(c.tables, SolverConfig(**{**base, "precision": precision})) as s:
            s.set_state(c.U)
            s.step("ssprk3", dt=dt, nsteps=20)
            return s.state()
    a, b = run_p(abi.MIXED), run_p(abi.FP64)
    err = rel_l2(a, b)
    assert np.all(err[[0, 1, 2, 4]] <= 1e-6), err
    # the viscous terms matter over these steps: an inviscid FP64 run differs
    with solver(c.tables, SolverConfig(**{**base, "visc": 0.0, "precision": abi.FP64})) as s:
        s.set_state(c.U)
        s.step("ssprk3", dt=dt, nsteps=20)
        assert np.max(rel_l2(s.state(), b)[[1, 2]]) > 1e-4


def test_uniform_two_pi_box_on_the_brick_kernel():
    """The 2*pi Taylor-Green box, uniform: its face areas follow the node
    coordinates and vary in the last bits from cell to cell (as the
    reference's areaproperties gives them); the slope-sharing brick kernel
    takes one FP32 area per level and axis and stays within 1e-6 of FP64."""
    c = cases.tgv(base_level=5, extra_levels=0)
    t = c.tables
    assert bricks_throughout(t)
    assert len(np.unique(t.area)) > 1  # the areas do vary
    dt = fixed_dt(c)
    a = run(c, abi.MIXED, 10, dt)
    b = run(c, abi.FP64, 10, dt)
    err = rel_l2_mom(a, b)
    assert np.all(err <= 1e-6), err


def _mixed_state(case, flags, nsteps, dt):
    cfg = SolverConfig(**{**case.cfg.__dict__, "precision": abi.MIXED, "flags": flags})
    with solver(case.tables, cfg) as s:
        s.set_state(case.U)
        s.step(case.scheme, dt=dt, nsteps=nsteps)
        return s.state()


def bricks_throughout(t) -> bool:
    """A uniform octree of level >= 3 is 8x8x4 bricks throughout: model 1 runs
    it on the slope-sharing brick kernel, FVGPU_FLAG_NO_BRICKS (and every
    other mesh) on the table-driven kernel family."""
    return bool(np.all(t.level == t.level[0])) and int(t.level[0]) >= 3


@pytest.mark.parametrize("name", ["periodic", "sod", "bump", "inflow", "bubble", "tgv", "tgv_walls"])
def test_brick_kernel_bit_identical_to_general_kernel(name):
    """Within the table-driven family the 8x8x4 / 4x4x4 brick kernels and the
    general kernel accumulate every cell's residual from the same canonical
    face fluxes in the same order: bit-identical.  On meshes of 8x8x4 bricks
    throughout the default run uses the slope-sharing kernel instead, which
    agrees with the table-driven family to FP32 rounding (<= 1e-6)."""
    if name == "periodic":
        c = cases.periodic(level=5)
    elif name == "sod":
        c = cases.sod(level=5)
    elif name == "bump":
        c = cases.bump(base_level=4, extra_levels=2)
        c.scheme = "ssprk3"
    elif name == "bubble":
        c = cases.bubble(base_level=4, extra_levels=1)
    elif name == "tgv":  # viscous: both kernels subtract the same FP32 viscous flux
        c = cases.tgv(base_level=5, extra_levels=1)
    elif name == "tgv_walls":  # viscous next to slip and no-slip walls
        from fv_140823_gb300.mesh import uniform_mesh
        g = cases.tgv(base_level=4, extra_levels=0)
        t = uniform_mesh(4, side_bc=(3, 4, 3, 4, 3, 4)).flatten()
        c = cases.Case("tgv_walls", t, g.U, g.cfg, cfl=0.5, nsteps=5)
    else:
        from fv_140823_gb300.mesh import uniform_mesh
        t = uniform_mesh(5, side_bc=(2, 2, 2, 1, 2, 2)).flatten()
        rho, u, p = 1.4, 3.0, 1.0
        e = rho * (p / (rho * 0.4) + 0.5 * u * u)
        U = cases.conservative_ideal(np.full(t.ncells, 1.0), np.full(t.ncells, 0.5), np.zeros(t.ncells),
                                     np.zeros(t.ncells), np.full(t.ncells, 1.0))
        c = cases.Case("inflow", t, U, SolverConfig(model=1, ischeme=2, inflow=(rho, rho * u, 0.0, 0.0, e)),
                       cfl=0.5, nsteps=5)
    dt = 2e-7 if name == "bubble" else fixed_dt(c)
    a = _mixed_state(c, 0, 4, dt)
    b = _mixed_state(c, abi.FLAG_NO_BRICKS, 4, dt)
    if bricks_throughout(c.tables) and c.cfg.model == 1:
        assert np.all(rel_l2_mom(a, b) <= 1e-6), rel_l2_mom(a, b)
    else:
        assert np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("flags", [0, abi.FLAG_NO_BRICKS])
def test_mixed_nonfinite_state_reports_and_context_recovers(flags):
    """A NaN in the state surfaces as FVGPU_ERR_NONFINITE / _EOS with a cell at
    the next synchronising call, in the brick and in the general kernel; the
    context then steps a clean state bit-identically to a fresh context."""
    from fv_140823_gb300.solver import FvGpuError
    c = cases.periodic(level=4)
    cfg = SolverConfig(**{**c.cfg.__dict__, "precision": abi.MIXED, "flags": flags})
    dt = fixed_dt(c)
    U = c.U.copy()
    U[0, 1234] = np.nan
    with solver(c.tables, cfg) as s:
        s.set_state(U)
        with pytest.raises(FvGpuError) as ei:
            s.step("ssprk3", dt=dt, nsteps=1)
            s.synchronize()
        assert ei.value.code in (abi.ERR_NONFINITE, abi.ERR_EOS)
        assert ei.value.cell >= 0
        s.set_state(c.U)
        s.step("ssprk3", dt=dt, nsteps=2)
        got = s.state()
    with solver(c.tables, cfg) as s:
        s.set_state(c.U)
        s.step("ssprk3", dt=dt, nsteps=2)
        assert np.array_equal(got.view(np.int64), s.state().view(np.int64))


@pytest.mark.parametrize("level", [1, 2, 3])
@pytest.mark.parametrize("periodic", [True, False])
def test_small_meshes_bricks_and_general_agree(level, periodic):
    """Meshes of 8, 64 and 512 cells: no brick, one 4x4x4 brick, two 8x8x4
    bricks; periodic ones wrap a brick onto itself.  Within one kernel family
    the bricks and the general kernel give the same bits (the 512-cell mesh
    runs the slope-sharing kernel by default and agrees with the table-driven
    family to FP32 rounding), and every run stays within 1e-6 of FP64."""
    from fv_140823_gb300.mesh import uniform_mesh
    m = uniform_mesh(level, periodic=(1, 1, 1)) if periodic else uniform_mesh(level, side_bc=(2,) * 6)
    t = m.flatten()
    x, y, z = t.centroid
    s2 = lambda q: np.sin(2.0 * np.pi * q)
    rho = 1.0 + 0.1 * s2(x) * s2(y + 0.25) * s2(z + 0.1)
    U = cases.conservative_ideal(rho, 0.2 * s2(y), 0.1 * s2(z), 0.15 * s2(x), 1.0 + 0.05 * s2(x + y))
    c = cases.Case("small", t, U, SolverConfig(model=1, ischeme=2), cfl=0.5, nsteps=3)
    dt = fixed_dt(c)
    a = _mixed_state(c, 0, 3, dt)
    b = _mixed_state(c, abi.FLAG_NO_BRICKS, 3, dt)
    if bricks_throughout(t):
        assert np.all(rel_l2_mom(a, b) <= 1e-6), rel_l2_mom(a, b)
    else:
        assert np.array_equal(a.view(np.int64), b.view(np.int64))
    ref = run(c, abi.FP64, 3, dt)
    assert np.all(rel_l2(a, ref) <= 1e-6) and np.all(rel_l2(b, ref) <= 1e-6)

