"""Adjoint of the FP64 residual and of RK steps (hand-written reverse kernels).

Checks, on the GPU through the C ABI:
  * transposition: <w, J v> from the dual-number oracle (exact forward-mode
    derivative of the reference arithmetic) equals <J^T w, v> from the GPU
    adjoint, on the reference's golden meshes (AMR 1:4 faces, periodic,
    inflow and transmissive boundaries, first order and MUSCL);
  * the full gradient J^T w against the CPU FP64 reference gradient built
    column by column from the oracle's tangents;
  * multi-step adjoints (per-step checkpoints) of Euler / SSP-RK2 / SSP-RK3
    against the oracle's step tangents, and the state they leave;
  * a functional J(U^1) = sum_{x > 0.75} p V after one SSP-RK3 step against
    central differences (h 1e-6) on 64 seeded entries, with kinks flagged;
    the same on the C4 AMR workload after one forward-Euler stage;
  * the viscous residual (gradients and viscous fluxes): transposition on the
    Taylor-Green golden, ten-step adjoints against the oracle's tangents and,
    on the C5 workload, the kinetic energy after ten steps against central
    differences;
  * determinism, the torch.autograd wrappers, unsupported configurations.
Tolerances: the oracle and the GPU differentiate the same branch of the same
arithmetic, so they differ by rounding only (relative 1e-11 on dot products
and 1e-10 on gradients); central differences carry O(h^2) truncation and
cancellation error (bound stated in the test).
"""
import numpy as np
import pytest

from fv_140823_gb300 import abi, cases
from fv_140823_gb300.abi import SolverConfig
from fvtest import bits_equal, load_golden
from pyoracle import Oracle, OracleAD

pytestmark = pytest.mark.gpu

AD_CASES = ["amr_periodic_first", "amr_periodic_muscl", "inflow_l3", "sod_l3", "tgv_l3"]


def solver(t, cfg):
    from fv_140823_gb300.solver import Solver
    return Solver(t, cfg)


def scaled_random(rng, U):
    return rng.standard_normal(U.shape) * np.abs(U).mean(axis=1, keepdims=True)


@pytest.mark.parametrize("name", AD_CASES)
def test_residual_vjp_transposes_oracle_jvp(name):
    t, cfg, z = load_golden(name)
    U = z["U"]
    rng = np.random.default_rng(3)
    V, W = scaled_random(rng, U), rng.standard_normal(U.shape)
    _, JV = OracleAD(t, cfg).jvp(U, V)
    with solver(t, cfg) as s:
        s.set_state(U)
        g = s.residual_vjp(W)
    lhs, rhs = float(np.sum(W * JV)), float(np.sum(g * V))
    assert abs(lhs - rhs) <= 1e-11 * max(np.abs(W * JV).sum(), 1e-300), (lhs, rhs)


@pytest.mark.parametrize("name", ["amr_periodic_muscl", "inflow_l3", "tgv_l3"])
def test_residual_vjp_full_gradient_matches_cpu_reference(name):
    t, cfg, z = load_golden(name)
    U = z["U"]
    ad = OracleAD(t, cfg)
    rng = np.random.default_rng(5)
    W = rng.standard_normal(U.shape)
    ref = np.empty(U.size)
    E = np.zeros(U.size)
    for i in range(U.size):  # column i of J, dotted with w
        E[i] = 1.0
        ref[i] = np.sum(W * ad.jvp(U, E.reshape(U.shape))[1])
        E[i] = 0.0
    with solver(t, cfg) as s:
        s.set_state(U)
        g = s.residual_vjp(W)
    err = np.abs(g.ravel() - ref).max() / np.abs(ref).max()
    assert err <= 1e-10, err


@pytest.mark.parametrize("name,scheme", [("amr_periodic_muscl", "ssprk3"), ("amr_periodic_first", "ssprk2"),
                                         ("inflow_l3", "euler"), ("amr_periodic_muscl", "ssprk2"),
                                         ("sod_l3", "ssprk3"), ("tgv_l3", "ssprk3")])
def test_adjoint_steps_transposes_oracle_step_tangent(name, scheme):
    t, cfg, z = load_golden(name)
    U, dt, nsteps = z["U"], float(z["dt"]), 3
    rng = np.random.default_rng(9)
    V, G = scaled_random(rng, U), rng.standard_normal(U.shape)
    S_ref, JV = OracleAD(t, cfg).steps_jvp(U, V, dt, scheme, nsteps)
    with solver(t, cfg) as s:
        s.set_state(U)
        g0 = s.adjoint_steps(G, dt, scheme, nsteps)
        S_after = s.state()
    assert bits_equal(S_after, S_ref)  # the forward sweep is the FP64 step, bit for bit
    lhs, rhs = float(np.sum(G * JV)), float(np.sum(g0 * V))
    assert abs(lhs - rhs) <= 1e-11 * max(np.abs(G * JV).sum(), 1e-300), (lhs, rhs)


def _pressure_functional(t, gamma):
    mask = t.centroid[0] > 0.75
    vol = t.vol

    def J(S):
        r, m, E = S[0], S[1:4], S[4]
        p = (gamma - 1.0) * (E - 0.5 * (m * m).sum(axis=0) / r)
        return float(np.sum((p * vol)[mask]))

    def dJ(S):
        r, m, E = S[0], S[1:4], S[4]
        g = np.zeros_like(S)
        w = (gamma - 1.0) * vol * mask
        g[0] = w * 0.5 * (m * m).sum(axis=0) / (r * r)
        g[1:4] = -w * m / r
        g[4] = w
        return g
    return J, dJ


def test_functional_gradient_matches_central_differences():
    """J = sum_{x > 0.75} p V after one SSP-RK3 step; central differences with
    the absolute step h = 1e-6 on 64 seeded entries.  The smooth periodic flow
    is perturbed by 0.1% seeded noise: its symmetric density field puts exact
    ties between neighbours (a zero jump, the minmod kink) on an 8^3 mesh.
    Tolerance: 1e-5 |g| plus the rounding bound of the difference quotient,
    10 u sum|p V| / h; an entry whose one-sided slopes disagree sits at a kink
    and is counted, not compared."""
    c = cases.periodic(level=3)
    t, cfg = c.tables, c.cfg
    U = c.U * (1.0 + 1e-3 * np.random.default_rng(77).standard_normal(c.U.shape))
    J, dJ = _pressure_functional(t, cfg.gamma)
    h, u = 1e-6, 2.0 ** -53
    with solver(t, cfg) as s:
        s.set_state(U)
        dt = s.compute_dt(0.5)
        s.step("ssprk3", dt=dt, nsteps=1)
        S1 = s.state()
        s.set_state(U)
        g = s.adjoint_steps(dJ(S1), dt, "ssprk3", 1)
        assert bits_equal(s.state(), S1)

        def Jat(Up):
            s.set_state(Up)
            s.step("ssprk3", dt=dt, nsteps=1)
            return J(s.state())

        J0 = J(S1)
        r, m, E = S1[0], S1[1:4], S1[4]
        p_abs = np.abs((cfg.gamma - 1.0) * (E - 0.5 * (m * m).sum(axis=0) / r) * t.vol)
        noise = 10 * u * float(p_abs[t.centroid[0] > 0.75].sum()) / h
        gmax = np.abs(g).max()
        live = np.flatnonzero(np.abs(g).ravel() > 1e-3 * gmax)
        rng = np.random.default_rng(2024)
        bad, kinks = [], []
        for i in rng.choice(live, size=64, replace=False):
            v, c_ = np.unravel_index(i, U.shape)
            Up, Um = U.copy(), U.copy()
            Up[v, c_] += h
            Um[v, c_] -= h
            Jp, Jm = Jat(Up), Jat(Um)
            fd = (Jp - Jm) / (2 * h)
            fwd, bwd = (Jp - J0) / h, (J0 - Jm) / h
            if abs(fwd - bwd) > 1e-3 * abs(fd) + 4 * noise:
                kinks.append(int(i))
                continue
            if abs(fd - g[v, c_]) > 1e-5 * abs(g[v, c_]) + noise:
                bad.append((int(i), fd, g[v, c_]))
    assert len(kinks) <= 2, kinks
    assert not bad, bad


def test_c4_functional_gradient_forward_euler_central_differences():
    """The C4 workload: level-5 base + 2 levels inside a sphere (105,113
    cells, 1:4 faces), J = sum_{x_c > 0.75} p(U1) V with U1 = U + dt R(U) / V
    (one forward-Euler stage); gradient with respect to all of U from the
    adjoint, central differences (h 1e-6) on 64 seeded random cells (every
    variable of each), kinks flagged as above."""
    c = cases.bump(base_level=5, extra_levels=2)
    t, cfg, U = c.tables, c.cfg, c.U
    J, dJ = _pressure_functional(t, cfg.gamma)
    h, u = 1e-6, 2.0 ** -53
    with solver(t, cfg) as s:
        s.set_state(U)
        dt = s.compute_dt(0.5)
        s.step("euler", dt=dt, nsteps=1)
        S1 = s.state()
        s.set_state(U)
        g = s.adjoint_steps(dJ(S1), dt, "euler", 1)

        def Jat(Up):
            s.set_state(Up)
            s.step("euler", dt=dt, nsteps=1)
            return J(s.state())

        J0 = J(S1)
        r, m, E = S1[0], S1[1:4], S1[4]
        p_abs = np.abs((cfg.gamma - 1.0) * (E - 0.5 * (m * m).sum(axis=0) / r) * t.vol)
        noise = 10 * u * float(p_abs[t.centroid[0] > 0.75].sum()) / h
        rng = np.random.default_rng(64)
        bad, kinks, compared = [], [], 0
        for cell in rng.choice(t.ncells, size=64, replace=False):
            for v in range(U.shape[0]):
                Up, Um = U.copy(), U.copy()
                Up[v, cell] += h
                Um[v, cell] -= h
                Jp, Jm = Jat(Up), Jat(Um)
                fd = (Jp - Jm) / (2 * h)
                if abs((Jp - J0) / h - (J0 - Jm) / h) > 1e-3 * abs(fd) + 4 * noise:
                    kinks.append((int(cell), v))
                    continue
                compared += 1
                if abs(fd - g[v, cell]) > 1e-5 * abs(g[v, cell]) + noise:
                    bad.append((int(cell), v, fd, g[v, cell]))
    assert compared >= 300 and len(kinks) <= 20, kinks
    assert not bad, bad


def _kinetic_energy(vol):
    def J(S):
        return float(np.sum(0.5 * (S[1:4] ** 2).sum(axis=0) / S[0] * vol))

    def dJ(S):
        g = np.zeros_like(S)
        g[0] = -0.5 * (S[1:4] ** 2).sum(axis=0) / (S[0] * S[0]) * vol
        g[1:4] = S[1:4] / S[0] * vol
        return g
    return J, dJ


def test_viscous_ten_step_adjoint_transposes_oracle_tangent():
    """Ten SSP-RK3 steps of the viscous Taylor-Green flow (levels 3-4, 1:4
    faces, energy work term): <G, J v> (dual-number oracle through the ten
    steps) = <J^T G, v> (GPU, one checkpoint per step)."""
    c = cases.tgv(base_level=3, extra_levels=1)
    t, cfg, U = c.tables, c.cfg, c.U
    with solver(t, cfg) as s:
        s.set_state(U)
        dt = s.compute_dt(0.5)
    rng = np.random.default_rng(10)
    V, G = scaled_random(rng, U), rng.standard_normal(U.shape)
    S_ref, JV = OracleAD(t, cfg).steps_jvp(U, V, dt, "ssprk3", 10)
    with solver(t, cfg) as s:
        s.set_state(U)
        g0 = s.adjoint_steps(G, dt, "ssprk3", 10)
        assert bits_equal(s.state(), S_ref)
    lhs, rhs = float(np.sum(G * JV)), float(np.sum(g0 * V))
    assert abs(lhs - rhs) <= 1e-11 * max(np.abs(G * JV).sum(), 1e-300), (lhs, rhs)


def test_c5_kinetic_energy_ten_step_adjoint_central_differences():
    """The C5 workload: viscous Taylor-Green vortex, Re 1600, Mach 0.1, levels
    5-7 by vorticity (179,712 cells); J = kinetic energy after ten SSP-RK3
    steps; gradient through the ten steps with one checkpoint per step,
    against central differences (h 1e-6) on 64 seeded cells (every variable).
    The vortex's symmetries put exact minmod ties between neighbours, so the
    state is perturbed by 0.1 % seeded noise first; entries whose one-sided
    slopes disagree sit at a branch switch (kink) and are counted, not
    compared.  Differences over ten steps resolve the gradient to about 1e-4
    (branch switches just outside +-h, rounding in ~1e4 touched cells); the
    exact transposition is checked to 1e-11 by the dual-number tests above."""
    c = cases.tgv(base_level=5, extra_levels=2)
    t, cfg = c.tables, c.cfg
    rng = np.random.default_rng(55)
    U = c.U * (1.0 + 1e-3 * rng.standard_normal(c.U.shape))
    U[3] += 1e-3 * rng.standard_normal(U.shape[1])
    J, dJ = _kinetic_energy(t.vol)
    h, u, nsteps = 1e-6, 2.0 ** -53, 10
    with solver(t, cfg) as s:
        s.set_state(U)
        dt = s.compute_dt(0.5)
        s.step("ssprk3", dt=dt, nsteps=nsteps)
        SN = s.state()
        s.set_state(U)
        g = s.adjoint_steps(dJ(SN), dt, "ssprk3", nsteps)

        def ke(S):  # per-cell contributions: differences are taken cell by cell
            return 0.5 * (S[1:4] ** 2).sum(axis=0) / S[0] * t.vol

        def Kat(Up):
            s.set_state(Up)
            s.step("ssprk3", dt=dt, nsteps=nsteps)
            return ke(s.state())

        K0 = ke(SN)
        kmax = float(np.abs(K0).max())
        bad, kinks, compared = [], [], 0
        for cell in rng.choice(t.ncells, size=64, replace=False):
            for v in range(U.shape[0]):
                Up, Um = U.copy(), U.copy()
                Up[v, cell] += h
                Um[v, cell] -= h
                Kp, Km = Kat(Up), Kat(Um)
                touched = int(np.count_nonzero((Kp != K0) | (Km != K0)))
                # rounding of the cell-by-cell differences: independent errors of
                # a few ulp in every touched cell
                noise = 10 * u * kmax * np.sqrt(max(touched, 1)) / h
                fd = float(np.sum(Kp - Km)) / (2 * h)
                fwd, bwd = float(np.sum(Kp - K0)) / h, float(np.sum(K0 - Km)) / h
                # over ten steps a branch switch inside [-h, h] bends the slope
                # only slightly: flag one-sided disagreements above the
                # comparison tolerance (a smooth J bends by h J'' ~ 1e-6 |J'|)
                if abs(fwd - bwd) > 2e-4 * abs(fd) + 4 * noise:
                    kinks.append((int(cell), v))
                    continue
                compared += 1
                if abs(fd - g[v, cell]) > 2e-4 * abs(g[v, cell]) + 2 * noise:
                    bad.append((int(cell), v, fd, g[v, cell]))
    # ten steps spread a perturbation over many cells: about 8 % of the 320
    # entries meet a branch switch within +-h
    assert compared >= 280 and len(kinks) <= 40, kinks
    assert not bad, bad


def test_adjoint_is_deterministic():
    c = cases.periodic(level=4)
    rng = np.random.default_rng(1)
    W = rng.standard_normal(c.U.shape)
    outs = []
    for _ in range(2):
        with solver(c.tables, c.cfg) as s:
            s.set_state(c.U)
            outs.append(s.residual_vjp(W))
            s.set_state(c.U)
            outs.append(s.adjoint_steps(W, 1e-3, "ssprk3", 2))
    assert bits_equal(outs[0], outs[2]) and bits_equal(outs[1], outs[3])


def test_autograd_wrappers():
    torch = pytest.importorskip("torch")
    from fv_140823_gb300.autograd import residual, steps
    t, cfg, z = load_golden("amr_periodic_muscl")
    U0, dt = z["U"], float(z["dt"])
    rng = np.random.default_rng(4)
    Wt = torch.from_numpy(rng.standard_normal(U0.shape))
    with solver(t, cfg) as s:
        U = torch.tensor(U0, requires_grad=True)
        R = residual(s, U)
        assert bits_equal(R.detach().numpy(), z["R"])
        (R * Wt).sum().backward()
        s.set_state(U0)
        assert bits_equal(U.grad.numpy(), s.residual_vjp(Wt.numpy()))
        U = torch.tensor(U0, requires_grad=True)
        S = steps(s, U, dt, "ssprk3", 2)
        assert bits_equal(S.detach().numpy(), Oracle(t, cfg).step(U0, dt, "ssprk3", 2))
        (S * Wt).sum().backward()
        s.set_state(U0)
        assert bits_equal(U.grad.numpy(), s.adjoint_steps(Wt.numpy(), dt, "ssprk3", 2))


def test_autograd_wrappers_on_cuda_tensors():
    """CUDA tensors go through the C ABI as device pointers: the same bits as
    the host path, forward and backward, with the results on the device."""
    torch = pytest.importorskip("torch")
    from fv_140823_gb300.autograd import residual, steps
    t, cfg, z = load_golden("amr_periodic_muscl")
    U0, dt = z["U"], float(z["dt"])
    rng = np.random.default_rng(5)
    W = rng.standard_normal(U0.shape)
    with solver(t, cfg) as s:
        for fn in (lambda U: residual(s, U), lambda U: steps(s, U, dt, "ssprk3", 2)):
            got = []
            for dev in ("cpu", "cuda"):
                U = torch.tensor(U0, device=dev, requires_grad=True)
                out = fn(U)
                assert out.device.type == dev
                (out * torch.from_numpy(W).to(dev)).sum().backward()
                got.append((out.detach().cpu().numpy(), U.grad.cpu().numpy()))
            assert bits_equal(got[0][0], got[1][0]) and bits_equal(got[0][1], got[1][1])


def _mixed_case(name):
    """A golden case for the FP32 reverse passes.  The Taylor-Green state is
    perturbed (relative 1e-3, seeded): on its symmetry planes the HLLC
    contact speed S* is zero in exact arithmetic, FP32 and FP64 round it to
    either sign, and the HLLC flux, continuous there, has different
    derivatives on the two sides."""
    t, cfg, z = load_golden(name)
    U = z["U"]
    if name == "tgv_l3":
        U = U * (1.0 + 1e-3 * np.random.default_rng(11).standard_normal(U.shape))
    return t, cfg, U


# FP32 reverse passes against FP64: (transposition vs the oracle, VJP, 3 SSP-RK3
# steps).  The Sod tube starts at rest, so in its first steps S* sits at the
# HLLC branch point on most faces and the two precisions take either branch.
MIXED_ADJ_TOL = {"amr_periodic_first": (5e-8, 1e-6, 1e-7), "amr_periodic_muscl": (5e-8, 1e-6, 1e-7),
                 "inflow_l3": (5e-8, 1e-6, 1e-7), "sod_l3": (5e-8, 1e-6, 1e-3), "tgv_l3": (5e-8, 1e-4, 1e-3)}


@pytest.mark.parametrize("name", AD_CASES)
def test_mixed_context_adjoint_in_fp32(name):
    """A context on the FP32-mixed path reverses the residual in FP32: it
    still transposes the oracle's exact tangent to FP32 rounding, and its
    VJP and 3-step adjoint stay close to the FP64 ones."""
    t, cfg, U = _mixed_case(name)
    tol_t, tol_v, tol_s = MIXED_ADJ_TOL[name]
    rng = np.random.default_rng(3)
    V, W = scaled_random(rng, U), rng.standard_normal(U.shape)
    _, JV = OracleAD(t, cfg).jvp(U, V)
    g = {}
    for prec in (abi.FP64, abi.MIXED):
        with solver(t, SolverConfig(**{**cfg.__dict__, "precision": prec})) as s:
            s.set_state(U)
            g[prec] = s.residual_vjp(W)
            s.set_state(U)
            g[("steps", prec)] = s.adjoint_steps(W, 1e-3, "ssprk3", 3)
    lhs, rhs = float(np.sum(W * JV)), float(np.sum(g[abi.MIXED] * V))
    assert abs(lhs - rhs) <= tol_t * np.abs(W * JV).sum(), (lhs, rhs)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(g[abi.MIXED], g[abi.FP64]) <= tol_v, rel(g[abi.MIXED], g[abi.FP64])
    assert rel(g[("steps", abi.MIXED)], g[("steps", abi.FP64)]) <= tol_s


@pytest.mark.parametrize("name", ["bubble_l3"])
def test_adjoint_rejects_unsupported(name):
    from fv_140823_gb300.solver import FvGpuError
    t, cfg, z = load_golden(name)
    with solver(t, cfg) as s:
        s.set_state(z["U"])
        with pytest.raises(FvGpuError) as ei:
            s.residual_vjp(np.ones_like(z["U"]))
    assert ei.value.code == abi.ERR_UNSUPPORTED


def test_adjoint_cost_within_three_residuals():
    c = cases.periodic(level=6)
    with solver(c.tables, SolverConfig(**{**c.cfg.__dict__, "precision": abi.FP64})) as s:
        s.set_state(c.U)
        ms_res, ms_vjp = s.profile_adjoint(reps=5)
    assert ms_vjp <= 3.0 * ms_res, (ms_res, ms_vjp)
