"""The dual-number restatement (oracle/fvoracle_ad.cpp) against the reference.

With T = double it must reproduce the reference's golden residuals and RK
steps bit for bit; its tangents must agree with central differences of the
oracle.  This pins the CPU reference gradient the GPU adjoint is tested
against.
"""
import numpy as np
import pytest

from fvtest import bits_equal, load_golden
from pyoracle import Oracle, OracleAD

AD_CASES = ["amr_periodic_first", "amr_periodic_muscl", "inflow_l3", "sod_l3", "tgv_l3"]


@pytest.mark.parametrize("name", AD_CASES)
def test_ad_residual_and_steps_match_reference_golden(name):
    t, cfg, z = load_golden(name)
    ad = OracleAD(t, cfg)
    U = z["U"]
    assert bits_equal(ad.residual(U), z["R"])
    S, JV = ad.steps_jvp(U, np.zeros_like(U), float(z["dt"]), str(z["scheme"]), int(z["nsteps"]))
    assert bits_equal(S, z["S_out"])
    assert not np.any(JV)


# Sod's piecewise-constant state sits on the minmod kink everywhere (a zero
# jump takes the |d0| <= 1e-10 branch; any perturbation leaves it), so the
# residual has no derivative there and central differences are meaningless.
@pytest.mark.parametrize("name", [c for c in AD_CASES if c not in ("sod_l3", "tgv_l3")])
def test_ad_jvp_matches_central_differences(name):
    t, cfg, z = load_golden(name)
    ad, orc = OracleAD(t, cfg), Oracle(t, cfg)
    U = z["U"]
    rng = np.random.default_rng(7)
    V = rng.standard_normal(U.shape) * np.abs(U).mean(axis=1, keepdims=True)
    R, JV = ad.jvp(U, V)
    assert bits_equal(R, z["R"])
    eps = 1e-6
    fd = (orc.residual(U + eps * V) - orc.residual(U - eps * V)) / (2 * eps)
    err = np.linalg.norm(JV - fd) / np.linalg.norm(fd)
    assert err <= 1e-6, err


def test_ad_viscous_jvp_matches_central_differences():
    """Gradients (gradcalc) and viscous fluxes (flux_viscous, energy work term
    on and off).  The Taylor-Green state's symmetries put minmod kinks
    everywhere, so it is perturbed by 0.1 % seeded noise; the viscous part of
    the tangent (tangent at visc minus tangent at visc = 0) is compared on its
    own, with viscosity raised so that it stands above the difference noise."""
    import dataclasses
    t, cfg, z = load_golden("tgv_l3")
    rng = np.random.default_rng(5)
    U = z["U"] * (1 + 1e-3 * rng.standard_normal(z["U"].shape))
    U[3] += 1e-3 * rng.standard_normal(U.shape[1])
    V = rng.standard_normal(U.shape) * np.abs(U).mean(axis=1, keepdims=True)
    eps = 1e-7
    for eos in (0, 1):
        parts = []
        for visc in (0.5, 0.0):
            c = dataclasses.replace(cfg, visc=visc, eos=eos)
            ad, orc = OracleAD(t, c), Oracle(t, c)
            R, JV = ad.jvp(U, V)
            assert bits_equal(R, orc.residual(U))
            fd = (orc.residual(U + eps * V) - orc.residual(U - eps * V)) / (2 * eps)
            parts.append((JV, fd))
        dj, dfd = parts[0][0] - parts[1][0], parts[0][1] - parts[1][1]
        err = np.linalg.norm(dj - dfd) / np.linalg.norm(dfd)
        assert err <= 1e-3, (eos, err)


def test_ad_step_tangent_matches_central_differences():
    t, cfg, z = load_golden("amr_periodic_muscl")
    ad, orc = OracleAD(t, cfg), Oracle(t, cfg)
    U, dt = z["U"], float(z["dt"])
    rng = np.random.default_rng(11)
    V = rng.standard_normal(U.shape) * np.abs(U).mean(axis=1, keepdims=True)
    # two steps: in the third a minmod branch of one cell flips within
    # U +- 1e-6 V, and a difference across a kink is no derivative
    _, JV = ad.steps_jvp(U, V, dt, "ssprk3", 2)
    eps = 1e-6
    fd = (orc.step(U + eps * V, dt, "ssprk3", 2) - orc.step(U - eps * V, dt, "ssprk3", 2)) / (2 * eps)
    err = np.linalg.norm(JV - fd) / np.linalg.norm(fd)
    assert err <= 1e-6, err


def test_fp64_operation_counts_match_committed_figures():
    """profiles/traffic.json carries the FP64 operation counts bench.py uses for
    the FP64 path's roofline; recount them (smaller mesh, same generator)."""
    import json
    import os

    from fv_140823_gb300 import cases
    with open(os.path.join(os.path.dirname(__file__), "..", "profiles", "traffic.json")) as fh:
        figs = json.load(fh)["fp64_ops"]
    c = cases.periodic(level=6)
    dt = Oracle(c.tables, c.cfg).cfl_dt(c.U, 0.5)
    fi, rr = OracleAD(c.tables, c.cfg).count_stage(c.U, 3, dt)
    n = c.tables.ncells
    assert rr.sum() / n == figs["residual_per_cell"]      # no data-dependent branch in the residual's count
    assert abs(fi.sum() / n - figs["faceinterp_per_cell"]) <= 0.01
