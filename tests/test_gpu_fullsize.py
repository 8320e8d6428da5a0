"""The FP64 GPU path at the workloads' full sizes and step counts.

* C1: the 3-D Sod tube as configured (32^3 leaves, MUSCL/minmod + HLLC,
  SSP-RK3, CFL 0.5, 100 steps): the final state's SHA-256 equals the one of
  the reference's own code run the same way (tests/golden/fullsize.json,
  made by make_golden.py from oracle/_ref).
* C3: the 128^3 periodic case, two CFL SSP-RK3 steps, bit for bit against the
  oracle (the reference's path restated in C, pinned to the reference's code
  bit for bit on smaller meshes) on the host's cores.
* C2: the two-phase bubble (16^3 + 3 levels), 200 CFL steps with a mesh
  adaptation every 10 (criterion on the device, host refine / merge with
  state transfer, re-upload): bit for bit against the oracle driven through
  the same adaptations; and the FP32-mixed path on the same meshes within
  1e-6 of FP64 per field.
"""
import json
import os
import sys

import numpy as np
import pytest

from fv_140823_gb300 import abi, cases
from fv_140823_gb300.abi import SolverConfig
from fv_140823_gb300.adaptive import AdaptConfig, run_adaptive, run_adaptive_gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

pytestmark = pytest.mark.gpu

# C2 adaptation: |grad rho| h > 50 kg/m^3 (h = V^(1/3)) asks for the finest
# level, levels 4..7; the mesh first sheds the wide initial refinement band
# (91k -> ~49k leaves), then follows the interface at ~43k leaves
BUBBLE_ADAPT = dict(every=10, kind=abi.CRIT_GRAD_RHO_H, threshold=50.0, min_level=4, max_level=7)


def _solver(t, cfg, precision=abi.FP64):
    from fv_140823_gb300.solver import Solver
    return Solver(t, SolverConfig(**{**cfg.__dict__, "precision": precision}))


def test_sod32_100_steps_match_the_reference_digest():
    from make_golden import state_digest
    with open(os.path.join(HERE, "golden", "fullsize.json")) as fh:
        want = json.load(fh)["c1_sod32_ssprk3_cfl05_100"]
    c = cases.sod(level=5)
    with _solver(c.tables, c.cfg) as s:
        s.set_state(c.U)
        s.step("ssprk3", cfl=0.5, nsteps=100)
        S = s.state()
    assert np.allclose(S.sum(axis=1), want["field_sums"], rtol=1e-12, atol=1e-12)
    assert state_digest(S) == want["sha256"]


def test_periodic128_two_steps_bit_identical_to_oracle():
    from pyoracle import Oracle
    c = cases.periodic(level=7)
    with _solver(c.tables, c.cfg) as s:
        s.set_state(c.U)
        s.step("ssprk3", cfl=0.5, nsteps=2)
        S = s.state()
    Oracle.set_threads(os.cpu_count() or 1)
    orc = Oracle(c.tables, c.cfg)
    R = c.U
    for _ in range(2):
        R = orc.step(R, orc.cfl_dt(R, 0.5), "ssprk3", 1)
    assert np.array_equal(S.view(np.int64), R.view(np.int64))


def _oracle_adaptive(case, nsteps, ac):
    from pyoracle import Oracle, criterion
    box = {"orc": Oracle(case.tables, case.cfg), "t": case.tables, "U": case.U}

    def step(k):
        for _ in range(k):
            box["U"] = box["orc"].step(box["U"], box["orc"].cfl_dt(box["U"], case.cfl), case.scheme, 1)
        return box["U"]

    def crit():
        SG = box["orc"].gradcalc(box["U"])
        return box["U"], criterion(box["U"], SG, box["t"].vol, ac.kind, ac.threshold, ac.max_level)

    def reload(tables, S):
        box["orc"] = Oracle(tables, case.cfg)
        box["t"], box["U"] = tables, S

    return run_adaptive(case.mesh, case.U, nsteps, ac, step, crit, reload)


def test_bubble_200_steps_with_adaptation_bit_identical_to_oracle():
    from pyoracle import Oracle
    Oracle.set_threads(os.cpu_count() or 1)
    ac = AdaptConfig(**BUBBLE_ADAPT)
    c = cases.bubble(base_level=4, extra_levels=3)
    with _solver(c.tables, c.cfg) as s:
        gpu = run_adaptive_gpu(s, c.mesh, c.U, 200, ac, c.scheme, c.cfl)
    c2 = cases.bubble(base_level=4, extra_levels=3)
    ref = _oracle_adaptive(c2, 200, ac)
    assert gpu.steps == ref.steps == 200 and len(gpu.cells) == 19
    assert gpu.cells == ref.cells
    assert len(set(gpu.cells)) > 1 or gpu.cells[0] != c.tables.ncells  # the mesh did change
    assert np.array_equal(gpu.state.view(np.int64), ref.state.view(np.int64))


def test_bubble_200_steps_with_adaptation_mixed_within_1e6():
    """FP64 and FP32-mixed contexts in lockstep on the same meshes (the
    FP64 state's criterion decides every adaptation; both states are
    transferred with the same plan)."""
    ac = AdaptConfig(**BUBBLE_ADAPT)
    c = cases.bubble(base_level=4, extra_levels=3)
    with _solver(c.tables, c.cfg) as s64, _solver(c.tables, c.cfg, abi.MIXED) as s32:
        s64.set_state(c.U)
        s32.set_state(c.U)
        dts = []

        def step(k):
            for _ in range(k):
                dt = s64.compute_dt(c.cfl)
                dts.append(dt)
                s64.step(c.scheme, dt=dt, nsteps=1)
                s32.step(c.scheme, dt=dt, nsteps=1)
            return lambda: (s32.state(), s64.state())

        def crit():
            box["U32"] = s32.state()
            S = s64.state()
            s64.gradcalc()
            return S, s64.criterion(ac.kind, ac.threshold, ac.max_level)

        def reload(tables, S):
            s64.upload_mesh(tables)
            s64.set_state(S)
            s32.upload_mesh(tables)
            s32.set_state(c.mesh.transfer(box["U32"]))

        box = {}
        run = run_adaptive(c.mesh, c.U, 200, ac, step, crit, reload)
    a, b = run.state
    nm = np.linalg.norm(b[1:4])
    err = [np.linalg.norm(a[v] - b[v]) / (nm if v in (1, 2, 3) else np.linalg.norm(b[v])) for v in range(5)]
    assert np.all(np.array(err) <= 1e-6), err
