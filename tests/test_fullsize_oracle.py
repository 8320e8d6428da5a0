"""The oracle at the Sod workload's full size: the C restatement run as
configured (32^3 leaves, MUSCL/minmod + HLLC, SSP-RK3, CFL 0.5, 100 steps)
ends in the same bits as the reference's own code
(tests/golden/fullsize.json, made by make_golden.py from oracle/_ref)."""
import json
import os
import sys

import numpy as np

from fv_140823_gb300 import cases

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def test_oracle_sod32_100_steps_matches_reference_digest():
    from make_golden import state_digest
    from pyoracle import Oracle
    with open(os.path.join(HERE, "golden", "fullsize.json")) as fh:
        want = json.load(fh)["c1_sod32_ssprk3_cfl05_100"]
    Oracle.set_threads(os.cpu_count() or 1)
    c = cases.sod(level=5)
    orc = Oracle(c.tables, c.cfg)
    S = c.U
    dts = []
    for _ in range(100):
        dts.append(orc.cfl_dt(S, 0.5))
        S = orc.step(S, dts[-1], "ssprk3", 1)
    assert dts[0] == want["dt_first"] and dts[-1] == want["dt_last"]
    assert np.allclose(S.sum(axis=1), want["field_sums"], rtol=1e-12, atol=1e-12)
    assert state_digest(S) == want["sha256"]
