"""Tecplot export fed from the device (loop.c:50-55: gradcalc on the GPU,
state and gradients downloaded, the host writer in libfvmesh) against the
digests of the reference writer's files (tests/golden/tecplot.json, made by
the reference's exportfield_linked_V3 through oracle/_ref).  The FP64 state
and gradients on the device are the reference's bit for bit, so the files
must be identical byte for byte."""
import hashlib
import json
import os

import numpy as np
import pytest

from fv_140823_gb300 import abi, tecplot
from fvtest import GOLDEN_DIR, load_golden

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN_DIR, "tecplot.json")) as _fh:
    GOLDEN = json.load(_fh)


@pytest.mark.parametrize("key", sorted(GOLDEN))
def test_device_export_matches_reference_file(key, tmp_path):
    from fv_140823_gb300.solver import Solver

    g = GOLDEN[key]
    t, cfg, z = load_golden(g["fixture"])
    with Solver(t, cfg) as s:
        s.set_state(z["U"])
        if g["steps"]:
            s.step(str(z["scheme"]), dt=float(z["dt"]), nsteps=g["steps"])
        path = tecplot.export_solver(s, t, str(tmp_path), g["tstep"], root_level=g["root_level"])
    assert os.path.basename(path) == "field_linked%08dprt00.dat" % g["tstep"]
    with open(path, "rb") as fh:
        data = fh.read()
    assert len(data) == g["bytes"]
    assert hashlib.sha256(data).hexdigest() == g["sha256"]


def test_mixed_context_export(tmp_path):
    """A mixed-precision run exports its FP64 state: same links and
    connectivity as the FP64 run's file, values within the mixed path's error."""
    from fv_140823_gb300.solver import Solver

    g = GOLDEN["amr_periodic_muscl/steps2/root2"]
    t, cfg, z = load_golden(g["fixture"])
    files = []
    for prec in (abi.FP64, abi.MIXED):
        with Solver(t, cfg) as s:
            s.set_precision(prec)
            s.set_state(z["U"])
            s.step(str(z["scheme"]), dt=float(z["dt"]), nsteps=g["steps"])
            d = tmp_path / str(prec)
            d.mkdir()
            files.append(open(tecplot.export_solver(s, t, str(d), 12, root_level=2)).read().split("\n"))
    a, b = files
    assert len(a) == len(b) and a[:2] == b[:2]
    npts = int(a[1].split("N=")[1].split(",")[0])
    assert a[2 + npts:] == b[2 + npts:]  # connectivity
    pa = np.array([list(map(float, ln.split())) for ln in a[2:2 + npts]])
    pb = np.array([list(map(float, ln.split())) for ln in b[2:2 + npts]])
    assert np.array_equal(pa[:, :5], pb[:, :5])  # coordinates, iel, part
    # conserved means and pressure: mixed error ~1e-7, printed to 7 digits
    np.testing.assert_allclose(pb[:, 5:11], pa[:, 5:11], rtol=2e-6, atol=1e-6)
