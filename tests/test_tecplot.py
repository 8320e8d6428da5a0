"""Tecplot export (exportfield_linked_V3.c:19-572) against the reference's own
writer: the file digests in tests/golden/tecplot.json come from the reference
writer run by oracle/_ref on the golden cases (make_golden.py tecplot).  Here
the host writer (libfvmesh) is fed the oracle's state and gradients; the GPU
test feeds it device downloads."""
import hashlib
import json
import os

import numpy as np
import pytest

from fvtest import GOLDEN_DIR, load_golden
from fv_140823_gb300 import tecplot
from fv_140823_gb300.mesh import refine_by, uniform_mesh

import pyoracle
from pyoracle import Oracle, PhysConfig, RefHarness

with open(os.path.join(GOLDEN_DIR, "tecplot.json")) as _fh:
    GOLDEN = json.load(_fh)


def sha256(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


@pytest.mark.parametrize("key", sorted(GOLDEN))
def test_writer_matches_reference_file(key, tmp_path):
    g = GOLDEN[key]
    t, cfg, z = load_golden(g["fixture"])
    orc = Oracle(t, cfg)
    S = z["U"]
    if g["steps"]:
        S = orc.step(S, float(z["dt"]), str(z["scheme"]), g["steps"])
    SG = orc.gradcalc(S)
    path = tecplot.write_field_linked(str(tmp_path / tecplot.file_name(g["tstep"])), t, S, SG, model=cfg.model,
                                      gamma=cfg.gamma, pinf=cfg.pinf, root_level=g["root_level"])
    assert os.path.getsize(path) == g["bytes"]
    with open(path, "rb") as fh:
        lines = fh.read().split(b"\n")
    assert lines[1].decode() == g["zone"] and lines[2].decode() == g["first_point"]
    assert sha256(path) == g["sha256"]


def _ref_available():
    return os.path.isfile(pyoracle.REF_LIB)


@pytest.mark.skipif(not _ref_available(), reason="the reference's objects (oracle/_ref) are not built here")
@pytest.mark.parametrize("periodic", [(1, 1, 1), (0, 1, 0)])
def test_writer_matches_reference_writer_on_amr(periodic, tmp_path):
    """Deeper AMR than the fixtures (levels 2..5), byte for byte against the
    reference writer run here."""
    rng = np.random.default_rng(7)
    m = uniform_mesh(2, periodic=periodic)
    c0 = rng.uniform(0.3, 0.7, 3)
    refine_by(m, lambda l, c: ((c - c0[:, None]) ** 2).sum(0) < 0.015 * (6 - l), 5)
    t = m.flatten()
    n = t.ncells
    U = np.zeros((5, n))
    U[0] = 1.0 + 0.3 * rng.random(n)
    U[1:4] = 0.3 * rng.standard_normal((3, n))
    U[4] = 2.5 + 0.5 * rng.random(n)
    from fv_140823_gb300.abi import SolverConfig

    cfg = SolverConfig(model=1, ischeme=2)
    ref = RefHarness(t, PhysConfig(model=1, ns=0, ischeme=2, iprimtv=0, eos=0, i_case=0, gamma=1.4, pinf=0.0,
                                   visc=0.0, ymin=0.0, dt=1e-3))
    try:
        ref.set_state(U)
        (tmp_path / "ref").mkdir()
        p_ref = ref.export(2, 3, str(tmp_path / "ref"))
    finally:
        ref.close()
    p_our = tecplot.write_field_linked(str(tmp_path / tecplot.file_name(3)), t, U, Oracle(t, cfg).gradcalc(U),
                                       model=1, gamma=1.4, pinf=0.0, root_level=2)
    with open(p_ref, "rb") as a, open(p_our, "rb") as b:
        assert a.read() == b.read()


@pytest.mark.skipif(not _ref_available(), reason="the reference's objects (oracle/_ref) are not built here")
def test_writer_matches_reference_writer_model2(tmp_path):
    """The barotropic liquid (model 2, four variables, barotropic_eos.c:3-30
    for the pressure column) on an AMR mesh, against the reference writer."""
    rng = np.random.default_rng(11)
    m = uniform_mesh(2)
    refine_by(m, lambda l, c: ((c - 0.5) ** 2).sum(0) < 0.04, 4)
    t = m.flatten()
    n = t.ncells
    U = np.vstack([997.0 + 3.0 * rng.random(n), 0.1 * rng.standard_normal((3, n))])
    from fv_140823_gb300.abi import SolverConfig

    cfg = SolverConfig(model=2, ischeme=1)
    ref = RefHarness(t, PhysConfig(model=2, ns=0, ischeme=1, iprimtv=0, eos=0, i_case=0, gamma=1.4, pinf=0.0,
                                   visc=0.0, ymin=0.0, dt=1e-3))
    try:
        ref.set_state(U)
        (tmp_path / "ref").mkdir()
        p_ref = ref.export(2, 5, str(tmp_path / "ref"))
    finally:
        ref.close()
    p_our = tecplot.write_field_linked(str(tmp_path / tecplot.file_name(5)), t, U, Oracle(t, cfg).gradcalc(U),
                                       model=2, gamma=1.4, pinf=0.0, root_level=2)
    with open(p_ref, "rb") as a, open(p_our, "rb") as b:
        assert a.read() == b.read()


def test_links_are_shared_corners(tmp_path):
    """Uniform 4^3 non-periodic: 5^3 links, each leaf's 8 link numbers are its
    corners on the 5^3 lattice, one-based, in Tecplot brick order."""
    t = uniform_mesh(2).flatten()
    n = t.ncells
    U = np.tile(np.array([[1.0], [0.0], [0.0], [0.0], [2.5]]), (1, n))
    p = tecplot.write_field_linked(str(tmp_path / "f.dat"), t, U, None, model=1, gamma=1.4, pinf=0.0)
    lines = open(p).read().split("\n")
    assert lines[0].startswith(' VARIABLES =  "X" "Y" "Z" "iel" "part" "rho"') and lines[0].endswith(" ")
    assert lines[1] == ' ZONE T="1",N=125,E=64,F=FEPOINT,ET=BRICK,DT=(double,double,double)'
    pts = [list(map(float, ln.split())) for ln in lines[2:2 + 125]]
    xyz = {tuple(round(v * 4) for v in p[:3]): i + 1 for i, p in enumerate(pts)}
    assert len(xyz) == 125
    assert all(p[5] == 1.0 and p[10] == 1.0 for p in pts)  # rho, P = (gamma - 1) rho e
    brick = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for c in range(n):
        ids = list(map(int, lines[2 + 125 + c].split()))
        want = [xyz[tuple(int(t.ijk[a, c]) + o[a] for a in range(3))] for o in brick]
        assert ids == want


def test_rejects_bad_input(tmp_path):
    t = uniform_mesh(2).flatten()
    U = np.ones((5, t.ncells))
    with pytest.raises(RuntimeError, match="coarser than root_level"):
        tecplot.write_field_linked(str(tmp_path / "f.dat"), t, U, None, model=1, gamma=1.4, pinf=0.0, root_level=3)
    with pytest.raises(ValueError):
        tecplot.write_field_linked(str(tmp_path / "f.dat"), t, U[:4], None, model=1, gamma=1.4, pinf=0.0)
    with pytest.raises(RuntimeError, match="cannot open"):
        tecplot.write_field_linked(str(tmp_path / "no" / "f.dat"), t, U, None, model=1, gamma=1.4, pinf=0.0)
