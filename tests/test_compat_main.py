"""The reference's own host program -- main() (main.c:16-187) and every file
it links, compiled unchanged -- built with the compat layer
(fv_140823_gb300/csrc/compat) and run on decks written by
fv_140823_gb300.decks, in two builds (tests/compat/build_main.py):

* ``cpu``  -- the reference's residual path in its own C code;
* ``shim`` -- RHS, RHS_nb, RK, faceinterp and gradcalc replaced by the drop-in
  shim (csrc/shim/fvshim.c) over a libfvgpu stand-in that computes with the
  oracle (tests/shim/fake_fvgpu.c).

Both must leave the same final state bit for bit and write the same Tecplot
files byte for byte; and the state equals that of the reference's residual
code driven by oracle/_ref on this repository's mesh tables.  CPU only: the
program needs the reference tree, which exists only here.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from fv_140823_gb300 import cases, decks
from fv_140823_gb300.abi import SolverConfig
from fv_140823_gb300.mesh import uniform_mesh

pyoracle = pytest.importorskip("pyoracle")
if not pyoracle.ref_available():
    pytest.skip("reference tree absent: main() is built from the reference's sources", allow_module_level=True)

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "compat"))
import build_main  # noqa: E402  (tests/compat/build_main.py)


@pytest.fixture(scope="module")
def exes():
    out = build_main.build()
    assert out is not None
    return out


def run_main(exe, directory, tables, ctl):
    decks.write_deck(str(directory), "c1", tables, ctl)
    r = subprocess.run([exe, "c1", "r1"], cwd=str(directory), env=dict(os.environ, FVCOMPAT_DUMP="dump.bin"),
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    raw = open(os.path.join(str(directory), "dump.bin"), "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    neq = int(np.frombuffer(raw[8:12], np.int32)[0])
    rec = np.dtype([("root", "<i4"), ("S", "<f8", (neq,)), ("geo", "<f8", (4,))])
    a = np.frombuffer(raw[12:], rec)
    assert len(a) == n
    S = np.empty((neq, n))
    S[:, a["root"]] = a["S"].T  # element (tree) order = the tables' leaf order
    files = {f: open(os.path.join(str(directory), f), "rb").read()
             for f in os.listdir(str(directory)) if f.startswith("field_linked")}
    return S, files


def harness_state(tables, U, ctl, scheme):
    ref = pyoracle.RefHarness(tables, pyoracle.PhysConfig(
        model=ctl.model, ns=ctl.ns, ischeme=ctl.ischeme, iprimtv=0, eos=0, i_case=0, gamma=ctl.gamma,
        pinf=ctl.pinf, visc=ctl.visc, ymin=0.0, dt=ctl.dt))
    try:
        ref.set_state(U)
        ref.step(scheme, ctl.nstep + 1)  # loop.c:35 runs nstep + 1 steps
        return ref.state()
    finally:
        ref.close()


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


def test_main_runs_c1_deck(exes, tmp_path):
    """C1 as configured: Sod tube on 32^3 leaves, MUSCL/minmod + HLLC,
    SSP-RK3, transmissive sides; three steps and an export."""
    c = cases.sod(level=5)
    ctl = decks.DeckControls(nstep=2, dt=2e-3, exstep=2)
    (tmp_path / "cpu").mkdir()
    (tmp_path / "shim").mkdir()
    S_cpu, f_cpu = run_main(exes["cpu"], tmp_path / "cpu", c.tables, ctl)
    S_shim, f_shim = run_main(exes["shim"], tmp_path / "shim", c.tables, ctl)
    assert np.array_equal(bits(S_cpu), bits(S_shim))
    assert sorted(f_cpu) == ["field_linked00000000prt00.dat", "field_linked00000002prt00.dat"]
    assert f_cpu == f_shim
    assert np.array_equal(bits(S_cpu), bits(harness_state(c.tables, c.U, ctl, "ssprk3")))


@pytest.mark.parametrize("method,scheme", [(1, "euler"), (2, "ssprk2")])
def test_main_first_order_and_rk_method(exes, tmp_path, method, scheme):
    """First-order faces, the deck's RK method read by both builds."""
    c = cases.sod(level=3)
    ctl = decks.DeckControls(nstep=3, dt=2e-3, ischeme=1, method=method)
    (tmp_path / "cpu").mkdir()
    (tmp_path / "shim").mkdir()
    S_cpu, _ = run_main(exes["cpu"], tmp_path / "cpu", c.tables, ctl)
    S_shim, _ = run_main(exes["shim"], tmp_path / "shim", c.tables, ctl)
    assert np.array_equal(bits(S_cpu), bits(S_shim))
    assert np.array_equal(bits(S_cpu), bits(harness_state(c.tables, c.U, ctl, scheme)))


def test_main_slip_and_noslip_walls(exes, tmp_path):
    """Slip walls on the y sides, no-slip on the z sides: the compat layer's
    wall ghosts (the reference declares bc_reflective / bc_wall without a
    body) against libfvgpu's, through the shim."""
    t = uniform_mesh(3, side_bc=(3, 2, 3, 2, 4, 4)).flatten()
    ctl = decks.DeckControls(nstep=3, dt=2e-3)
    (tmp_path / "cpu").mkdir()
    (tmp_path / "shim").mkdir()
    S_cpu, f_cpu = run_main(exes["cpu"], tmp_path / "cpu", t, ctl)
    S_shim, f_shim = run_main(exes["shim"], tmp_path / "shim", t, ctl)
    assert np.array_equal(bits(S_cpu), bits(S_shim))
    assert f_cpu == f_shim


def test_deck_rejects_what_the_reference_cannot_read(tmp_path):
    c = cases.sod(level=2)
    with pytest.raises(ValueError, match="1 to 4"):
        decks.write_deck(str(tmp_path), "toolong", c.tables, decks.DeckControls())
    with pytest.raises(ValueError, match="periodic"):
        decks.write_deck(str(tmp_path), "c1", uniform_mesh(2, periodic=(1, 0, 0)).flatten(), decks.DeckControls())
