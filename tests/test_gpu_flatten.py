"""Device-side flattening (fvgpu_upload_leaves) against the host flattener.

The tables built on the GPU from the leaf list must equal the host
builder's (csrc/host/fvmesh.cpp) bit for bit: the mesh signature covers the
neighbour codes and faces, areas, volumes, 1:4 records and levels; residuals
and steps cover the MUSCL distances.  Unsorted and unbalanced leaf lists are
rejected.
"""
import numpy as np
import pytest

from fv_140823_gb300 import abi, cases
from fv_140823_gb300.abi import SolverConfig
from fv_140823_gb300.mesh import uniform_mesh
from fvtest import bits_equal

pytestmark = pytest.mark.gpu


def _cases():
    t5 = uniform_mesh(4, side_bc=(2, 2, 2, 1, 2, 2)).flatten()
    rho = np.ones(t5.ncells)
    inflow = cases.Case("inflow", t5, cases.conservative_ideal(rho, 0.5 * rho, 0 * rho, 0 * rho, rho),
                        SolverConfig(model=1, ischeme=2, inflow=(1.4, 4.2, 0.0, 0.0, 8.8)), cfl=0.5, nsteps=1)
    return {"periodic": cases.periodic(level=4), "sod": cases.sod(level=4),
            "bump": cases.bump(base_level=4, extra_levels=2), "tgv": cases.tgv(base_level=3, extra_levels=2),
            "bubble": cases.bubble(base_level=3, extra_levels=2), "inflow": inflow}


CASES = _cases()


@pytest.mark.parametrize("name", list(CASES))
def test_device_tables_equal_host_tables(name):
    from fv_140823_gb300.solver import Solver
    c = CASES[name]
    with Solver(c.tables, c.cfg) as host, Solver.from_leaves(c.tables, c.cfg) as dev:
        assert host.mesh_signature() == dev.mesh_signature()
        host.set_state(c.U)
        dev.set_state(c.U)
        assert bits_equal(host.residual(), dev.residual())
        dt = 2e-7 if name == "bubble" else host.compute_dt(c.cfl)
        host.set_state(c.U)
        dev.set_state(c.U)
        host.step(c.scheme, dt=dt, nsteps=2)
        dev.step(c.scheme, dt=dt, nsteps=2)
        assert bits_equal(host.state(), dev.state())


def test_device_flattening_rejects_bad_leaf_lists():
    from fv_140823_gb300.solver import FvGpuError, Solver
    t = cases.bump(base_level=3, extra_levels=1).tables
    cfg = SolverConfig(model=1, ischeme=2)
    with Solver(None, cfg) as s:
        lvl, ijk = t.level.copy(), t.ijk.copy()
        lvl[[3, 4]], ijk[:, [3, 4]] = lvl[[4, 3]], ijk[:, [4, 3]]    # two leaves swapped: not Morton order
        with pytest.raises(FvGpuError) as ei:
            s.upload_leaves(lvl, ijk, t.lo, t.length, t.periodic, t.side_bc)
        assert ei.value.code == abi.ERR_MESH
        # unbalanced: a level-5 region of a level-3 mesh (a face sees two levels)
        m = uniform_mesh(3)
        tt = m.flatten()
        keep = np.ones(tt.ncells, bool)
        keep[0] = False
        kids = []
        for ch in range(8):                     # cell 0 replaced by 64 level-5 cells
            for g in range(8):
                kids.append((5, 4 * 0 + 2 * (ch & 1) + (g & 1), 2 * ((ch >> 1) & 1) + ((g >> 1) & 1),
                             2 * ((ch >> 2) & 1) + ((g >> 2) & 1)))
        lv = np.concatenate([[k[0] for k in kids], tt.level[keep]]).astype(np.int32)
        pos = np.concatenate([np.array([[k[1], k[2], k[3]] for k in kids]).T, tt.ijk[:, keep]], axis=1)
        key = [sum(((int(pos[a, i]) << (18 - int(lv[i]))) >> b & 1) << (3 * b + a) for b in range(18) for a in range(3))
               for i in range(lv.size)]
        order = np.argsort(key)
        with pytest.raises(FvGpuError) as ei:
            s.upload_leaves(lv[order], pos[:, order], tt.lo, tt.length, tt.periodic, tt.side_bc)
        assert ei.value.code == abi.ERR_MESH
