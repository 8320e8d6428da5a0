"""Shared helpers of the test suite."""
from __future__ import annotations

import glob
import os

import numpy as np

from fv_140823_gb300.abi import SolverConfig
from fv_140823_gb300.mesh import MeshTables

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    t = MeshTables(
        ncells=int(z["ncells"]), nhang=int(z["nhang"]), level=z["level"], ijk=z["ijk"], nbr=z["nbr"],
        nbr_face=z["nbr_face"], area=z["area"], dcf=z["dcf"], dcc=z["dcc"], vol=z["vol"],
        centroid=z["centroid"], hang_nbr=z["hang_nbr"], hang_area=z["hang_area"],
        hang_cell=z["hang_cell"], hang_face=z["hang_face"], frames=z["frames"],
        lo=tuple(z["lo"]), length=tuple(z["length"]), periodic=tuple(int(p) for p in z["periodic"]),
        side_bc=tuple(int(b) for b in z["side_bc"]))
    ci, cf = z["cfg"], z["cfg_f"]
    cfg = SolverConfig(model=int(ci[0]), ns=int(ci[1]), ischeme=int(ci[2]), eos=int(ci[3]),
                       gamma=float(cf[0]), pinf=float(cf[1]), visc=float(cf[2]), ymin=float(cf[3]),
                       inflow=tuple(z["inflow"]))
    return t, cfg, z


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def max_rel(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def random_ideal_state(n, rng, amp=0.3):
    U = np.zeros((5, n))
    U[0] = 1.0 + amp * rng.random(n)
    U[1:4] = amp * rng.standard_normal((3, n))
    U[4] = 2.5 + 0.5 * rng.random(n)
    return U
