"""Time loop with mesh adaptation: the reference's loop.c:26-60, which
advances the solution (the missing advancetimeexplicit) and calls
meshadaptation() every few steps (meshadaptation.c:23-58).

The host keeps the octree; after every adaptation it flattens the leaves
again and re-uploads the tables once.  One adaptation here is:

1. the refinement criterion of the current state (criterionsplt.c:24-86,
   ``fvgpu_criterion`` on the device after ``fvgpu_gradcalc``): a target
   level per leaf;
2. ``OctreeMesh.adapt``: each leaf moves at most one level toward its target
   (criterionsmth.c), siblings merge (refineh_1.c), 2:1 face balance;
3. ``OctreeMesh.transfer``: children inherit the parent's state (split.c:493),
   a merged parent takes the mean of its children (merge.c:93-101);
4. the new tables (``OctreeMesh.flatten`` and ``fvgpu_upload_mesh``, or the
   leaf list flattened on the device by ``fvgpu_upload_leaves``) and
   ``fvgpu_upload_state`` of the transferred state.

:func:`run_adaptive` is the loop with the stepping, criterion and reload
supplied by the caller; :func:`run_adaptive_gpu` binds it to a
:class:`~fv_140823_gb300.solver.Solver`.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi
from .mesh import OctreeMesh


@dataclass
class AdaptConfig:
    every: int = 10                      # steps between adaptations
    kind: int = abi.CRIT_GRAD_RHO_H      # criterion (fvgpu.h FVGPU_CRIT_*)
    threshold: float = 5.0
    min_level: int = 1
    max_level: int = 7


@dataclass
class AdaptiveRun:
    state: np.ndarray
    steps: int
    cells: list = field(default_factory=list)  # leaf count after each adaptation


def run_adaptive(mesh: OctreeMesh, U: np.ndarray, nsteps: int, ac: AdaptConfig, step, criterion, reload,
                 flatten=True):
    """Advance `nsteps` steps, adapting the mesh after every `ac.every` steps
    (not after the last one).

    step(k) advances the current state k steps; criterion() returns
    (state, target levels) of the current mesh; reload(tables, state) puts
    the adapted mesh and the transferred state in place (with flatten=False
    reload receives the mesh itself instead of its flattened tables)."""
    done = 0
    cells = []
    final = None
    while done < nsteps:
        k = min(ac.every, nsteps - done)
        final = step(k)
        done += k
        if done >= nsteps:
            break
        S, split = criterion()
        mesh.adapt(split, ac.min_level, ac.max_level)
        S_new = mesh.transfer(S)
        reload(mesh.flatten() if flatten else mesh, S_new)
        cells.append(mesh.ncells)
    return AdaptiveRun(state=final() if callable(final) else final, steps=done, cells=cells)


def run_adaptive_gpu(solver, mesh: OctreeMesh, U: np.ndarray, nsteps: int, ac: AdaptConfig,
                     scheme: str = "ssprk3", cfl: float = 0.5) -> AdaptiveRun:
    """The loop on a :class:`Solver` whose tables are ``mesh.flatten()``:
    CFL steps of `scheme`, the criterion on the device (the FP64 Green-Gauss
    gradients of the current state), adaptation on the host, and the adapted
    leaf list flattened on the device (``fvgpu_upload_leaves``, the same
    tables as the host flattener's)."""
    solver.set_state(U)

    def step(k):
        solver.step(scheme, cfl=cfl, nsteps=k)
        return solver.state

    def criterion():
        S = solver.state()
        solver.gradcalc()
        return S, solver.criterion(ac.kind, ac.threshold, ac.max_level)

    def reload(m, S):
        level, ijk = m.leaf_cells()
        solver.upload_leaves(level, ijk, m.lo, m.length, m.periodic, m.side_bc)
        solver.set_state(S)

    return run_adaptive(mesh, U, nsteps, ac, step, criterion, reload, flatten=False)
