"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own residual / RK C code (oracle/_ref/libfvref.so, the
reference sources compiled unchanged with oracle/ref_harness.c) on small
seeded cases and stores, per case, the flattened mesh tables, the
configuration, the input state and the reference outputs:

    R      residual of the input state (RHS after faceinterp / gradcalc)
    SF     MUSCL face values (ischeme 2)
    SG     Green-Gauss gradients (ns 1)
    S_out  state after `nsteps` RK steps of `scheme` with time step `dt`

The stored tables are the exact inputs the reference saw, so the fixtures pin
any implementation that reads them (the oracle on every host, libfvgpu on the
GPU) without the reference tree.  Needs the reference tree; run from the
repository root:  python tests/golden/make_golden.py
(`python tests/golden/make_golden.py fullsize` writes fullsize.json: the
reference's 100-step Sod run as configured, see fullsize();
`python tests/golden/make_golden.py tecplot` writes tecplot.json: digests of
the reference's Tecplot files for these cases, see tecplot()).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

from fv_140823_gb300 import cases  # noqa: E402
from fv_140823_gb300.mesh import refine_by, uniform_mesh  # noqa: E402
from pyoracle import Oracle, PhysConfig, RefHarness  # noqa: E402


def _phys(cfg, dt, i_case=0):
    return PhysConfig(model=cfg.model, ns=cfg.ns, ischeme=cfg.ischeme, iprimtv=0, eos=cfg.eos,
                      i_case=i_case, gamma=cfg.gamma, pinf=cfg.pinf, visc=cfg.visc, ymin=cfg.ymin, dt=dt)


def _random_ideal(n, rng):
    U = np.zeros((5, n))
    U[0] = 1.0 + 0.3 * rng.random(n)
    U[1:4] = 0.3 * rng.standard_normal((3, n))
    U[4] = 2.5 + 0.5 * rng.random(n)
    return U


def _save(name, t, cfg, U, dt, scheme, nsteps, i_case=0):
    ref = RefHarness(t, _phys(cfg, dt, i_case))
    R = ref.residual(U)
    out = dict(
        R=R, U=U, dt=np.float64(dt), scheme=np.array(scheme), nsteps=np.int64(nsteps),
        cfg=np.array([cfg.model, cfg.ns, cfg.ischeme, cfg.eos], np.int64),
        cfg_f=np.array([cfg.gamma, cfg.pinf, cfg.visc, cfg.ymin], np.float64),
        inflow=np.array(cfg.inflow, np.float64),
        ncells=np.int64(t.ncells), nhang=np.int64(t.nhang), level=t.level, ijk=t.ijk, nbr=t.nbr,
        nbr_face=t.nbr_face, area=t.area, dcf=t.dcf, dcc=t.dcc, vol=t.vol, centroid=t.centroid,
        hang_nbr=t.hang_nbr, hang_area=t.hang_area, hang_cell=t.hang_cell, hang_face=t.hang_face,
        frames=t.frames, lo=np.array(t.lo), length=np.array(t.length),
        periodic=np.array(t.periodic), side_bc=np.array(t.side_bc))
    if cfg.ischeme == 2:
        out["SF"] = ref.sf()
    if cfg.ns == 1:
        out["SG"] = ref.sg()
    ref.set_state(U)
    ref.step(scheme, nsteps)
    out["S_out"] = ref.state()
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {t.ncells} cells, {t.nhang} 1:4 faces -> {os.path.relpath(path, REPO)}")


def main():
    rng = np.random.default_rng(20231408)
    # 1. Sod tube, uniform level 3, MUSCL, SSP-RK3
    c = cases.sod(level=3)
    _save("sod_l3", c.tables, c.cfg, c.U, 2e-3, "ssprk3", 3)
    # 2. AMR, periodic on x and z, random ideal-gas state, MUSCL and first order
    m = uniform_mesh(2, periodic=(1, 0, 1))
    refine_by(m, lambda l, cen: ((cen[0] - 0.6) ** 2 + (cen[1] - 0.5) ** 2 + (cen[2] - 0.45) ** 2) < 0.07, 4)
    t = m.flatten()
    U = _random_ideal(t.ncells, rng)
    c1 = cases.SolverConfig(model=1, ischeme=2)
    _save("amr_periodic_muscl", t, c1, U, 1e-3, "ssprk3", 2)
    c2 = cases.SolverConfig(model=1, ischeme=1)
    _save("amr_periodic_first", t, c2, U, 1e-3, "ssprk2", 2)
    # 3. two-phase mixture (model 3) on a small AMR bubble
    cb = cases.bubble(base_level=3, extra_levels=1)
    _save("bubble_l3", cb.tables, cb.cfg, cb.U, 1e-7, "ssprk3", 2)
    # 4. viscous Taylor-Green with the energy work term
    ct = cases.tgv(base_level=3, extra_levels=1)
    _save("tgv_l3", ct.tables, ct.cfg, ct.U, 1e-3, "ssprk3", 2)
    # 5. inflow boundary (bc 1) on the -x side, the reference's i_case 200 state
    m5 = uniform_mesh(3, side_bc=(2, 2, 2, 1, 2, 2))
    t5 = m5.flatten()
    g, rho, u, p = 1.4, 1.4, 3.0, 1.0
    e = rho * ((p + g * 0.0) / (rho * (g - 1.0)) + 0.5 * (u * u + 0.0 * 0.0 + 0.0 * 0.0))
    c5 = cases.SolverConfig(model=1, ischeme=2, inflow=(rho, rho * u, 0.0, 0.0, e))
    _save("inflow_l3", t5, c5, _random_ideal(t5.ncells, rng), 1e-3, "ssprk3", 2, i_case=200)


def state_digest(S: np.ndarray) -> str:
    """SHA-256 of the state's little-endian FP64 bytes, [neq][n] order."""
    return hashlib.sha256(np.ascontiguousarray(S, dtype="<f8").tobytes()).hexdigest()


def fullsize():
    """The 3-D Sod tube as configured (32^3 leaves, MUSCL/minmod + HLLC,
    SSP-RK3, 100 steps at CFL 0.5, transmissive sides) run by the reference's
    own RK / residual code.  The reference has no CFL rule (inputset.c:90
    reads a fixed dt): each step's dt comes from the oracle's CFL restatement
    on the reference's own state.  Stored: the SHA-256 of the final state, its
    per-field sums and the first and last dt (tests/golden/fullsize.json)."""
    c = cases.sod(level=5)
    orc = Oracle(c.tables, c.cfg)
    ref = RefHarness(c.tables, _phys(c.cfg, 1.0))
    S = c.U
    dts = []
    try:
        for _ in range(100):
            dt = orc.cfl_dt(S, 0.5)
            dts.append(dt)
            ref.set_dt(dt)
            ref.set_state(S)
            ref.step("ssprk3", 1)
            S = ref.state()
    finally:
        ref.close()
    out = {"c1_sod32_ssprk3_cfl05_100": {
        "workload": "Sod tube, 32^3 uniform leaves, MUSCL/minmod + HLLC, SSP-RK3, CFL 0.5, 100 steps",
        "ncells": int(c.tables.ncells), "steps": 100, "sha256": state_digest(S),
        "field_sums": [float(x) for x in S.sum(axis=1)], "dt_first": dts[0], "dt_last": dts[-1]}}
    path = os.path.join(HERE, "fullsize.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print(f"fullsize: {os.path.relpath(path, REPO)}")


def tecplot_cases():
    """(fixture, steps, root_level, i_case) of the Tecplot fixtures: every
    golden case at its first export (no gradcalc before it), the inviscid
    ones also after their RK steps, and one case as a single tree."""
    out = []
    for path in sorted(os.listdir(HERE)):
        if not path.endswith(".npz"):
            continue
        name = path[:-4]
        z = np.load(os.path.join(HERE, path))
        ic = 200 if name.startswith("inflow") else 0
        rl = int(z["level"].min())
        out.append((name, 0, rl, ic))
        if int(z["cfg"][1]) == 0:
            out.append((name, int(z["nsteps"]), rl, ic))
    out.append(("sod_l3", 0, 0, 0))
    return out


def tecplot():
    """The reference's Tecplot writer (exportfield_linked_V3.c, after gradcalc
    as loop.c:50-55 calls it) on the golden cases: SHA-256 and size of each
    file, its ZONE line and first point line (tests/golden/tecplot.json)."""
    import tempfile

    sys.path.insert(0, os.path.dirname(HERE))
    from fvtest import load_golden  # noqa: E402

    out = {}
    for name, steps, rl, ic in tecplot_cases():
        t, cfg, z = load_golden(name)
        ref = RefHarness(t, _phys(cfg, float(z["dt"]), ic))
        try:
            ref.set_state(z["U"])
            if steps:
                ref.step(str(z["scheme"]), steps)
            with tempfile.TemporaryDirectory() as d:
                with open(ref.export(rl, 12, d), "rb") as fh:
                    data = fh.read()
        finally:
            ref.close()
        lines = data.split(b"\n")
        out[f"{name}/steps{steps}/root{rl}"] = {
            "fixture": name, "steps": steps, "root_level": rl, "tstep": 12, "i_case": ic,
            "sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data),
            "zone": lines[1].decode(), "first_point": lines[2].decode()}
    path = os.path.join(HERE, "tecplot.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print(f"tecplot: {len(out)} files -> {os.path.relpath(path, REPO)}")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "fullsize":
        fullsize()
    elif len(sys.argv) > 1 and sys.argv[1] == "tecplot":
        tecplot()
    else:
        main()
