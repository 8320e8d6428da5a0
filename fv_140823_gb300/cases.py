"""Synthetic workloads: meshes and initial states of the five benchmark cases.

The reference ships no input decks, so each case is generated from its
description with seeded numpy generators.

* ``sod``      -- 3-D Sod tube on [0,1]^3, uniform level 5 (32^3), ideal gas
                  1.4, x<0.5 (rho,p)=(1,1) else (0.125,0.1), transmissive
                  (the reference's i_case 91 initial state, init_domain.c:224-240).
* ``bubble``   -- two-phase gas bubble in liquid, mixture EOS (model 3), base
                  level 4 plus up to 3 levels refined on |grad rho| h.
* ``periodic`` -- 128^3 periodic ideal gas with smooth seeded Fourier
                  velocities (8 modes per axis), sinusoidal density and noisy
                  pressure (PCG64 seed 1234).
* ``bump``     -- level-5 base with 2 more levels inside a seeded sphere of
                  radius 0.2 carrying a smooth density bump 1 -> 2.
* ``tgv``      -- Taylor-Green vortex on [0,2pi]^3, Re 1600, Mach 0.1,
                  viscous, levels refined on vorticity.

Every builder accepts a ``level`` override so the same case runs at the
small sizes a CPU oracle finishes in seconds.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .abi import SolverConfig
from .mesh import BC_TRANSMISSIVE, MeshTables, OctreeMesh, refine_by, uniform_mesh

GAMMA = 1.4


@dataclass
class Case:
    name: str
    tables: MeshTables
    U: np.ndarray          # (neq, ncells) conservative state
    cfg: SolverConfig
    cfl: float
    nsteps: int
    scheme: str = "ssprk3"
    mesh: OctreeMesh | None = None  # the host octree the tables were flattened from


def conservative_ideal(rho, u, v, w, p, gamma=GAMMA, pinf=0.0):
    """Init_S.c:3-17: E = rho (e + |u|^2 / 2), e = (p + gamma pinf) / (rho (gamma - 1))."""
    rho = np.asarray(rho, dtype=np.float64)
    e_int = (p + gamma * pinf) / (rho * (gamma - 1.0))
    U = np.empty((5,) + rho.shape)
    U[0] = rho
    U[1] = rho * u
    U[2] = rho * v
    U[3] = rho * w
    U[4] = rho * (e_int + 0.5 * (u * u + v * v + w * w))
    return U


def sod(level: int = 5) -> Case:
    m = uniform_mesh(level, side_bc=(BC_TRANSMISSIVE,) * 6)
    t = m.flatten()
    x = t.centroid[0]
    left = x < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    z = np.zeros_like(rho)
    U = conservative_ideal(rho, z, z, z, p)
    return Case("sod", t, U, SolverConfig(model=1, ischeme=2, gamma=GAMMA), cfl=0.5, nsteps=100)


def periodic(level: int = 7, seed: int = 1234) -> Case:
    m = uniform_mesh(level, periodic=(1, 1, 1))
    t = m.flatten()
    rng = np.random.Generator(np.random.PCG64(seed))
    x, y, z = t.centroid
    twopi = 2.0 * math.pi
    rho = 1.0 + 0.1 * np.sin(twopi * x) * np.sin(twopi * y) * np.sin(twopi * z)
    vel = []
    coords = (x, y, z)
    for _comp in range(3):
        field = np.zeros_like(x)
        for axis in range(3):
            k = np.arange(1, 9)
            a = rng.standard_normal(8) / k
            phi = rng.uniform(0.0, twopi, 8)
            for kk, aa, ph in zip(k, a, phi):
                field += aa * np.sin(twopi * kk * coords[axis] + ph)
        field *= 0.3 / np.max(np.abs(field))
        vel.append(field)
    p = 1.0 + 0.05 * rng.uniform(-1.0, 1.0, x.shape)
    U = conservative_ideal(rho, vel[0], vel[1], vel[2], p)
    return Case("periodic", t, U, SolverConfig(model=1, ischeme=2, gamma=GAMMA), cfl=0.5, nsteps=50)


# mixture constants of barotropic_multiphase_eos (barotropic_eos.c:41-47)
R_G, T_REF, R_SAT, P_SAT, C_LIQ = 286.0, 293.15, 998.1618, 2340.0, 1482.5


def _bubble_state(cen, h, p_bg=1e5, p_slab=1e6, radius=0.15, slab=0.1, width=2.0):
    x, y, zc = cen
    r = np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2 + (zc - 0.5) ** 2)
    alpha = 0.5 * (1.0 - np.tanh((r - radius) / (width * h)))       # gas volume fraction
    p = np.where(x < slab, p_slab, p_bg)
    rho_l = R_SAT + (p - P_SAT) / (C_LIQ * C_LIQ)
    rho_g = p_bg / (R_G * T_REF)
    rho = alpha * rho_g + (1.0 - alpha) * rho_l
    Y = alpha * rho_g / rho
    U = np.zeros((5,) + x.shape)
    U[0] = rho
    U[4] = rho * Y
    return U


def bubble(base_level: int = 4, extra_levels: int = 3, threshold: float = 0.05) -> Case:
    m = uniform_mesh(base_level)
    maxl = base_level + extra_levels

    def crit(level, cen):
        h = np.ldexp(1.0, -level.astype(np.int64))
        rho = _bubble_state(cen, h)[0]
        # density jump across the cell measured against its neighbours' scale:
        # |grad rho| h ~ |rho(x + h) - rho(x - h)| / 2 summed over axes
        g = np.zeros_like(rho)
        for a in range(3):
            cp = cen.copy()
            cm = cen.copy()
            cp[a] += h
            cm[a] -= h
            g += np.abs(_bubble_state(cp, h)[0] - _bubble_state(cm, h)[0]) * 0.5
        return g / np.maximum(rho, 1e-300) > threshold

    refine_by(m, crit, maxl)
    t = m.flatten()
    h = np.ldexp(1.0, -t.level.astype(np.int64))
    U = _bubble_state(t.centroid, h)
    cfg = SolverConfig(model=3, ischeme=2, ymin=1e-6)
    return Case("bubble", t, U, cfg, cfl=0.5, nsteps=200, mesh=m)


def bump(base_level: int = 5, extra_levels: int = 2, seed: int = 7, radius: float = 0.2) -> Case:
    rng = np.random.Generator(np.random.PCG64(seed))
    centre = rng.uniform(0.3, 0.7, 3)
    m = uniform_mesh(base_level)

    def inside(level, cen):
        d = np.sqrt(((cen - centre[:, None]) ** 2).sum(axis=0))
        return d < radius

    refine_by(m, inside, base_level + extra_levels)
    t = m.flatten()
    d = np.sqrt(((t.centroid - centre[:, None]) ** 2).sum(axis=0))
    rho = 1.0 + 0.5 * (1.0 + np.cos(np.pi * np.clip(d / radius, 0.0, 1.0)))  # 2 at centre -> 1 at r
    z = np.zeros_like(rho)
    U = conservative_ideal(rho, z + 0.1, z, z, np.ones_like(rho))
    return Case("bump", t, U, SolverConfig(model=1, ischeme=2, gamma=GAMMA), cfl=0.5, nsteps=1,
                scheme="euler")


def tgv(base_level: int = 5, extra_levels: int = 2, threshold: float = 0.5, Re: float = 1600.0,
        mach: float = 0.1) -> Case:
    L = 2.0 * math.pi
    m = OctreeMesh((0.0, 0.0, 0.0), (L, L, L), base_level, periodic=(1, 1, 1))
    U0, rho0 = 1.0, 1.0
    p0 = rho0 * U0 * U0 / (GAMMA * mach * mach)

    def vort(cen):
        x, y, z = cen
        # |omega| of the TGV velocity field
        wx = -U0 * np.cos(x) * np.sin(y) * np.sin(z)
        wy = -U0 * np.sin(x) * np.cos(y) * np.sin(z)
        wz = 2.0 * U0 * np.sin(x) * np.sin(y) * np.cos(z)
        return np.sqrt(wx * wx + wy * wy + wz * wz)

    refine_by(m, lambda level, cen: vort(cen) > threshold * 2.0 * U0 + 0.5 * (level - base_level),
              base_level + extra_levels)
    t = m.flatten()
    x, y, z = t.centroid
    u = U0 * np.sin(x) * np.cos(y) * np.cos(z)
    v = -U0 * np.cos(x) * np.sin(y) * np.cos(z)
    w = np.zeros_like(x)
    p = p0 + rho0 * U0 * U0 / 16.0 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0)
    rho = p / p0 * rho0
    U = conservative_ideal(rho, u, v, w, p)
    mu = rho0 * U0 * 1.0 / Re
    cfg = SolverConfig(model=1, ischeme=2, ns=1, eos=1, visc=mu, gamma=GAMMA)
    return Case("tgv", t, U, cfg, cfl=0.5, nsteps=10)


BUILDERS = {"sod": sod, "periodic": periodic, "bubble": bubble, "bump": bump, "tgv": tgv}
