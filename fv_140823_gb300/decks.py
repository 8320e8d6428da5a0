"""Input decks of the reference's host program for a conforming hex mesh.

The reference's ``main()`` (main.c:16-187) reads a case as files named
``<case>.ct`` (run controls, inputset.c:33-117), ``<case>.nd`` (nodes) and
``<case>.el`` (elements; createtopo.c:37-70) and ``<case>.ba``-``.bd``
(boundary faces of codes 1-4, boundary.c:42-55).  :func:`write_deck` writes
them for the leaves of a flattened mesh whose leaves all have one level:
every leaf becomes one tree (an element of the input mesh) in the leaves'
order, with its 8 nodes in the reference's hexahedron numbering (node n at
offset (n & 1, n >> 1 & 1, n >> 2 & 1) along x, y, z, the numbering its
face tables in operatetp.c imply).  Node coordinates are printed with 17
significant digits, so the program reads back the same doubles.

The case name must be at most 4 characters: filenames.c:15-25 allocates
sizeof(int) + 4 bytes for each file name.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

# reference face index -> (axis, side) of the box face it lies on
_FACE_AXIS = (1, 0, 1, 0, 2, 2)
_FACE_SIDE = (0, 1, 1, 0, 0, 1)


@dataclass
class DeckControls:
    """The .ct fields (inputset.c:33-117), models 1 and 2."""

    i_case: int = 91          # init_domain.c:223-240: the Sod states split at x = 0.5
    model: int = 1
    ns: int = 0
    ischeme: int = 2
    iprimtv: int = 0
    method: int = 3           # RK order of advancetimeexplicit: 3 = SSP-RK3
    halfdt: int = 0
    limiter: int = 0
    level: int = 1
    pinf: float = 0.0
    gamma: float = 1.4
    visc: float = 0.0
    nstep: int = 10
    dt: float = 1e-3
    exstep: int = 1000000
    ststep: int = 1000000
    geo_adapth: int = 0
    adapth: int = 0
    adapthstep: int = 1000000
    start: int = 0
    translator: int = 0
    bcoverwrt: tuple = field(default_factory=lambda: (0, 0, 0, 0, 0, 0))
    mscale: float = 1.0
    splitmode: int = 8
    nquad: tuple = (0.0, 0.0, 0.0)


def _ct_text(c: DeckControls) -> str:
    if c.model not in (1, 2):
        raise ValueError("write_deck supports models 1 and 2")
    rows = [("verbose", 0), ("i_case", c.i_case), ("model", c.model), ("ns", c.ns), ("ischeme", c.ischeme),
            ("iprimtv", c.iprimtv), ("RK", c.method), ("halfdt", c.halfdt), ("limiter", c.limiter),
            ("level", c.level), ("materpinf", repr(float(c.pinf))), ("matergama", repr(float(c.gamma))),
            ("matervisc", repr(float(c.visc))), ("nstep", c.nstep), ("dt", "%.17e" % c.dt),
            ("exstep", c.exstep), ("ststep", c.ststep), ("geo_adapth", c.geo_adapth), ("adapth", c.adapth),
            ("adapthstep", c.adapthstep), ("start", c.start), ("translator", c.translator)]
    out = "".join(f"{k}\t{v}\n" for k, v in rows)
    out += "bc" + "".join(f"\t{int(b)}" for b in c.bcoverwrt) + "\n"
    out += f"mscale\t{c.mscale!r}\nsplitmode\t{c.splitmode}\n"
    out += "".join(f"{k}\t{float(v)!r}\n" for k, v in zip(("nxquad", "nyquad", "nzquad"), c.nquad))
    return out


def write_deck(directory: str, case: str, tables, controls: DeckControls) -> list[str]:
    """Write the deck of `tables` (a flattened mesh whose leaves share one
    level; no periodic axis) into `directory`; returns the paths written."""
    if not 1 <= len(case) <= 4:
        raise ValueError("the case name must have 1 to 4 characters (filenames.c allocates 8 bytes)")
    if any(tables.periodic):
        raise ValueError("the reference's input mesh has no periodic boundary")
    lv = np.unique(tables.level)
    if lv.size != 1:
        raise ValueError("every leaf must have the same level: the trees of the input mesh are conforming")
    l = int(lv[0])
    n = int(tables.ncells)
    nl = 1 << l
    ijk = np.asarray(tables.ijk, dtype=np.int64)
    lo = np.asarray(tables.lo, dtype=np.float64)
    ln = np.asarray(tables.length, dtype=np.float64)
    # lattice nodes used by the leaves, numbered in order of first use
    offs = np.array([[(k >> a) & 1 for a in range(3)] for k in range(8)], dtype=np.int64)  # [8][3]
    corner = ijk.T[:, None, :] + offs[None, :, :]  # [n][8][3]
    key = (corner[..., 2] * (nl + 1) + corner[..., 1]) * (nl + 1) + corner[..., 0]
    flat = key.reshape(-1)
    uniq, first = np.unique(flat, return_index=True)
    order = np.argsort(first)
    node_id = np.empty(uniq.size, dtype=np.int64)
    node_id[order] = np.arange(uniq.size)
    elem = node_id[np.searchsorted(uniq, flat)].reshape(n, 8) + 1
    pts = uniq[order]
    P = np.stack([pts % (nl + 1), (pts // (nl + 1)) % (nl + 1), pts // ((nl + 1) * (nl + 1))], axis=1)
    xyz = lo[None, :] + P.astype(np.float64) * np.ldexp(ln, -l)[None, :]

    os.makedirs(directory, exist_ok=True)
    paths = []

    def put(ext, text):
        p = os.path.join(directory, case + ext)
        with open(p, "w") as fh:
            fh.write(text)
        paths.append(p)

    put(".ct", _ct_text(controls))
    put(".nd", f"{len(pts)}\n" + "".join("%d\t%.17e\t%.17e\t%.17e\n" % (i + 1, x, y, z)
                                         for i, (x, y, z) in enumerate(xyz)))
    put(".el", f"{n}\n" + "".join(f"{c + 1}\t4" + "".join(f"\t{v}" for v in elem[c]) + "\n" for c in range(n)))
    nbr = np.asarray(tables.nbr)
    for bc, ext in ((1, ".ba"), (2, ".bb"), (3, ".bc"), (4, ".bd")):
        rows = [(c + 1, f + 1) for c in range(n) for f in range(6) if nbr[f, c] == -1 - bc]
        put(ext, f"{len(rows)}\n" + "".join(f"{c}\t{f}\n" for c, f in rows))
    return paths
