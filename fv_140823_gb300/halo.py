"""Domain decomposition of a flattened mesh: rank meshes with a ghost layer
and the exchange plan of one halo per RK stage.

The reference partitions its trees with ParMETIS (repartition_parmetis.c:226)
and exchanges interface states between ranks once per stage
(communicate_S, communicate1.c:44-229).  Here the leaves are already in Morton
order, so a rank owns a contiguous Morton range; its mesh holds its own cells
followed by every cell within ``depth`` face hops (2 for MUSCL: the face
values of a neighbour read that neighbour's neighbours), with the links of the
outermost ghosts that leave the rank mesh turned into transmissive faces.
Owned cells see exactly the neighbours, areas and distances of the global
mesh, so their residuals and stage updates are bit-identical to a
single-domain run once the ghosts hold the owners' current state.

Exchange per stage (before face values are built): the owner packs the cells
other ranks hold as ghosts (``fvgpu_halo_pack``), the buffers travel
(:class:`TorchExchange`: point-to-point sends over ``torch.distributed``, NCCL
on GPUs, gloo on CPUs; or a device copy between contexts on one GPU), and the
receiver unpacks them into its ghost cells (``fvgpu_halo_unpack``).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .mesh import BC_TRANSMISSIVE, HANG0, MeshTables


def partition(ncells: int, nparts: int) -> np.ndarray:
    """Rank of every cell: contiguous Morton ranges of near-equal size."""
    return (np.arange(ncells, dtype=np.int64) * nparts // max(ncells, 1)).astype(np.int32)


def _neighbours(t: MeshTables, c: int) -> list[int]:
    out = []
    for f in range(6):
        code = int(t.nbr[f, c])
        if code >= 0:
            out.append(code)
        elif code <= HANG0:
            out.extend(int(k) for k in t.hang_nbr[HANG0 - code])
    return out


@dataclass
class RankMesh:
    rank: int
    tables: MeshTables          # owned cells first, then ghosts
    owned: np.ndarray           # global ids of the owned cells (local 0 .. nowned-1)
    ghosts: np.ndarray          # global ids of the ghosts (local nowned ..)
    recv: dict = field(default_factory=dict)  # source rank -> local ghost ids, in exchange order
    send: dict = field(default_factory=dict)  # destination rank -> local owned ids, in exchange order

    @property
    def nowned(self) -> int:
        return int(self.owned.size)

    def send_list(self) -> np.ndarray:
        return np.concatenate([self.send[r] for r in sorted(self.send)] or [np.zeros(0, np.int32)])

    def recv_list(self) -> np.ndarray:
        return np.concatenate([self.recv[r] for r in sorted(self.recv)] or [np.zeros(0, np.int32)])

    def segments(self, which: str) -> list[tuple[int, int, int]]:
        """(peer, offset, count) of each peer's part of the send / recv list."""
        d = self.send if which == "send" else self.recv
        out, off = [], 0
        for r in sorted(d):
            out.append((r, off, int(d[r].size)))
            off += int(d[r].size)
        return out


def _ghost_set(t: MeshTables, part: np.ndarray, rank: int, depth: int) -> np.ndarray:
    owned = np.flatnonzero(part == rank)
    inside = np.zeros(t.ncells, bool)
    inside[owned] = True
    frontier = owned
    for _ in range(depth):
        nxt = set()
        for c in frontier:
            for k in _neighbours(t, int(c)):
                if not inside[k]:
                    inside[k] = True
                    nxt.add(k)
        frontier = np.fromiter(sorted(nxt), dtype=np.int64)
    ghosts = np.flatnonzero(inside & (part != rank))
    return owned, ghosts


def rank_mesh(t: MeshTables, part: np.ndarray, rank: int, depth: int = 2) -> RankMesh:
    owned, ghosts = _ghost_set(t, part, rank, depth)
    glob = np.concatenate([owned, ghosts]).astype(np.int64)
    n = glob.size
    local = np.full(t.ncells, -1, np.int64)
    local[glob] = np.arange(n)
    transmissive = -1 - BC_TRANSMISSIVE
    nbr = np.empty((6, n), np.int32)
    nbr_face = np.empty((6, n), np.int32)
    hang_nbr, hang_area, hang_cell, hang_face = [], [], [], []
    for f in range(6):
        for i, g in enumerate(glob):
            code = int(t.nbr[f, g])
            nf = int(t.nbr_face[f, g])
            if code >= 0:
                k = local[code]
                if k >= 0:
                    nbr[f, i], nbr_face[f, i] = k, nf
                else:
                    nbr[f, i], nbr_face[f, i] = transmissive, -1
            elif code <= HANG0:
                r = HANG0 - code
                ks = local[t.hang_nbr[r]]
                if np.all(ks >= 0):
                    nbr[f, i], nbr_face[f, i] = HANG0 - len(hang_nbr), nf
                    hang_nbr.append(ks.astype(np.int32))
                    hang_area.append(t.hang_area[r])
                    hang_cell.append(i)
                    hang_face.append(f)
                else:
                    nbr[f, i], nbr_face[f, i] = transmissive, -1
            else:
                nbr[f, i], nbr_face[f, i] = code, nf
    # a link whose far side was cut (only between outermost ghosts) becomes a
    # transmissive face on both sides; repeat until every link is reciprocal
    alive = [True] * len(hang_nbr)
    changed = True
    while changed:
        changed = False
        for f in range(6):
            for i in range(n):
                code = int(nbr[f, i])
                if code >= 0:
                    back = int(nbr[int(nbr_face[f, i]), code])
                    ok = back == i or (back <= HANG0 and alive[HANG0 - back] and i in hang_nbr[HANG0 - back])
                elif code <= HANG0:
                    r = HANG0 - code
                    nf = int(nbr_face[f, i])
                    ok = all(int(nbr[nf, k]) == i for k in hang_nbr[r])
                    if not ok:
                        alive[r] = False
                else:
                    continue
                if not ok:
                    nbr[f, i], nbr_face[f, i] = transmissive, -1
                    changed = True
    hn, ha, hc, hf = [], [], [], []
    for r in range(len(hang_nbr)):
        if alive[r]:
            nbr[hang_face[r], hang_cell[r]] = HANG0 - len(hn)
            hn.append(hang_nbr[r])
            ha.append(hang_area[r])
            hc.append(hang_cell[r])
            hf.append(hang_face[r])
    nh = len(hn)
    lt = MeshTables(
        ncells=n, nhang=nh, level=t.level[glob].copy(), ijk=t.ijk[:, glob].copy(), nbr=nbr, nbr_face=nbr_face,
        area=t.area[:, glob].copy(), dcf=t.dcf[:, glob].copy(), dcc=t.dcc[:, glob].copy(), vol=t.vol[glob].copy(),
        centroid=t.centroid[:, glob].copy(),
        hang_nbr=np.array(hn, np.int32).reshape(nh, 4), hang_area=np.array(ha, np.float64).reshape(nh, 4),
        hang_cell=np.array(hc, np.int32), hang_face=np.array(hf, np.int32), frames=t.frames.copy(),
        lo=t.lo, length=t.length, periodic=t.periodic, side_bc=t.side_bc)
    return RankMesh(rank=rank, tables=lt, owned=owned.astype(np.int64), ghosts=ghosts.astype(np.int64))


def plan(t: MeshTables, part: np.ndarray, depth: int = 2) -> list[RankMesh]:
    """Rank meshes of every rank with their send / receive lists."""
    nparts = int(part.max()) + 1
    meshes = [rank_mesh(t, part, r, depth) for r in range(nparts)]
    for m in meshes:
        for q in range(nparts):
            if q == m.rank:
                continue
            sel = np.flatnonzero(part[m.ghosts] == q)
            if sel.size == 0:
                continue
            gids = m.ghosts[sel]                       # ascending global ids
            m.recv[q] = (m.nowned + sel).astype(np.int32)
            owner = meshes[q]
            pos = np.searchsorted(owner.owned, gids)   # owner's local id = rank in its owned list
            owner.send[m.rank] = pos.astype(np.int32)
    return meshes


class TorchExchange:
    """One halo exchange over torch.distributed point-to-point messages.

    ``send`` / ``recv`` are tensors [neq, nsend] / [neq, nrecv] on the
    communication device; segments come from :meth:`RankMesh.segments`."""

    def __init__(self, mesh: RankMesh, neq: int, device):
        import torch
        self.mesh = mesh
        self.send = torch.empty((neq, int(mesh.send_list().size)), dtype=torch.float64, device=device)
        self.recv = torch.empty((neq, int(mesh.recv_list().size)), dtype=torch.float64, device=device)
        self._send_segs = mesh.segments("send")
        self._recv_segs = mesh.segments("recv")

    def exchange(self):
        import torch
        import torch.distributed as dist
        reqs, rbufs = [], []
        for peer, off, cnt in self._recv_segs:
            buf = torch.empty((self.recv.shape[0], cnt), dtype=self.recv.dtype, device=self.recv.device)
            rbufs.append((off, cnt, buf))
            reqs.append(dist.irecv(buf, src=peer))
        for peer, off, cnt in self._send_segs:
            reqs.append(dist.isend(self.send[:, off:off + cnt].contiguous(), dst=peer))
        for r in reqs:
            r.wait()
        for off, cnt, buf in rbufs:
            self.recv[:, off:off + cnt] = buf
        del torch
