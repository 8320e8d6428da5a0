"""Domain decomposition with one halo exchange per RK stage
(fv_140823_gb300/halo.py; the reference's communicate_S, communicate1.c:44-229).

* the plan: owned cells keep their full neighbourhood, send and receive lists
  pair up between ranks;
* ranks emulated in one process with the oracle: after every step the owned
  cells equal the single-domain result bit for bit;
* two gloo ranks (separate processes, torch.distributed point-to-point);
* GPU: two libfvgpu contexts on one device exchanging through device buffers
  with fvgpu_halo_pack / fvgpu_halo_unpack (gpu marker).
"""
import os
import tempfile

import numpy as np
import pytest

from fv_140823_gb300 import halo
from fvtest import bits_equal, load_golden
from pyoracle import SCHEMES, Oracle

CASES = ["amr_periodic_muscl", "amr_periodic_first", "sod_l3", "inflow_l3"]


@pytest.mark.parametrize("name", CASES + ["bubble_l3"])
@pytest.mark.parametrize("nparts", [2, 3])
def test_plan_keeps_owned_neighbourhoods(name, nparts):
    t, _, _ = load_golden(name)
    part = halo.partition(t.ncells, nparts)
    meshes = halo.plan(t, part)
    assert sum(m.nowned for m in meshes) == t.ncells
    for m in meshes:
        lt = m.tables
        glob = np.concatenate([m.owned, m.ghosts])
        for c in range(m.nowned):  # owned cells: identical links (mapped to local ids)
            g = glob[c]
            for f in range(6):
                code, lc = int(t.nbr[f, g]), int(lt.nbr[f, c])
                if code >= 0:
                    assert lc >= 0 and glob[lc] == code
                elif code <= halo.HANG0:
                    assert lc <= halo.HANG0
                    assert np.array_equal(glob[lt.hang_nbr[halo.HANG0 - lc]], t.hang_nbr[halo.HANG0 - code])
                else:
                    assert lc == code
        recv = m.recv_list()
        assert np.unique(recv).size == recv.size and np.all(recv >= m.nowned)
        for q, lst in m.recv.items():
            assert meshes[q].send[m.rank].size == lst.size
            assert np.array_equal(meshes[q].owned[meshes[q].send[m.rank]], glob[lst])


def _oracle_partitioned(t, cfg, U, dt, scheme, nsteps, nparts):
    part = halo.partition(t.ncells, nparts)
    meshes = halo.plan(t, part)
    orcs = [Oracle(m.tables, cfg) for m in meshes]
    S = [np.ascontiguousarray(U[:, np.concatenate([m.owned, m.ghosts])]) for m in meshes]
    for _ in range(nsteps):
        SN = [s.copy() for s in S]
        for irk in SCHEMES[scheme]:
            bufs = {(m.rank, q): S[m.rank][:, m.send[q]].copy() for m in meshes for q in m.send}
            for m in meshes:
                for q, lst in m.recv.items():
                    S[m.rank][:, lst] = bufs[(q, m.rank)]
            for m, o in zip(meshes, orcs):
                R = o.rhs(S[m.rank], o.faceinterp(S[m.rank]) if cfg.ischeme == 2 else None,
                          o.gradcalc(S[m.rank]) if cfg.ns == 1 else None)
                o.rk(irk, dt, S[m.rank], SN[m.rank], R)
    out = np.empty_like(U)
    for m in meshes:
        out[:, m.owned] = S[m.rank][:, :m.nowned]
    return out


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("nparts", [2, 3])
def test_partitioned_steps_are_bit_identical(name, nparts):
    t, cfg, z = load_golden(name)
    U, dt = z["U"], float(z["dt"])
    ref = Oracle(t, cfg).step(U, dt, "ssprk3", 3)
    assert bits_equal(_oracle_partitioned(t, cfg, U, dt, "ssprk3", 3, nparts), ref)


def _gloo_rank(rank, world, port, name, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import torch
        t, cfg, z = load_golden(name)
        U, dt = z["U"], float(z["dt"])
        m = halo.plan(t, halo.partition(t.ncells, world))[rank]
        orc = Oracle(m.tables, cfg)
        S = np.ascontiguousarray(U[:, np.concatenate([m.owned, m.ghosts])])
        ex = halo.TorchExchange(m, S.shape[0], "cpu")
        send, recv = m.send_list(), m.recv_list()
        for _ in range(2):
            SN = S.copy()
            for irk in SCHEMES["ssprk3"]:
                ex.send.copy_(torch.from_numpy(S[:, send]))
                ex.exchange()
                S[:, recv] = ex.recv.numpy()
                R = orc.rhs(S, orc.faceinterp(S) if cfg.ischeme == 2 else None)
                orc.rk(irk, dt, S, SN, R)
        owned = torch.from_numpy(np.ascontiguousarray(S[:, :m.nowned]))
        if rank == 0:
            parts = [owned]
            for q in range(1, world):
                n_q = int(np.sum(halo.partition(t.ncells, world) == q))
                buf = torch.empty((S.shape[0], n_q), dtype=torch.float64)
                dist.recv(buf, src=q)
                parts.append(buf)
            np.save(out_path, torch.cat(parts, dim=1).numpy())
        else:
            dist.send(owned, dst=0)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["amr_periodic_muscl", "sod_l3"])
def test_two_gloo_ranks_match_single_domain(name):
    torch = pytest.importorskip("torch")
    import socket
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "owned.npy")
        torch.multiprocessing.start_processes(_gloo_rank, args=(2, port, name, out), nprocs=2, join=True,
                                              start_method="spawn")
        got = np.load(out)
    t, cfg, z = load_golden(name)
    ref = Oracle(t, cfg).step(z["U"], float(z["dt"]), "ssprk3", 2)
    assert bits_equal(got, ref)  # partition ranges are Morton-contiguous: owned blocks concatenate in order


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["amr_periodic_muscl", "inflow_l3"])
def test_gpu_self_exchange_two_contexts(name):
    import torch
    from fv_140823_gb300.solver import Solver
    t, cfg, z = load_golden(name)
    U, dt = z["U"], float(z["dt"])
    with Solver(t, cfg) as whole:
        whole.set_state(U)
        whole.step("ssprk3", dt=dt, nsteps=2)
        ref = whole.state()
    meshes = halo.plan(t, halo.partition(t.ncells, 2))
    solvers = [Solver(m.tables, cfg) for m in meshes]
    try:
        send, recv = {}, {}
        for m, s in zip(meshes, solvers):
            s.set_state(np.ascontiguousarray(U[:, np.concatenate([m.owned, m.ghosts])]))
            s.halo_set(m.send_list(), m.recv_list())
            send[m.rank] = torch.empty((s.neq, m.send_list().size), dtype=torch.float64, device="cuda")
            recv[m.rank] = torch.empty((s.neq, m.recv_list().size), dtype=torch.float64, device="cuda")
        for _ in range(2):
            for s in solvers:
                s.rk(0, dt)
            for irk in SCHEMES["ssprk3"]:
                for m, s in zip(meshes, solvers):
                    s.halo_pack(send[m.rank].data_ptr())
                    s.synchronize()
                for m in meshes:  # peer-to-peer copies of each segment
                    for q, off, cnt in m.segments("recv"):
                        qoff = dict((r, o) for r, o, _ in meshes[q].segments("send"))[m.rank]
                        recv[m.rank][:, off:off + cnt] = send[q][:, qoff:qoff + cnt]
                torch.cuda.synchronize()
                for m, s in zip(meshes, solvers):
                    s.halo_unpack(recv[m.rank].data_ptr())
                    if cfg.ischeme == 2:
                        s.faceinterp()
                    s.rhs()
                    s.rk(irk, dt)
        got = np.empty_like(U)
        for m, s in zip(meshes, solvers):
            got[:, m.owned] = s.state()[:, :m.nowned]
    finally:
        for s in solvers:
            s.close()
    assert bits_equal(got, ref)
