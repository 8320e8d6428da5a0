"""fvgpu_conservation_noalloc: the conservation sums for host codes that may
not allocate device memory (a solver that reserves all of its device memory
at start-up and forbids allocation in its time loop, or a process whose
device-memory cap is already committed).  The entry point takes device arrays
the caller owns and keeps its scratch in a fixed array inside the library.

Checked against the context entry point fvgpu_conservation on two calls in a
row with different states, so a stale scratch array would show.  Both use the
same partition and reduction order, so the sums must agree bit for bit (the
tolerance the conservation tests use elsewhere is 1e-13 relative; bitwise is
stricter).  This file is collected last so that a failure here leaves every
other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from fv_140823_gb300 import abi, cases
from fv_140823_gb300._native import load_gpu_lib
from fvtest import bits_equal, random_ideal_state

pytestmark = pytest.mark.gpu


def context_sums(tables, cfg, U):
    from fv_140823_gb300.solver import Solver
    with Solver(tables, cfg) as s:
        s.set_state(U)
        return s.conservation()


def test_noalloc_conservation_matches_context_entry_point():
    import torch
    lib = load_gpu_lib()
    c = cases.bump(base_level=4, extra_levels=2)
    t = c.tables
    n = t.ncells
    states = [c.U, random_ideal_state(n, np.random.default_rng(99))]
    dev = torch.device("cuda", 0)
    vol = torch.from_numpy(np.ascontiguousarray(t.vol)).to(dev)
    sums = torch.empty(8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for U in states:
        want = context_sums(t, c.cfg, U)
        S = torch.from_numpy(np.ascontiguousarray(U)).to(dev)
        sums.fill_(float("nan"))
        rc = lib.fvgpu_conservation_noalloc(C.c_void_p(S.data_ptr()), C.c_void_p(vol.data_ptr()),
                                            C.c_int64(n), 5, C.c_void_p(sums.data_ptr()),
                                            C.c_void_p(stream.cuda_stream))
        assert rc == abi.OK
        stream.synchronize()
        got = sums[:6].cpu().numpy()
        assert bits_equal(got, want), (got, want)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    lib = load_gpu_lib()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    p = C.c_void_p(buf.data_ptr())
    assert lib.fvgpu_conservation_noalloc(p, p, C.c_int64(2), 6, p, None) == abi.ERR_ARG
    assert lib.fvgpu_conservation_noalloc(p, p, C.c_int64(0), 5, p, None) == abi.ERR_ARG
    assert lib.fvgpu_conservation_noalloc(p, p, C.c_int64(1 << 31), 5, p, None) == abi.ERR_ARG
