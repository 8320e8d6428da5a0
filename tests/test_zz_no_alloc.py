"""fvgpu_conservation_noalloc: the conservation sums for host codes that may
not allocate device memory (a solver that reserves all of its device memory
at start-up and forbids allocation in its time loop, or a process whose
device-memory cap is already committed).  The entry point takes device arrays
the caller owns and keeps its scratch in a fixed array inside the library.

Checked against the context entry point fvgpu_conservation on two calls in a
row with different states, so a stale scratch array would show, for five and
for four conserved variables; a fresh process checks that a first call on a
new context allocates no device memory.  Both use the
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


def test_noalloc_conservation_four_variables():
    """neq = 4 (the barotropic liquid, model 2): two calls in a row against the
    context entry point of a model-2 context on the same mesh."""
    import torch
    lib = load_gpu_lib()
    c = cases.bump(base_level=4, extra_levels=1)
    t = c.tables
    n = t.ncells
    cfg = abi.SolverConfig(model=2, ischeme=1)
    rng = np.random.default_rng(5)
    dev = torch.device("cuda", 0)
    vol = torch.from_numpy(np.ascontiguousarray(t.vol)).to(dev)
    sums = torch.empty(8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for k in range(2):
        U = np.vstack([1000.0 + rng.random(n), 0.1 * rng.standard_normal((3, n))])
        want = context_sums(t, cfg, U)
        S = torch.from_numpy(np.ascontiguousarray(U)).to(dev)
        sums.fill_(float("nan"))
        rc = lib.fvgpu_conservation_noalloc(C.c_void_p(S.data_ptr()), C.c_void_p(vol.data_ptr()),
                                            C.c_int64(n), 4, C.c_void_p(sums.data_ptr()),
                                            C.c_void_p(stream.cuda_stream))
        assert rc == abi.OK
        stream.synchronize()
        got = sums[:5].cpu().numpy()
        assert bits_equal(got, want), (k, got, want)


_FRESH_PROCESS = r"""
import ctypes as C, os, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from fv_140823_gb300._native import load_gpu_lib
lib = load_gpu_lib()          # registered before the context exists: loaded with it (eager loading)
import torch
dev = torch.device("cuda", 0)
n = 100000
S = torch.rand(5, n, dtype=torch.float64, device=dev)
vol = torch.rand(n, dtype=torch.float64, device=dev)
sums = torch.zeros(8, dtype=torch.float64, device=dev)
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info(0)[0]
for _ in range(2):
    rc = lib.fvgpu_conservation_noalloc(C.c_void_p(S.data_ptr()), C.c_void_p(vol.data_ptr()), C.c_int64(n), 5,
                                        C.c_void_p(sums.data_ptr()), None)
    assert rc == 0, rc
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info(0)[0]
ref = [float((S[v] * vol).sum()) for v in range(5)] + [float(vol.sum())]
got = sums[:6].cpu().numpy()
assert np.allclose(got, ref, rtol=1e-13, atol=0), (got, ref)
print(free0 - free1)
"""


def test_noalloc_first_call_allocates_nothing():
    """In a fresh process (so the call is the first on a new context), the
    device's free memory is the same before and after two calls.  The library
    is loaded before the context exists and CUDA loads modules eagerly, so its
    code and its static scratch array are in place before the first reading;
    any cudaMalloc by the entry point would show as a drop of at least a page."""
    import os
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    r = subprocess.run([sys.executable, "-c", _FRESH_PROCESS, repo], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert int(r.stdout.strip().splitlines()[-1]) == 0, r.stdout


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    lib = load_gpu_lib()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    p = C.c_void_p(buf.data_ptr())
    assert lib.fvgpu_conservation_noalloc(p, p, C.c_int64(2), 6, p, None) == abi.ERR_ARG
    assert lib.fvgpu_conservation_noalloc(p, p, C.c_int64(0), 5, p, None) == abi.ERR_ARG
    assert lib.fvgpu_conservation_noalloc(p, p, C.c_int64(1 << 31), 5, p, None) == abi.ERR_ARG
