"""In-tree build of the package's native libraries.

* ``_lib/libfvmesh.so`` -- host octree mesh builder / flattener (C++).
* ``_lib/libfvgpu.so``  -- the CUDA residual / RK library for sm_103a.

Both are compiled straight into the package directory (no install step), so
the loaded ``.so`` files are always the in-tree ones.  Host code is built with
``-ffp-contract=off`` so no multiply-add is fused on either host ISA, and the
device code with ``-fmad=false`` on the FP64 parity path (see the kernel
sources for where fused forms are used deliberately).
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
LIB = os.path.join(PKG, "_lib")
INCLUDE = os.path.join(REPO, "include")
CSRC = os.path.join(PKG, "csrc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_mesh() -> str:
    os.makedirs(LIB, exist_ok=True)
    out = os.path.join(LIB, "libfvmesh.so")
    _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-fopenmp",
          "-Wall", "-I", INCLUDE, os.path.join(CSRC, "host", "fvmesh.cpp"),
          os.path.join(CSRC, "host", "fvexport.cpp"), "-o", out])
    return out


def _file_flags(path: str) -> list[str]:
    """Per-file nvcc flags from a leading ``// fvbuild: <flags>`` line."""
    with open(path) as fh:
        first = fh.readline()
    tag = "// fvbuild:"
    return first[len(tag):].split() if first.startswith(tag) else []


def gpu_sources() -> list[str]:
    d = os.path.join(CSRC, "gpu")
    if not os.path.isdir(d):
        return []
    return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(".cu"))


def build_gpu(extra_flags: list[str] | None = None) -> str | None:
    srcs = gpu_sources()
    if not srcs:
        return None
    os.makedirs(LIB, exist_ok=True)
    obj_dir = os.path.join(LIB, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    flags = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", os.path.join(CSRC, "gpu"),
             *(extra_flags or [])]
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(obj_dir, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        jobs.append(["nvcc", *flags, *_file_flags(s), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    out = os.path.join(LIB, "libfvgpu.so")
    _run(["nvcc", *ARCH, "-shared", *objs, "-o", out, "-lcudart"])
    return out


def build_all() -> dict:
    with ThreadPoolExecutor(max_workers=2) as ex:
        fm = ex.submit(build_mesh)
        fg = ex.submit(build_gpu)
        return {"mesh": fm.result(), "gpu": fg.result()}


if __name__ == "__main__":
    print(build_all())
