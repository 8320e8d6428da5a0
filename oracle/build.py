"""Build recipes for the oracle (test infrastructure only).

Two shared libraries come out of this script:

* ``oracle/_build/liboracle.so`` -- the CPU restatement of the reference's
  residual / RK path (``oracle/fvoracle.c``), plain C.  Built on every machine.
* ``oracle/_ref/libfvref.so`` -- the reference's own hot-path sources,
  compiled unchanged from the reference tree, linked with
  ``oracle/ref_harness.c``.  Built only where the reference tree exists.

Both use ``-O2 -fno-fast-math -ffp-contract=off`` so that no multiply-add is
fused on any host (GCC fuses by default on aarch64), which keeps the
arithmetic identical to the reference's order of operations.

Usage: ``python oracle/build.py [--ref-root PATH]``.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CFLAGS = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-fPIC", "-std=gnu99"]


def default_ref_root() -> str:
    """The reference tree: FV_REFERENCE_ROOT, else a directory named
    "reference" beside the repository."""
    return os.environ.get("FV_REFERENCE_ROOT") or os.path.join(os.path.dirname(REPO), "reference")


# The reference files on the residual / RK path, plus the allocation helpers
# the harness calls (leafallocation, memallocation, createutility) and what
# they pull in at link time.
REF_SOURCES = [
    "RK", "RHS", "RHS_nb", "residual_faces_AMR", "hllc_euler", "compute_wave_speeds",
    "star_region_euler", "flux_adv", "flux_viscous", "facevalues", "facercnstr", "bc",
    "bc_inlet", "asinvalues", "asinvalues_multiphase", "barotropic_eos", "rotate_vectors",
    "pvrs_mc", "leafallocation", "memallocation", "createutility", "faceinterp", "distance",
    "deltavalues", "facevalues_MUSCL", "reconctruct_V3", "cons2primtv", "prim2conc",
    "operatetp", "gradcalc", "timecpu", "criterionsplt",
    # the Tecplot writer (loop.c:55) and what it links: volmvalues, message, getMemory,
    # tag2adr (communicate1.c)
    "exportfield_linked_V3", "volmvalues", "message", "getMemory", "communicate1",
    # the geometry routines (refh_geometry): areas, volumes, face frames
    "meshproperties", "normalvector", "tagvector",
]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_oracle() -> str:
    """Compile the C restatement into oracle/_build/liboracle.so."""
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle.so")
    src = os.path.join(HERE, "fvoracle.c")
    _run(["gcc", *CFLAGS, "-fopenmp", "-shared", "-I", os.path.join(REPO, "include"), src, "-o", out,
          "-lm"])
    return out


def build_oracle_ad() -> str:
    """Compile the scalar-templated restatement (exact JVPs) into
    oracle/_build/liboracle_ad.so."""
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle_ad.so")
    _run(["g++", "-O2", "-std=c++17", "-fno-fast-math", "-ffp-contract=off", "-fPIC", "-shared", "-I",
          os.path.join(REPO, "include"), os.path.join(HERE, "fvoracle_ad.cpp"), "-o", out])
    return out


def build_ref(ref_root: str | None = None) -> str | None:
    ref_root = ref_root or default_ref_root()
    """Compile the reference's hot path + harness into oracle/_ref/libfvref.so.

    Returns None when the reference tree is absent (e.g. on a GPU host)."""
    if not os.path.isfile(os.path.join(ref_root, "strdata.h")):
        return None
    out_dir = os.path.join(HERE, "_ref")
    obj_dir = os.path.join(out_dir, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "stubs"), "-I", ref_root]
    jobs = []
    for name in REF_SOURCES:
        jobs.append(["gcc", *CFLAGS, "-w", *inc, "-c", os.path.join(ref_root, name + ".c"),
                     "-o", os.path.join(obj_dir, name + ".o")])
    jobs.append(["gcc", *CFLAGS, "-Wall", "-Wno-unused-function", *inc, "-c",
                 os.path.join(HERE, "ref_harness.c"), "-o", os.path.join(obj_dir, "ref_harness.o")])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    out = os.path.join(out_dir, "libfvref.so")
    objs = [os.path.join(obj_dir, n + ".o") for n in REF_SOURCES + ["ref_harness"]]
    _run(["gcc", "-shared", *objs, "-o", out, "-lm"])
    return out


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=None, help="reference tree (default: FV_REFERENCE_ROOT, else ../reference)")
    a = ap.parse_args(argv)
    print(build_oracle())
    print(build_oracle_ad())
    print(build_ref(a.ref_root))
    return 0


if __name__ == "__main__":
    sys.exit(main())
