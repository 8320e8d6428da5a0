"""Builds the reference's host program, main() included, as two executables
(test infrastructure only; needs the reference tree):

* ``tests/compat/_build/refmain_cpu`` -- every reference source compiled
  unchanged, the compat layer (fv_140823_gb300/csrc/compat: serial MPI,
  METIS/ParMETIS/PETSc stand-ins, cellallocation, brchconn, wall ghosts) and
  its CPU time step (fvcompat_cpu.c);
* ``tests/compat/_build/refmain_shim`` -- the same minus RHS, RHS_nb, RK,
  faceinterp and gradcalc, with the drop-in shim (csrc/shim/fvshim.c) in their
  place and tests/shim/fake_fvgpu.c serving its libfvgpu calls from the
  oracle's C restatement.

Both wrap advancetimeexplicit with tests/compat/dump_wrap.c, which writes the
leaves' final state to $FVCOMPAT_DUMP.  Run as ``<exe> <case> <run>`` in the
directory of a deck (fv_140823_gb300.decks.write_deck).
"""
from __future__ import annotations

import glob
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")
CFLAGS = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-std=gnu99"]
REPLACED = ("RHS", "RHS_nb", "RK", "faceinterp", "gradcalc")


def default_ref_root() -> str:
    return os.environ.get("FV_REFERENCE_ROOT") or os.path.join(os.path.dirname(REPO), "reference")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(ref_root: str | None = None) -> dict[str, str] | None:
    ref_root = ref_root or default_ref_root()
    if not os.path.isfile(os.path.join(ref_root, "strdata.h")):
        return None
    compat = os.path.join(REPO, "fv_140823_gb300", "csrc", "compat")
    inc = ["-I", os.path.join(compat, "include"), "-I", ref_root, "-I", os.path.join(REPO, "include")]
    obj = os.path.join(OUT, "obj")
    os.makedirs(obj, exist_ok=True)
    ref_names = sorted(os.path.basename(p)[:-2] for p in glob.glob(os.path.join(ref_root, "*.c")))
    jobs = [["gcc", *CFLAGS, "-w", *inc, "-c", os.path.join(ref_root, n + ".c"), "-o", os.path.join(obj, n + ".o")]
            for n in ref_names]
    own = {
        "fvcompat": os.path.join(compat, "fvcompat.c"),
        "fvcompat_cpu": os.path.join(compat, "fvcompat_cpu.c"),
        "fvshim": os.path.join(REPO, "fv_140823_gb300", "csrc", "shim", "fvshim.c"),
        "fake_fvgpu": os.path.join(REPO, "tests", "shim", "fake_fvgpu.c"),
        "fvoracle": os.path.join(REPO, "oracle", "fvoracle.c"),
        "dump_wrap": os.path.join(HERE, "dump_wrap.c"),
    }
    for n, src in own.items():
        jobs.append(["gcc", *CFLAGS, "-Wall", "-Wno-unused-function", *inc, "-c", src, "-o", os.path.join(obj, n + ".o")])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    o = lambda names: [os.path.join(obj, n + ".o") for n in names]  # noqa: E731
    wrap = ["-Wl,--wrap=advancetimeexplicit"]
    exes = {
        "cpu": (o(ref_names) + o(["fvcompat", "fvcompat_cpu", "dump_wrap"])),
        "shim": (o([n for n in ref_names if n not in REPLACED]) +
                 o(["fvcompat", "fvshim", "fake_fvgpu", "fvoracle", "dump_wrap"])),
    }
    out = {}
    for k, objs in exes.items():
        path = os.path.join(OUT, "refmain_" + k)
        _run(["gcc", *objs, *wrap, "-o", path, "-lm"])
        out[k] = path
    return out


if __name__ == "__main__":
    print(build())
