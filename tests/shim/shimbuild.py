"""Builds tests/shim/_build/libshimtest.so (test infrastructure only).

The library is the reference's own host-side objects (the oracle recipe's
source list minus RHS, RHS_nb, RK, faceinterp and gradcalc), the harness that
builds a RUN from flattened tables (oracle/ref_harness.c), the drop-in shim
(fv_140823_gb300/csrc/shim/fvshim.c) in place of the five removed objects,
and tests/shim/fake_fvgpu.c, which serves the shim's libfvgpu calls with the
oracle's C restatement.  Built only where the reference tree exists.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

def _load_oracle_build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("fv_oracle_build", os.path.join(REPO, "oracle", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


oracle_build = _load_oracle_build()

REPLACED = ("RHS", "RHS_nb", "RK", "faceinterp", "gradcalc")
OUT = os.path.join(HERE, "_build", "libshimtest.so")


def build_shim_test(ref_root: str | None = None) -> str | None:
    ref_root = ref_root or oracle_build.default_ref_root()
    if not os.path.isfile(os.path.join(ref_root, "strdata.h")):
        return None
    obj_dir = os.path.join(HERE, "_build", "obj")
    os.makedirs(obj_dir, exist_ok=True)
    cflags = oracle_build.CFLAGS
    inc = ["-I", os.path.join(REPO, "oracle", "stubs"), "-I", ref_root, "-I", os.path.join(REPO, "include")]
    names = [n for n in oracle_build.REF_SOURCES if n not in REPLACED]
    jobs, objs = [], []
    for n in names:
        o = os.path.join(obj_dir, n + ".o")
        jobs.append(["gcc", *cflags, "-w", *inc, "-c", os.path.join(ref_root, n + ".c"), "-o", o])
        objs.append(o)
    extra = {
        "ref_harness": os.path.join(REPO, "oracle", "ref_harness.c"),
        "fvshim": os.path.join(REPO, "fv_140823_gb300", "csrc", "shim", "fvshim.c"),
        "fake_fvgpu": os.path.join(HERE, "fake_fvgpu.c"),
        "fvoracle": os.path.join(REPO, "oracle", "fvoracle.c"),
    }
    for n, src in extra.items():
        o = os.path.join(obj_dir, n + ".o")
        jobs.append(["gcc", *cflags, "-Wall", "-Wno-unused-function", *inc, "-c", src, "-o", o])
        objs.append(o)
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(oracle_build._run, jobs))
    oracle_build._run(["gcc", "-shared", *objs, "-o", OUT, "-lm"])
    return OUT


if __name__ == "__main__":
    print(build_shim_test())
