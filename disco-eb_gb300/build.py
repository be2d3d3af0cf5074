"""Build the CUDA library (sm_103a) in-tree: ``disco-eb_gb300/_build/libdiscoeb_gb300.so``.

The translation units are compiled to objects in parallel, then linked.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = [os.path.join(HERE, "csrc", f) for f in ("deb_solver.cu", "deb_adjoint.cu", "deb_observables.cu", "deb_tables.cu")]
HDRS = [os.path.join(HERE, "csrc", f) for f in ("deb_core.cuh", "deb_adjoint.cuh", "deb_tables_core.cuh",
                                                 "deb_internal.h")]
DEPS = SRC + HDRS + [os.path.join(ROOT, "include", "discoeb_gb300.h")]
OUT = os.path.join(HERE, "_build", "libdiscoeb_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(p) for p in DEPS)
        if os.path.getmtime(OUT) >= newest:
            return OUT
    inc = ["-I", os.path.join(ROOT, "include")]
    objs = [os.path.join(HERE, "_build", os.path.basename(s)[:-3] + ".o") for s in SRC]

    def compile_one(i):
        cmd = [nvcc()] + FLAGS + (["-Xptxas=-v"] if verbose else []) + inc + ["-c", SRC[i], "-o", objs[i]]
        subprocess.check_call(cmd)

    with ThreadPoolExecutor(max_workers=len(SRC)) as ex:
        list(ex.map(compile_one, range(len(SRC))))
    subprocess.check_call([nvcc(), ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", OUT] + objs)
    return OUT


if __name__ == "__main__":
    print(build(force=True, verbose=True))
