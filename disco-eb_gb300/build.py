"""Build the CUDA library (sm_103a) in-tree: ``disco-eb_gb300/_build/libdiscoeb_gb300.so``."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = [os.path.join(HERE, "csrc", "deb_solver.cu"), os.path.join(HERE, "csrc", "deb_observables.cu"),
       os.path.join(HERE, "csrc", "deb_tables.cu")]
DEPS = SRC + [os.path.join(HERE, "csrc", "deb_core.cuh"), os.path.join(ROOT, "include", "discoeb_gb300.h")]
OUT = os.path.join(HERE, "_build", "libdiscoeb_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(p) for p in DEPS)
        if os.path.getmtime(OUT) >= newest:
            return OUT
    cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), "-o", OUT] + SRC
    if verbose:
        cmd.insert(3, "-Xptxas=-v")
    subprocess.check_call(cmd)
    return OUT


if __name__ == "__main__":
    print(build(force=True, verbose=True))
