"""Build the CUDA engine (liblpg.so) in-tree for sm_103a with nvcc.

    python -m laser_polio_gb300.build

Each translation unit compiles to an object in parallel; one nvcc call
links them into the shared library.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build" / "liblpg.so"
SOURCES = [CSRC / "lpg_engine.cu", CSRC / "lpg_ops.cu", CSRC / "lpg_adjoint.cu", CSRC / "lpg_init.cu",
           CSRC / "lpg_export.cpp", CSRC / "lpg_network.cpp"]
DEPS = SOURCES + [CSRC / "lpg_kernels.cuh", CSRC / "lpg_engine.cuh", CSRC / "lpg_rng.h", CSRC / "lpg_detmath.h",
                  CSRC / "lpg_ri.h", CSRC / "lpg_init.h", ROOT / "include" / "lpg.h"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler",
         "-fPIC,-ffp-contract=off,-fno-math-errno,-pthread"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def build(force: bool = False, verbose: bool = False) -> Path:
    newest = max(p.stat().st_mtime for p in DEPS)
    if OUT.exists() and OUT.stat().st_mtime >= newest and not force:
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tag = os.getpid()
    objs = [OUT.parent / f"{s.stem}.{tag}.o" for s in SOURCES]
    procs = []
    for src, obj in zip(SOURCES, objs):
        cmd = [nvcc(), ARCH, *FLAGS, f"-I{ROOT / 'include'}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((cmd, subprocess.Popen(cmd)))
    failed = [cmd for cmd, p in procs if p.wait() != 0]
    if failed:
        for obj in objs:
            obj.unlink(missing_ok=True)
        raise subprocess.CalledProcessError(1, failed[0])
    tmp = OUT.with_suffix(f".{tag}.tmp")
    try:
        subprocess.run([nvcc(), ARCH, "-shared", "-Xcompiler", "-pthread", *[str(o) for o in objs], "-o", str(tmp)],
                       check=True)
    finally:
        for obj in objs:
            obj.unlink(missing_ok=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    import sys

    print(build(force=True, verbose="-v" in sys.argv))
