"""Build the CUDA engine (liblpg.so) in-tree for sm_103a with nvcc.

    python -m laser_polio_gb300.build
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
SOURCES = [CSRC / "lpg_engine.cu"]
DEPS = SOURCES + [CSRC / "lpg_kernels.cuh", CSRC / "lpg_engine.cuh", CSRC / "lpg_rng.h", CSRC / "lpg_detmath.h",
                  ROOT / "include" / "lpg.h"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def build(force: bool = False, verbose: bool = False) -> Path:
    newest = max(p.stat().st_mtime for p in DEPS)
    if OUT.exists() and OUT.stat().st_mtime >= newest and not force:
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(f".{os.getpid()}.tmp")
    cmd = [
        nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-shared",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-math-errno",
        f"-I{ROOT / 'include'}", f"-I{CSRC}",
        *[str(s) for s in SOURCES], "-o", str(tmp),
    ]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    import sys

    print(build(force=True, verbose="-v" in sys.argv))
