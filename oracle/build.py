"""Compile the C restatement of the reference tick into oracle/_build/.

Test infrastructure (see oracle/__init__.py).  gcc only, no build system:
    python -m oracle.build
"""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_build" / "liblpg_oracle.so"
SRC = HERE / "lpg_oracle.c"
HEADERS = [ROOT / "include" / "lpg.h", ROOT / "laser_polio_gb300" / "csrc" / "lpg_rng.h",
           ROOT / "laser_polio_gb300" / "csrc" / "lpg_detmath.h", ROOT / "laser_polio_gb300" / "csrc" / "lpg_init.h"]


def build(force: bool = False) -> Path:
    newest = max(p.stat().st_mtime for p in [SRC, *HEADERS])
    if OUT.exists() and OUT.stat().st_mtime >= newest and not force:
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(f".{os.getpid()}.tmp")
    cmd = [
        os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-math-errno",
        "-fPIC", "-shared", "-Wall", "-Wno-unused-function",
        f"-I{ROOT / 'include'}", f"-I{ROOT / 'laser_polio_gb300' / 'csrc'}",
        str(SRC), "-o", str(tmp), "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
