"""The C ABI: header, ctypes mirror and built library agree (no GPU needed)."""

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from laser_polio_gb300 import _abi
from laser_polio_gb300 import _lib
from laser_polio_gb300 import build

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "lpg.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lpg_[a-z_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = C.CDLL(str(path))
    missing = [name for name in declared_functions() if not hasattr(lib, name)]
    assert not missing, f"not exported: {missing}"
    assert set(declared_functions()) <= set(_lib.SIGNATURES), "ctypes wrapper lacks a declared entry point"
    assert lib.lpg_version() == 1


def test_struct_layout_matches_header(tmp_path):
    structs = {
        "lpg_sim_desc": _abi.lpg_sim_desc,
        "lpg_columns": _abi.lpg_columns,
        "lpg_results_view": _abi.lpg_results_view,
        "lpg_sia_event": _abi.lpg_sia_event,
        "lpg_seed_event": _abi.lpg_seed_event,
        "lpg_dist": _abi.lpg_dist,
        "lpg_sim_state": _abi.lpg_sim_state,
        "lpg_profile": _abi.lpg_profile,
        "lpg_incidence_in": _abi.lpg_incidence_in,
        "lpg_incidence_grad": _abi.lpg_incidence_grad,
        "lpg_incidence_params": _abi.lpg_incidence_params,
        "lpg_init_desc": _abi.lpg_init_desc,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "lpg.h"', "int main(void){"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{name}.{fname} %zu\\n", offsetof({name}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.rsplit(" ", 1) for line in out if line)
    for name, cls in structs.items():
        assert int(got[name]) == C.sizeof(cls), name
        for fname, _ in cls._fields_:
            assert int(got[f"{name}.{fname}"]) == getattr(cls, fname).offset, f"{name}.{fname}"


def test_create_without_gpu_reports_cuda_error():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    d = _abi.lpg_sim_desc()
    h = C.c_void_p()
    rc = lib.lpg_create(C.byref(d), 1, 0, C.byref(h))
    assert rc != 0
    lib.lpg_destroy(h)


def test_counter_names_follow_header_enum():
    text = HEADER.read_text()
    found = dict((m.group(1).lower(), int(m.group(2))) for m in re.finditer(r"LPG_CTR_([A-Z_]+)\s*=\s*(\d+)", text))
    assert [found[n] for n in _abi.COUNTER_NAMES] == list(range(len(_abi.COUNTER_NAMES)))
    assert int(re.search(r"LPG_NUM_COUNTERS\s*=\s*(\d+)", text).group(1)) == len(_abi.COUNTER_NAMES)
