"""Grid sizes of the tick kernels, picked by timing them on the run itself.

The engine launches every grid-stride kernel with as many CTAs as fit at
once (occupancy x SM count).  That is a guess: a kernel whose work per tick
is small (the due list, the selection's few thousand targets, the queues)
can finish sooner on fewer CTAs, and a batch of many replicates may want
more.  The results do not depend on the grid sizes (every kernel updates
exact integer totals; claims and queues do not depend on which CTA runs
them), so the choice can be made on the run's own first ticks:

  - each tunable kernel gets a few candidate sizes (multiples of the SM
    count, the engine's default among them);
  - the tuner steps ``rounds`` x (number of candidates) ticks in profiling
    mode (one CUDA-event pair per kernel launch); on each tick every kernel
    runs its next candidate, so all kernels are measured on the same ticks;
  - each kernel keeps the candidate with the smallest median time, unless it
    is within ``margin`` of the default's, which it then keeps;
  - the choice is cached on disk, keyed by the GPU, the number of replicates,
    nodes and agents (rounded to a power of two), and applied at once to the
    next handle with the same key.

No counterpart in the reference (its calibration runs each replicate as its
own process, calib/objective.py:47-70).
"""

from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np

from . import _abi

DEFAULT_MULTIPLES = {
    "due": (2, 4, 8),
    "sweep_due": (1, 2, 4),
    "select": (1, 2),
    "rounds": (1, 2, 4),
}


def cache_path() -> Path:
    env = os.environ.get("LPG_AUTOTUNE_CACHE")
    if env:
        return Path(env)
    return Path(os.environ.get("XDG_CACHE_HOME", Path.home() / ".cache")) / "laser_polio_gb300" / "autotune.json"


def workload_key(gpu: str, sm_count: int, n_reps: int, nodes: int, agents: int) -> str:
    """Replicates, nodes and agents rounded to powers of two: a key that
    similar runs share."""
    def p2(x):
        return int(2 ** round(np.log2(max(1, x))))

    return f"{gpu}|{sm_count}|reps{p2(n_reps)}|nodes{p2(nodes)}|agents{p2(agents)}"


def candidates(sm_count: int, default: int, multiples, limit):
    """Multiples of the SM count and the default, at most ``limit`` (None:
    the default is the largest)."""
    if limit is None:
        limit = default
    out = sorted({min(limit, max(1, m * sm_count)) for m in multiples} | {default})
    return out


def choose(times: dict, default: int, margin: float = 0.03) -> int:
    """The candidate with the smallest median time; the default unless
    another beats it by more than ``margin`` (relative).  times: candidate ->
    list of times."""
    med = {c: float(np.median(v)) for c, v in times.items() if len(v)}
    if not med:
        return default
    best = min(med, key=lambda c: (med[c], c != default))
    if default in med and med[best] >= med[default] * (1.0 - margin):
        return default
    return best


def load_cache(path=None) -> dict:
    p = Path(path) if path is not None else cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path=None) -> None:
    p = Path(path) if path is not None else cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(f".{os.getpid()}.tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass  # an unwritable cache only means tuning again next time


def tune(handle, key: str, sm_count: int, rounds: int = 3, kernels=None, margin: float = 0.03, cache=True,
         path=None):
    """Grid sizes for ``handle`` (started, at the start of its run): from the
    cache when ``key`` is there, else measured on the next
    rounds x max(candidates) ticks, which advance the run as usual.  Applies
    them and returns ({kernel: blocks}, ticks stepped)."""
    kernels = dict(DEFAULT_MULTIPLES if kernels is None else kernels)
    store = load_cache(path) if cache else {}
    if key in store:
        chosen = {k: int(v) for k, v in store[key].items() if k in _abi.LAUNCH}
        for k, v in chosen.items():
            handle.set_launch(_abi.LAUNCH[k][0], v)
        return chosen, 0
    defaults = {k: handle.get_launch(_abi.LAUNCH[k][0]) for k in kernels}
    cands = {k: candidates(sm_count, defaults[k], kernels[k], _abi.LAUNCH[k][1]) for k in kernels}
    n = max(len(c) for c in cands.values())
    times = {k: {c: [] for c in cands[k]} for k in kernels}
    handle.set_profiling(True)
    try:
        for r in range(rounds):
            for j in range(n):
                pick = {k: cands[k][(j + r) % len(cands[k])] for k in kernels}
                for k, v in pick.items():
                    handle.set_launch(_abi.LAUNCH[k][0], v)
                before = handle.profile()
                handle.step(1)
                handle.sync()
                after = handle.profile()
                for k, v in pick.items():
                    ms = sum(after.get(e, (0.0, 0))[0] - before.get(e, (0.0, 0))[0] for e in _abi.LAUNCH[k][2])
                    ran = sum(after.get(e, (0.0, 0))[1] - before.get(e, (0.0, 0))[1] for e in _abi.LAUNCH[k][2])
                    if ran:
                        times[k][v].append(ms)
    finally:
        handle.set_profiling(False)
    chosen = {k: choose(times[k], defaults[k], margin) for k in kernels}
    for k, v in chosen.items():
        handle.set_launch(_abi.LAUNCH[k][0], v)
    if cache:
        store = load_cache(path)
        store[key] = chosen
        save_cache(store, path)
    return chosen, rounds * n
