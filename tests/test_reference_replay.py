"""Parity with the reference's own code, in replay mode.

tests/golden/reference_replay.npz holds what the reference's unmodified
laser_polio (SEIR_ABM.run with its five components, imported by
tests/golden/make_reference_fixtures.py) computed on small cases
(tests/golden/replay_cases.py) when every random call of its per-tick step
was answered with the counter-based draw the oracle and the engine use for
the same purpose, tick and slot or node.  Everything else in those runs is
the reference's own arithmetic: its float32 per-thread sums, 1 - exp(-rate),
the float64 cumulative sums and searchsorted of the weighted selection, its
int8/int16 timer arithmetic, its schedules and its early stop.

Here the same description (as the reference computed it: network,
seasonality, birth rates, Kaplan-Meier table, schedules) and the same initial
agent table go to the C oracle (CPU) and to the CUDA engine (GPU).  Every
results array, every agent column, the final tick, count and stop flag must
equal the reference's.  The fixture also records how many draws of each kind
the reference made, so a case that silently stopped exercising a draw fails.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from laser_polio_gb300.engine import make_desc

FIXTURE = Path(__file__).resolve().parent / "golden" / "reference_replay.npz"
CASES = ("busy", "zamfara", "collisions", "stop")


def _load():
    with np.load(FIXTURE) as z:
        return {k: z[k] for k in z.files}


_DATA = None


def data():
    global _DATA
    if _DATA is None:
        _DATA = _load()
    return _DATA


def case(name):
    z = data()
    pre = f"{name}/desc/"
    scal = json.loads(bytes(z[pre + "scalars"]).decode())
    p = dict(scal)
    for k, v in z.items():
        if k.startswith(pre) and "/sia_mask/" not in k and k != pre + "scalars":
            p[k[len(pre):]] = v
    p["dur_inf"] = tuple(scal["dur_inf"])
    p["seeds"] = [tuple(e) for e in scal["seeds"]]
    p["sia"] = [(*e, z[f"{pre}sia_mask/{j}"]) for j, e in enumerate(scal["sia"])]
    p["R_preseed"] = None
    cols = {k.split("/")[-1]: v.copy() for k, v in z.items() if k.startswith(f"{name}/in/")}
    res = {k.split("/")[-1]: v for k, v in z.items() if k.startswith(f"{name}/res/")}
    t, count, stopped = (int(x) for x in z[f"{name}/state"])
    final = {}
    for k, v in z.items():  # the final columns, stored as their XOR with the initial ones
        if k.startswith(f"{name}/out/"):
            col = k.split("/")[-1]
            init = cols[col][:count]
            final[col] = (init.view(v.dtype) ^ v).view(init.dtype)
    calls = json.loads(bytes(z[f"{name}/calls"]).decode())
    return p, cols, res, final, (t, count, stopped), calls


def _results_like(p):
    from laser_polio_gb300 import _abi

    nt, n, ns = p["nt"], p["n_nodes"], p["n_strains"]
    return {name: np.zeros((nt, n, ns) if wide else (nt, n), np.int32) for name, wide in _abi.RESULT_FIELDS}


def _compare(name, res_ref, final_ref, state_ref, res, cols, state):
    assert state == state_ref, f"{name}: (t, count, stopped) {state} vs the reference's {state_ref}"
    for k, a in res_ref.items():
        b = res[k]
        if not np.array_equal(a, b):
            idx = np.argwhere(a != b)
            raise AssertionError(f"{name}: results.{k} differs from the reference's at {len(idx)} entries, "
                                 f"first {idx[:3].tolist()}: {a[tuple(idx[0])]} vs {b[tuple(idx[0])]}")
    count = state_ref[1]
    for k, a in final_ref.items():
        b = cols[k][:count]
        if not np.array_equal(a, b):
            idx = np.flatnonzero(a != b)
            raise AssertionError(f"{name}: people.{k} differs from the reference's at {len(idx)} slots, "
                                 f"first {idx[:5].tolist()}: {a[idx[0]]} vs {b[idx[0]]}")


def test_fixture_exercises_every_draw():
    """Across the cases the reference made every kind of draw of the
    per-tick step, and the cases cover births, SIA, RI, seeds and the stop."""
    total = {}
    for name in CASES:
        *_, state, calls = case(name)
        for k, v in calls.items():
            total[k] = total.get(k, 0) + v
    for k in ("paralysis", "ri", "sia", "zero_inflation", "negbinom", "poisson", "select", "strain", "births", "km",
              "seed_pick", "seed_timer"):
        assert total.get(k, 0) > 0, f"no {k} draw in the replay cases"
    p, _, res, _, state, _ = case("stop")
    assert state[2] == 1 and state[0] < p["nt"]
    _, _, res, _, _, _ = case("busy")
    assert res["sia_vaccinated"].sum() > 0 and res["ri_vaccinated"].sum() > 0 and res["births"].sum() > 0
    assert res["new_paralyzed"].sum() > 0 and res["ipv_vaccinated"].sum() > 0


@pytest.mark.parametrize("name", CASES)
def test_oracle_equals_the_reference(name):
    from oracle.oracle import OracleSim

    p, cols, res_ref, final_ref, state_ref, _ = case(name)
    desc, keep = make_desc(p)
    o = OracleSim(desc, keepalive=keep)
    try:
        o.bind_columns(cols)
        o.start()
        o.step(p["nt"] - 1)
        res = _results_like(p)
        o.read_results(res)
        o.read_columns(cols)
        st = o.state()
    finally:
        o.close()
    _compare(name, res_ref, final_ref, state_ref, res, cols, (st.t, st.count, st.stopped))


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_engine_equals_the_reference(name):
    from laser_polio_gb300._lib import Handle

    p, cols, res_ref, final_ref, state_ref, _ = case(name)
    desc, keep = make_desc(p)
    h = Handle([desc])
    try:
        h.bind_columns(0, cols)
        h.start()
        h.step(p["nt"] - 1)
        h.sync()
        res = _results_like(p)
        h.read_results(0, res)
        h.read_columns(0, cols)
        st = h.state(0)
    finally:
        h.close()
    _compare(name, res_ref, final_ref, state_ref, res, cols, (st.t, st.count, st.stopped))
