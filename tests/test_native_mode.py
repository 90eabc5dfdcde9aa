"""Native mode: per-node incidence distributions against the reference's.

tests/golden/reference_native.npz holds the new exposures per tick and node
of 200 runs of the reference's unmodified laser_polio (numpy's own generator,
seeds 1..200, no draw hook; tests/golden/make_reference_fixtures.py --native)
on one case: 14 nodes, about 2e4 agents, 120 ticks, all five components, an
outbreak growing from the same initial agent table in every run.

The oracle (CPU) and the engine (GPU) run the same description and table
with their own counter-based draws, seeds 1..200.  Their per-node weekly
incidence must have the reference's distribution:
  - every node-week (14 nodes x 17 weeks): two-sample Kolmogorov-Smirnov,
    family-wise alpha 1e-3 with a Bonferroni correction over the node-weeks
    that have any exposure;
  - every week's total over nodes: Welch's t-test on the means, same
    correction;
  - the run's total: Welch's t-test at alpha 1e-3.
"""

import json
from pathlib import Path

import numpy as np
import pytest
from scipy import stats

from laser_polio_gb300.engine import make_desc

FIXTURE = Path(__file__).resolve().parent / "golden" / "reference_native.npz"
CASE = "native"
ALPHA = 1e-3
WEEKS = 17  # ticks 1..119


def _load():
    with np.load(FIXTURE) as z:
        d = {k: z[k] for k in z.files}
    pre = f"{CASE}/desc/"
    scal = json.loads(bytes(d[pre + "scalars"]).decode())
    p = dict(scal)
    for k, v in d.items():
        if k.startswith(pre) and "/sia_mask/" not in k and k != pre + "scalars":
            p[k[len(pre):]] = v
    p["dur_inf"] = tuple(scal["dur_inf"])
    p["seeds"] = [tuple(e) for e in scal["seeds"]]
    p["sia"] = [(*e, d[f"{pre}sia_mask/{j}"]) for j, e in enumerate(scal["sia"])]
    p["R_preseed"] = None
    cols = {k.split("/")[-1]: v for k, v in d.items() if k.startswith(f"{CASE}/in/")}
    return p, cols, d[f"{CASE}/new_exposed"], d[f"{CASE}/seeds"]


def weekly(new_exposed):
    """[runs, ticks, nodes] -> [runs, WEEKS, nodes]: sums over ticks 7w+1 .. 7w+7."""
    x = new_exposed[:, 1 : 1 + 7 * WEEKS, :]
    return x.reshape(x.shape[0], WEEKS, 7, x.shape[2]).sum(axis=2)


def compare(ours, ref):
    """The tests of the module docstring; returns the smallest p-values."""
    a, b = weekly(ours), weekly(ref)
    live = [(w, n) for w in range(WEEKS) for n in range(a.shape[2]) if a[:, w, n].any() or b[:, w, n].any()]
    assert len(live) > 100
    ks = [stats.ks_2samp(a[:, w, n], b[:, w, n], method="asymp").pvalue for w, n in live]
    worst_ks = min(ks)
    assert worst_ks > ALPHA / len(live), f"node-week incidence differs (KS p = {worst_ks:.3g}, {len(live)} tests)"
    ta, tb = a.sum(axis=2), b.sum(axis=2)
    tt = [stats.ttest_ind(ta[:, w], tb[:, w], equal_var=False).pvalue for w in range(WEEKS) if ta[:, w].any()]
    worst_t = min(tt)
    assert worst_t > ALPHA / len(tt), f"weekly total incidence differs (t-test p = {worst_t:.3g})"
    tot = stats.ttest_ind(ta.sum(axis=1), tb.sum(axis=1), equal_var=False).pvalue
    assert tot > ALPHA, f"total incidence differs (t-test p = {tot:.3g})"
    return worst_ks, worst_t, tot


def _results(p):
    return np.zeros((p["nt"], p["n_nodes"]), np.int32)


def test_oracle_native_incidence_matches_the_reference():
    from oracle.oracle import OracleSim

    p, cols, ref, seeds = _load()
    assert ref.shape[0] >= 200
    runs = []
    for s in seeds:
        desc, keep = make_desc(dict(p, seed=int(s)))
        o = OracleSim(desc, keepalive=keep)
        try:
            o.bind_columns({k: v.copy() for k, v in cols.items()})
            o.start()
            o.step(p["nt"] - 1)
            ne = _results(p)
            o.read_results({"new_exposed": ne})
        finally:
            o.close()
        runs.append(ne)
    compare(np.stack(runs), ref)


@pytest.mark.gpu
def test_gpu_native_incidence_matches_the_reference():
    """The 200 runs as one batch of replicates on the device."""
    from laser_polio_gb300._lib import Handle

    p, cols, ref, seeds = _load()
    descs = [make_desc(dict(p, seed=int(s))) for s in seeds]
    h = Handle([d for d, _ in descs])
    try:
        for i in range(len(descs)):
            h.bind_columns(i, {k: v.copy() for k, v in cols.items()})
        h.start()
        h.step(p["nt"] - 1)
        h.sync()
        runs = []
        for i in range(len(descs)):
            ne = _results(p)
            h.read_results(i, {"new_exposed": ne})
            runs.append(ne)
    finally:
        h.close()
    compare(np.stack(runs), ref)
