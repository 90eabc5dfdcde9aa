"""Golden outputs of the reference's own code, for the parity tests.

    python tests/golden/make_reference_fixtures.py <reference checkout> [--cases busy,stop]
    python tests/golden/make_reference_fixtures.py <reference checkout> --native 200
    python tests/golden/make_reference_fixtures.py <reference checkout> --init 16

Imports the unmodified laser_polio package from <checkout>/src with the
stand-ins and the draw hook of reference_harness.py, and writes:

  reference_replay.npz  per replay case (replay_cases.py): the simulation
      description the engine takes (as the reference computed it: network,
      seasonality, birth rates, Kaplan-Meier table, schedules), the initial
      agent table, and what the reference's SEIR_ABM.run() left with the
      counter-based draws: every results array, the final agent columns
      (stored as their XOR with the initial ones, which is mostly zeros),
      t, count and the stop flag, and how many draws of each kind it made.
  reference_native.npz  (--native N) the native case's description and
      initial table, and the new exposures per tick and node of N reference
      runs with numpy's own generator (seeds 1 .. N), without the hook.
  reference_init.npz  (--init N) statistics of the reference's own
      initialisation (SEIR_ABM and the five constructors) of the init case,
      seeds 1 .. N: per-node state counts, the missed count, histograms of
      the timers, ages, ages at death and RI offsets, a (risk, infectivity)
      sample, and the age pyramid it read.

The reference checkout is read, never written; the reference's logger writes
its log files under a temporary working directory.
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

DIST_KINDS = {"constant": 0, "exponential": 1, "gamma": 2, "lognormal": 3, "normal": 4, "poisson": 5, "uniform": 6,
              "lognormal_int": 7}


def dist_spec(d):
    """(kind, p1, p2) of a reference Distribution, in lpg_dist's terms."""
    k = d.dist_type
    q = d.pars
    if k == "constant":
        return 0, float(q.get("value", 1)), 0.0
    if k == "exponential":
        return 1, float(q.get("scale", 1.0)), 0.0
    if k == "gamma":
        return 2, float(q.get("shape", 2.0)), float(q.get("scale", 1.0))
    if k in ("lognormal", "lognormal_int"):
        return DIST_KINDS[k], float(q.get("mean", 1.0)), float(q.get("sigma", 0.5))
    if k == "normal":
        return 4, float(q.get("mean", 0.0)), float(q.get("std", 1.0))
    if k == "poisson":
        return 5, float(q.get("lam", 5)), 0.0
    if k == "uniform":
        return 6, float(q.get("min", 2)), float(q.get("max", 10))
    raise ValueError(k)


def vaccine_strain(vt):
    if "nOPV" in vt:
        return 2
    return 1


def describe(lp, sim):
    """make_desc's parameters from the reference's own objects."""
    pars = sim.pars
    inst = {type(c).__name__: c for c in sim.instances}
    n = len(sim.nodes)
    ns = len(pars.strain_ids)
    bits = {"VitalDynamics_ABM": 1, "DiseaseState_ABM": 2, "RI_ABM": 4, "SIA_ABM": 8, "Transmission_ABM": 16}
    mask = sum(b for name, b in bits.items() if name in inst)
    vd, ds, tx, sia = (inst.get(k) for k in ("VitalDynamics_ABM", "DiseaseState_ABM", "Transmission_ABM", "SIA_ABM"))
    seeds = []
    for t, entries in ds.seed_schedule.items():
        for node, value in entries:
            seeds.append((int(t), int(node), 0 if isinstance(value, float) else 1, float(value)))
    seas = np.zeros(sim.nt)
    t0 = sim.t
    for t in range(sim.nt):  # the reference's own get_seasonality at every tick
        sim.t = t
        seas[t] = lp.get_seasonality(sim)
    sim.t = t0
    events = []
    if sia is not None and pars.vx_prob_sia is not None:
        for ev in sia.sia_schedule:
            t = (lp.date(ev["date"]) - pars.start_date).days
            if 1 <= t < sim.nt:
                mask_n = np.zeros(n, np.uint8)
                mask_n[ev["nodes"]] = 1
                events.append((t, vaccine_strain(ev["vaccinetype"]), int(ev["age_range"][0]), int(ev["age_range"][1]),
                               float(pars["vx_efficacy"][ev["vaccinetype"]]), mask_n))
    ri_type = pars["ri_vaccine_type"] if "ri_vaccine_type" in pars else "tOPV"

    def node_vec(v, dtype=np.float64):
        a = np.asarray(v, dtype=dtype)
        return np.full(n, a, dtype=dtype) if a.ndim == 0 else a

    return {
        "n_nodes": n, "n_strains": ns, "nt": sim.nt, "count": sim.people.count, "capacity": sim.people.capacity,
        "seed": int(pars.seed), "components": mask,
        "stop_if_no_cases": int(bool(pars["stop_if_no_cases"])),
        "vd_step": int(pars.step_size_VitalDynamics_ABM), "birth_rate": np.asarray(vd.birth_rate, np.float64),
        "km_cumdeaths": np.asarray(vd.death_estimator.cumulative_deaths, np.int64), "km_max_year": 100,
        "p_paralysis": float(np.float32(pars.p_paralysis)), "seeds": seeds, "dur_inf": dist_spec(pars.dur_inf),
        "ri_step": int(pars.step_size_RI_ABM), "ri_enabled": int(pars["vx_prob_ri"] is not None),
        "ri_strain": vaccine_strain(ri_type),
        "vx_prob_ri": node_vec(pars["vx_prob_ri"] if pars["vx_prob_ri"] is not None else 0.0),
        "vx_prob_ipv": node_vec(pars["vx_prob_ipv"] if pars["vx_prob_ipv"] is not None else 0.0),
        "sia": events,
        "vx_prob_sia": node_vec(pars.vx_prob_sia if pars.vx_prob_sia is not None else 0.0, np.float32),
        "strain_r0_scalars": np.array(list(pars.strain_r0_scalars.values()), np.float64)[:ns],
        "network": np.asarray(tx.network, np.float64), "r0_scalars": node_vec(pars.r0_scalars),
        "seasonality": seas, "zero_inflation": float(pars.node_seeding_zero_inflation),
        "nb_r": int(max(1, int(np.round(pars.node_seeding_dispersion)))),
        "pop0": np.asarray(sim.results.pop[0], np.int32), "R_preseed": None,
    }


def changed_bits(final, initial):
    """final XOR initial, as unsigned integers of the column's width."""
    u = np.dtype(f"u{final.dtype.itemsize}")
    return final.view(u) ^ initial.view(u)


def pack_desc(prefix, p, out):
    """Arrays under prefix/…; scalars, seed events and SIA events as JSON."""
    scal = {}
    for k, v in p.items():
        if k == "sia":
            scal["sia"] = [[int(e[0]), int(e[1]), int(e[2]), int(e[3]), float(e[4])] for e in v]
            for j, e in enumerate(v):
                out[f"{prefix}/sia_mask/{j}"] = e[5]
        elif k == "seeds":
            scal["seeds"] = [list(e) for e in v]
        elif k == "dur_inf":
            scal["dur_inf"] = list(v)
        elif isinstance(v, np.ndarray):
            out[f"{prefix}/{k}"] = v
        else:
            scal[k] = v
    out[f"{prefix}/scalars"] = np.frombuffer(json.dumps(scal).encode(), dtype=np.uint8)


def run_replay(lp, harness, cases_mod, name, pyramid):
    from laser_core.propertyset import PropertySet  # the stand-in

    pars = cases_mod.make_pars(name, lp, PropertySet, pyramid)
    sim = lp.SEIR_ABM(pars)  # the reference's own init, with numpy's global RNG
    sim.components = cases_mod.components(lp)
    cols = cases_mod.initial_columns(name, sim.people.count, sim.people.capacity, np.asarray(sim.pars.init_pop),
                                     seed=1000 + sum(map(ord, name)))
    for k, v in cols.items():
        getattr(sim.people, k)[:] = v
    desc = describe(lp, sim)
    vd = next(c for c in sim.instances if type(c).__name__ == "VitalDynamics_ABM")
    hook = harness.DrawHook(sim, [(s[0], s[1], s[3]) for s in desc["seeds"]], desc["dur_inf"])
    mods = [sys.modules["laser_polio.model"], sys.modules["laser_polio.distributions"]]
    vd.death_estimator.predict_age_at_death = harness.km_hook_factory(hook, desc["km_cumdeaths"], 100)
    harness.attach(mods, hook)
    try:
        sim.run()
    finally:
        harness.detach(mods)
    res = {k: v for k, v in vars(sim.results).items() if isinstance(v, np.ndarray) and v.dtype == np.int32}
    final = {k: np.array(getattr(sim.people, k)) for k in cols}
    state = {"t": int(sim.t), "count": int(sim.people.count), "stopped": int(bool(sim.should_stop))}
    return desc, cols, res, final, state, hook.calls


NATIVE_CASE = "native"
_NATIVE = {}


def _native_worker_init(ref):
    import reference_harness as harness

    os.chdir(tempfile.mkdtemp())  # the reference's logger writes logs/ into the working directory
    _NATIVE["lp"] = harness.import_reference(Path(ref) / "src")
    _NATIVE["pyramid"] = Path(ref) / "data" / "Nigeria_age_pyramid_2024.csv"


def _native_run(seed):
    """One reference run of the native case with numpy's own generator
    seeded with ``seed`` (laser_core's seed, through SEIR_ABM's init): the
    new exposures per tick and node."""
    import replay_cases
    from laser_core.propertyset import PropertySet

    lp = _NATIVE["lp"]
    pars = replay_cases.make_pars(NATIVE_CASE, lp, PropertySet, _NATIVE["pyramid"])
    pars.seed = int(seed)
    sim = lp.SEIR_ABM(pars)
    sim.components = replay_cases.components(lp)
    cols = replay_cases.initial_columns(NATIVE_CASE, sim.people.count, sim.people.capacity,
                                        np.asarray(sim.pars.init_pop), seed=1000 + sum(map(ord, NATIVE_CASE)))
    for k, v in cols.items():
        getattr(sim.people, k)[:] = v
    sim.run()
    return np.asarray(sim.results.new_exposed, np.int32)


def native(ref, n_seeds, out_path, workers):
    """reference_native.npz: the native case's description and initial table
    (as in the replay file) and the reference's new exposures per tick and
    node for seeds 1 .. n_seeds."""
    import multiprocessing as mp

    import reference_harness as harness
    import replay_cases

    cwd = os.getcwd()
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            lp = harness.import_reference(Path(ref) / "src")
            from laser_core.propertyset import PropertySet

            pars = replay_cases.make_pars(NATIVE_CASE, lp, PropertySet, Path(ref) / "data" / "Nigeria_age_pyramid_2024.csv")
            sim = lp.SEIR_ABM(pars)
            sim.components = replay_cases.components(lp)
            cols = replay_cases.initial_columns(NATIVE_CASE, sim.people.count, sim.people.capacity,
                                                np.asarray(sim.pars.init_pop), seed=1000 + sum(map(ord, NATIVE_CASE)))
            for k, v in cols.items():
                getattr(sim.people, k)[:] = v
            pack_desc(f"{NATIVE_CASE}/desc", describe(lp, sim), out)
            for k, v in cols.items():
                out[f"{NATIVE_CASE}/in/{k}"] = v
        finally:
            os.chdir(cwd)
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers, initializer=_native_worker_init, initargs=(str(ref),)) as pool:
        runs = pool.map(_native_run, range(1, n_seeds + 1))
    out[f"{NATIVE_CASE}/new_exposed"] = np.stack(runs)
    out[f"{NATIVE_CASE}/seeds"] = np.arange(1, n_seeds + 1)
    np.savez_compressed(out_path, **out)
    tot = out[f"{NATIVE_CASE}/new_exposed"].sum(axis=(1, 2))
    print(f"wrote {out_path}: {n_seeds} reference runs, total new exposures mean {tot.mean():.1f} "
          f"sd {tot.std():.1f} ({Path(out_path).stat().st_size} bytes)")


INIT_CASE = "init"

def _init_run(seed):
    import replay_cases
    from laser_core.propertyset import PropertySet
    from replay_cases import init_statistics

    lp = _NATIVE["lp"]
    pars = replay_cases.make_pars(INIT_CASE, lp, PropertySet, _NATIVE["pyramid"])
    pars.seed = int(seed)
    sim = lp.SEIR_ABM(pars)
    sim.components = replay_cases.components(lp)
    return init_statistics(sim.people, sim.people.count, sim.people.capacity), int(sim.people.capacity)


def init_fixture(ref, n_seeds, out_path, workers):
    """reference_init.npz: statistics of the reference's own initialisation
    of the init case for seeds 1 .. n_seeds, summed over seeds (histograms,
    counts) or stacked (the risk and infectivity sample of each run), with
    the age pyramid it read."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Pool(workers, initializer=_native_worker_init, initargs=(str(ref),)) as pool:
        runs = pool.map(_init_run, range(1, n_seeds + 1))
    out = {}
    for k in runs[0][0]:
        vals = [r[0][k] for r in runs]
        out[k] = np.concatenate(vals, axis=1) if k == "risk_inf" else (np.stack(vals) if k in ("state_by_node", "missed")
                                                                       else np.sum(vals, axis=0))
    import reference_harness  # noqa: F401
    from laser_polio_gb300.core import load_pyramid_csv

    out["pyramid"] = load_pyramid_csv(Path(ref) / "data" / "Nigeria_age_pyramid_2024.csv")
    out["capacity"] = np.array([runs[0][1]])
    out["seeds"] = np.arange(1, n_seeds + 1)
    np.savez_compressed(out_path, **out)
    print(f"wrote {out_path}: {n_seeds} reference initialisations ({Path(out_path).stat().st_size} bytes)")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference", help="path of the laser-polio checkout")
    ap.add_argument("--cases", default=None)
    ap.add_argument("--out", default=str(HERE / "reference_replay.npz"))
    ap.add_argument("--native", type=int, default=0, metavar="N",
                    help="instead: N reference runs of the native case with numpy's own generator")
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--init", type=int, default=0, metavar="N",
                    help="instead: statistics of N reference initialisations of the init case")
    args = ap.parse_args()
    ref = Path(args.reference).resolve()
    if args.init:
        init_fixture(ref, args.init, HERE / "reference_init.npz", args.workers)
        return
    if args.native:
        native(ref, args.native, HERE / "reference_native.npz", args.workers)
        return
    pyramid = ref / "data" / "Nigeria_age_pyramid_2024.csv"
    import reference_harness as harness
    import replay_cases

    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)  # the reference's logger writes logs/ into the working directory
        try:
            lp = harness.import_reference(ref / "src")
            out = {}
            names = args.cases.split(",") if args.cases else list(replay_cases.CASES)
            for name in names:
                desc, cols, res, final, state, calls = run_replay(lp, harness, replay_cases, name, pyramid)
                pack_desc(f"{name}/desc", desc, out)
                for k, v in cols.items():
                    out[f"{name}/in/{k}"] = v
                for k, v in res.items():
                    out[f"{name}/res/{k}"] = v
                for k, v in final.items():  # stored as the bits that changed (mostly zeros)
                    out[f"{name}/out/{k}"] = changed_bits(v[: state["count"]], cols[k][: state["count"]])
                out[f"{name}/state"] = np.array([state["t"], state["count"], state["stopped"]], np.int64)
                out[f"{name}/calls"] = np.frombuffer(json.dumps(calls).encode(), dtype=np.uint8)
                print(f"{name}: t={state['t']} count={state['count']} stopped={state['stopped']} "
                      f"new_exposed={int(res['new_exposed'].sum())} draws={calls}", flush=True)
        finally:
            os.chdir(cwd)
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out} ({Path(args.out).stat().st_size} bytes)")


if __name__ == "__main__":
    main()
