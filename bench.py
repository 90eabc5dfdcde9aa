"""Benchmark: agent-ticks/s of the per-tick agent step at the Nigeria scale.

Workload (one "step" = one tick of the full agent step: VitalDynamics,
DiseaseState, RI, SIA and Transmission, with the SEIR log) over a synthetic
774-node, 2.2e8-agent population (capacity +30%), seeded numpy draws with
the distributions of the Nigeria-scale configuration.  agent-ticks = sum
over the timed ticks of people.count (slots scanned, dead included, as the
reference's loops do).

  value     W untimed ticks, then K ticks timed with CUDA events on the
            engine's stream, state resident in HBM (the agent table is far
            larger than L2, so no flush is needed between ticks).
  e2e       a full run through the C ABI from pinned host columns to pinned
            host result arrays and columns: upload, layout, all ticks, read
            back results and columns (phases_s gives the split).
  roofline  per-kernel CUDA-event times from a second run of the same ticks
            in profiling mode; the dominant kernel's algorithmic bytes per
            launch / its mean launch time against the measured HBM peak.
  cpu_baseline  the C/OpenMP oracle on the machine's cores over the same W + K
            ticks of the same population (ticks W+1 .. W+K timed).
  parity    the oracle's results and agent columns after those ticks
            compared, every array and every slot, with the end-to-end run's.
  full_run  the whole 2555-tick run replayed on the device, and the mean
            time of each kind of tick (plain, births, RI, SIA days).
  e2e_api   the user's path at the same scale: SEIR_ABM(pars), the five
            components (agent table initialised on the device), run() over
            all ticks; wall time of construction and run.
  batch     the metric's second half: 64 calibration replicates (1e6-2e7
            agents each, about 4e8 in all) over the same ticks in one handle,
            against the same replicates run one after another.

Other lines, one per call:
  --batch R       the batch measurement alone.
  --incidence T   the adjoint of expected incidence over T ticks, on
                  aggregates recorded by Nigeria-scale forward runs
                  (--incidence-data synthetic: seeded aggregates).
  --continental   4000 nodes, 1e9 agents, 365 ticks through SEIR_ABM, a
                  profiling pass over the whole run and 4 parameter-set
                  replicates of one table (with --incidence: the adjoint on
                  aggregates of the continental shapes).
  --export        the results CSV writer (host only).

python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""

from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# column bytes the reference's per-tick loops read per agent-tick, each column once, by tick type
B_EVERY = 18.0  # state, node, strain, 3 timers, pp, paralyzed, ipv, risk, infectivity
B_VD = 4.0  # date_of_death on VD ticks
B_RI = 5.0  # ri_timer read + write, chronically_missed on RI ticks
B_SIA = 5.0  # date_of_birth, chronically_missed on SIA days


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--agents", type=float, default=None, help="agents (2.2e8; 1e9 with --continental)")
    ap.add_argument("--nodes", type=int, default=None, help="nodes (774; 4000 with --continental)")
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--cpu-seconds", type=float, default=25.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--no-full-run", action="store_true")
    ap.add_argument("--no-api", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-reps", type=int, default=64, help="replicates of the batch leg of the default line")
    ap.add_argument("--parity-ticks", type=int, default=60,
                    help="the oracle's parity leg runs min(W + K, this) ticks of the same population")
    ap.add_argument("--out", default=None)
    ap.add_argument("--batch", type=int, default=0,
                    help="instead: R calibration replicates (730 ticks) batched in one handle vs run one by one")
    ap.add_argument("--incidence", type=int, default=0, metavar="T",
                    help="instead: loss and gradient of the expected incidence over T ticks (the adjoint)")
    ap.add_argument("--incidence-data", default="replay", choices=["replay", "synthetic"],
                    help="the adjoint's aggregates: recorded by Nigeria-scale forward runs, or seeded numpy")
    ap.add_argument("--continental", action="store_true",
                    help="instead: the 4000-node, 1e9-agent workload through the user's path (365 ticks); "
                         "with --incidence, the adjoint on seeded aggregates of its shapes")
    ap.add_argument("--continental-reps", type=int, default=4,
                    help="parameter-set replicates of the continental table in one handle (1e9 agents in all)")
    ap.add_argument("--export", action="store_true",
                    help="instead: save_sim_results' CSV of a Nigeria-scale results table (host only)")
    args = ap.parse_args()
    if args.agents is None:
        args.agents = 1e9 if args.continental else 2.2e8
    if args.nodes is None:
        args.nodes = 4000 if args.continental else 774
    return args


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_over_ranks(ms, agent_ticks, ws, device):
    """Whole-job figures of N independent replicas (one per rank): the
    slowest rank's time and the agent-ticks of all ranks."""
    if ws <= 1:
        return ms, agent_ticks
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    a = torch.tensor([agent_ticks], device=device, dtype=torch.float64)
    dist.all_reduce(a)
    return float(t.item()), float(a.item())


def tick_bytes(params, t):
    """Bytes per agent slot on tick t of every column the reference's loops
    read that tick, each counted once (state, node, strain, three timers,
    paralysis flags, IPV flag, risk, infectivity; date of death on VD ticks;
    RI timer and chronically-missed flag on RI ticks; date of birth and the
    flag on SIA days)."""
    b = B_EVERY
    if t % params["vd_step"] == 0:
        b += B_VD
    if params["ri_enabled"] and t % params["ri_step"] == 0:
        b += B_RI
    b += B_SIA * sum(1 for e in params["sia"] if e[0] == t)
    return b


def sweep_b_bytes(params, t):
    """Column bytes k_sweep_rs stages per agent slot on tick t: on SIA days
    state, chronically_missed and date_of_birth, plus ri_timer and the
    reference index when RI falls on the same day; 0 on other ticks (RI
    alone goes through the due index, counted by the work counters)."""
    ri = bool(params["ri_enabled"]) and t % params["ri_step"] == 0
    sia = any(e[0] == t for e in params["sia"])
    if not sia:
        return 0.0
    return 1.0 + 1.0 + 4.0 + (6.0 if ri else 0.0)


# DRAM bytes ncu measured per unit of counted work, by kernel: (counter,
# bytes per unit, bytes per launch besides), and where they were measured.
NCU_TRAFFIC_PER_UNIT = {"k_select": ("sel_targets", 950.0, 0.0)}
NCU_TRAFFIC_SOURCE = {
    "k_select": "ncu DRAM read+write of k_sel_round0 + k_sel_rounds per target located, "
                "on tick 151 of the 5e7-agent Nigeria-like case, times the targets of the timed ticks",
}


# Algorithmic bytes per unit of counted work (the device work counters of
# lpg_read_counters), by kernel:
#   k_due: 4 B per sub-block index entry read; 8 B per due sub-block
#     listed.
#   k_sweep_due (k_sweep_a): per listed 128-slot sub-block its 8 B list
#     entry and 128 state bytes; 512 B of event ticks and a 4 B index write
#     when an event is due; 512 B of dates of death and a 4 B index write
#     when a death is due; per queue entry the 8 B entry written and read
#     back, then state, strain, three timers and the event tick read (9 B)
#     and state, timers and event tick written (8 B).
#   k_evb: per queue entry the 8 B entry, then state, RI timer, flags and
#     date of birth read (10 B) and state and timer written (5 B).
#   k_select: per target located, the chunk prefix entry and chunk id
#     (12 B), the sub-block totals (16 x 8 B), the sub-block's 128 state
#     bytes and 128 risks (512 B); per agent exposed, its reference index,
#     state (claimed, then exposed), strain, timers, event tick and its
#     index (15 B).
#   k_sweep_rs (k_sweep_b) on RI ticks: 4 B per RI due index entry read; per visited
#     sub-block its state, chronically-missed flags, RI timers, reference
#     indexes and dates of birth (128 x 12 B) and the index write (4 B).
#   k_node_mix: per tick, the network entries of the sources with infected
#     agents (nodes x such sources x 16 B per simulation, two 8-byte
#     fixed-point parts per entry: entries of sources without infectivity
#     add nothing to the exact sums and are not read), the infectivity
#     totals (nodes x strains x 8 B) and, per chunk of the population, its
#     list entry, weight and prefix (20 B).
#   k_node_tx: per node its population inputs (last row, births, deaths:
#     12 B), seasonality, R0 scalar and row sum (24 B), per strain the
#     infectivity total and incoming infectivity (16 B x 3), susceptible
#     weight and count (12 B) read; population, per-strain probability
#     (4 + 8 x 3 B), count, target totals (24 B) and the selection record
#     (96 B) written: 248 B.
SWEEP_INDEX_B, SWEEP_DUE_B, SWEEP_EVT_B, SWEEP_DOD_B, QUEUE_ENTRY_B = 4.0, 128.0, 516.0, 516.0, 8.0
DUE_ITEM_B = 8.0
DSQ_ENTRY_B = 8.0 + 9.0 + 8.0
EVB_ENTRY_B = 8.0 + 10.0 + 5.0
SEL_TARGET_B = 12.0 + 128.0 + 128.0 + 512.0
SEL_CLAIM_B = 15.0
NODE_TX_CHUNK_B = 20.0
NODE_TX_NET_B = 16.0  # a network entry in its two fixed-point parts
NODE_TX_NODE_B = 248.0
RI_INDEX_B, RI_DUE_B = 4.0, 128.0 * 12.0 + 4.0


def merge_selection(prof):
    """The selection's two kernels (k_sel_round0, k_sel_rounds) as one
    entry, k_select, per tick."""
    out = {}
    for k, (ms, n) in prof.items():
        if k.startswith("k_sel_"):
            m0, n0 = out.get("k_select", (0.0, 0))
            out["k_select"] = (m0 + ms, max(n0, n))
        else:
            out[k] = (ms, n)
    return out


def kernel_alg_bytes(params, ticks, cnt, work, new_exposed, sources):
    """Algorithmic bytes of each modelled kernel over the ticks (total, all
    launches), from the work counters of the same ticks.  ``params``,
    ``cnt`` and ``sources`` (per tick, the nodes with infected agents: the
    results' I row > 0) may be lists (the simulations of one handle): the
    per-simulation terms are summed; the work counters are the handle's."""
    plist = params if isinstance(params, list) else [params]
    clist = cnt if isinstance(params, list) else [cnt]
    slist = sources if isinstance(params, list) else [sources]
    staged = sum(float(sum(sweep_b_bytes(p, t) * c[t] for t in ticks)) for p, c in zip(plist, clist))
    node_mix = sum(float(sum(p["n_nodes"] * (src[t] * NODE_TX_NET_B + p["n_strains"] * 8.0) for t in ticks))
                   + len(ticks) * NODE_TX_CHUNK_B * float(p["capacity"]) / 2048.0
                   for p, src in zip(plist, slist))
    out = {
        "k_due": SWEEP_INDEX_B * work["sweep_index"] + DUE_ITEM_B * work["sweep_due"],
        "k_sweep_a": (DUE_ITEM_B * work["sweep_due"] + SWEEP_DUE_B * work["sweep_due"]
                      + SWEEP_EVT_B * work["sweep_evt_due"] + SWEEP_DOD_B * work["sweep_dod_due"]
                      + (QUEUE_ENTRY_B + DSQ_ENTRY_B) * work["queue_ds"]),
        "k_sweep_b": staged + RI_INDEX_B * work["ri_index"] + RI_DUE_B * work["ri_due"]
                     + QUEUE_ENTRY_B * work["queue_rs"],
        "k_evb": EVB_ENTRY_B * work["queue_rs"],
        "k_select": SEL_TARGET_B * work["sel_targets"] + SEL_CLAIM_B * float(new_exposed),
        "k_node_mix": node_mix,
        "k_node_tx": sum(len(ticks) * p["n_nodes"] * NODE_TX_NODE_B for p in plist),
    }
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_ready(self, timeout=10.0):
        """Block until nvidia-smi has printed its first sample: its start-up
        takes driver locks that would otherwise land inside a timed region."""
        t0 = time.perf_counter()
        while self.proc is not None and not self.lines and time.perf_counter() - t0 < timeout:
            time.sleep(0.02)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[3:7], strict=False):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def counts_per_tick(params, births):
    """cnt[t] = people.count after tick t's births: the slots tick t scans."""
    per_tick_births = births.sum(axis=1).astype(np.int64)
    return params["count"] + np.cumsum(per_tick_births)


def warm_up_api(args, dev):
    """One small run through the same calls (create, bind, start, a few
    ticks, reads, destroy) before a timed end-to-end region: the process's
    one-time costs (loading the library's kernels on first launch, the
    allocator's first mappings) are not the workload's."""
    from laser_polio_gb300 import synthetic
    from laser_polio_gb300._lib import Handle
    from laser_polio_gb300.engine import make_desc

    p, c = synthetic.bundle("nigeria", n_agents=200_000, n_nodes=args.nodes, seed=args.seed + 1000)
    d, keep = make_desc(p)
    h = Handle([d], device=dev)
    try:
        h.bind_columns(0, c)
        h.start()
        h.step(16)
        h.sync()
        h.read_results(0, result_arrays(p))
        h.read_columns(0, {k: np.empty_like(v) for k, v in c.items()})
    finally:
        h.close()


def make_bundle(args, rank, pinned):
    from laser_polio_gb300 import synthetic

    alloc = None
    if pinned:
        import torch

        def alloc(name, n, dtype):
            t = torch.empty(n, dtype=getattr(torch, np.dtype(dtype).name), pin_memory=True)
            return t.numpy()

    return synthetic.bundle("nigeria", n_agents=int(args.agents), n_nodes=args.nodes, seed=args.seed + rank, alloc=alloc)


def pinned_empty(shape, dtype):
    """A numpy array over page-locked host memory (torch's pinned allocator)."""
    import torch

    n = int(np.prod(shape))
    t = torch.empty(n, dtype=getattr(torch, np.dtype(dtype).name), pin_memory=True)
    return t.numpy().reshape(shape)


def result_arrays(params, pinned=False):
    from laser_polio_gb300 import _abi

    nt, n, ns = params["nt"], params["n_nodes"], params["n_strains"]
    out = {}
    for name, wide in _abi.RESULT_FIELDS:
        shape = (nt, n, ns) if wide else (nt, n)
        if pinned:
            a = pinned_empty(shape, np.int32)
            a.fill(0)
        else:
            a = np.zeros(shape, np.int32)
        out[name] = a
    return out


def workload_config(params, W, K, ws=1):
    """The `config` of both arms' lines: the same workload and the same ticks."""
    return {"workload": f"nigeria_like {params['n_nodes']} nodes x {params['count']:.3g} agents, capacity +30%, "
                        f"ticks {W + 1}-{W + K} of a {params['nt'] - 1}-tick run",
            "agents": params["count"], "capacity": params["capacity"], "nodes": params["n_nodes"],
            "l2": "state columns larger than L2 (no flush needed)", "replicas": ws}


def oracle_leg(params, cols, warmup, steps, seconds=None):
    """The oracle (C/OpenMP restatement of the reference's loops) over ticks
    1 .. warmup+steps of the same population: `warmup` untimed ticks, then up
    to `steps` timed ticks (fewer only when `seconds` runs out).  Returns the
    timing and the open OracleSim for the parity comparison."""
    from laser_polio_gb300.engine import make_desc
    from oracle.oracle import OracleSim
    from oracle.oracle import num_threads

    d, keep = make_desc(params)
    o = OracleSim(d, keepalive=keep)
    o.bind_columns(cols)
    o.start()
    o.step(warmup)
    done, agent_ticks = 0, 0
    t0 = time.perf_counter()
    while done < steps:
        o.step(1)
        done += 1
        agent_ticks += o.state().count
        if seconds is not None and time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": agent_ticks / dt, "ticks": done, "seconds": dt, "cores": num_threads(), "warmup": warmup,
            "oracle": o, "keep": keep}


def compare_with_oracle(o, res_gpu, read_gpu_column, params, count):
    """Every result array and every agent column of the GPU run against the
    oracle's after the same ticks; columns one at a time through a reusable
    buffer (the oracle keeps its own copy of the table)."""
    from laser_polio_gb300 import _abi

    mismatch = []
    res_o = result_arrays(params)
    o.read_results(res_o)
    for name, a in res_o.items():
        if not np.array_equal(a, res_gpu[name]):
            mismatch.append(f"result {name}: {int((a != res_gpu[name]).sum())} entries")
    n_cols = 0
    for name, _, dtype in _abi.COLUMN_FIELDS:
        buf = np.empty(count, dtype=dtype)
        o.read_columns({name: buf})
        gpu = read_gpu_column(name, dtype)
        n_cols += 1
        if not np.array_equal(buf, gpu[:count]):
            mismatch.append(f"column {name}: {int((buf != gpu[:count]).sum())} slots")
    return {"bit_exact": not mismatch, "results_compared": len(res_o), "columns_compared": n_cols,
            "slots_compared": int(count), "mismatches": mismatch[:8]}


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    params, cols = make_bundle(args, 0, pinned=False)
    W, K = args.warmup, args.steps
    if W + K > params["nt"] - 1:
        K = max(1, params["nt"] - 1 - W)
    cpu = oracle_leg(params, cols, W, K, args.cpu_seconds)
    cpu["oracle"].close()
    sample = (f"ticks {W + 1}-{W + cpu['ticks']} after {W} untimed of the {params['count']:.3g}-agent, "
              f"{params['n_nodes']}-node population ({cpu['seconds']:.1f} s)")
    line = {
        "impl": "reference",
        "metric": "agent-ticks/s (774 nodes, 2.2e8 agents, full agent step)",
        "value": cpu["value"],
        "unit": "agent-ticks/s",
        "n_gpus": ws,
        "steps": cpu["ticks"],
        "warmup": W,
        "ms_per_step": cpu["seconds"] / max(1, cpu["ticks"]) * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int8/int32 state, f64 node FOI",
        "data": "synthetic (seeded numpy, Nigeria-scale shapes)",
        "config": workload_config(params, W, K, ws),
        "cpu_baseline": {"value": cpu["value"], "unit": "agent-ticks/s", "cores": cpu["cores"], "kind": "port",
                         "sample": sample},
        "e2e": {"value": cpu["value"], "unit": "agent-ticks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def api_run(args, dev):
    """The user's whole path at the Nigeria scale: SEIR_ABM(pars) and the
    five components (the agent table initialised on the device), then run()
    over all 2555 ticks with results landing in sim.results; wall time of
    each phase, with the device synchronised at the end of each."""
    import torch

    import laser_polio_gb300 as lp
    from laser_polio_gb300 import synthetic

    pars, immun, rng = synthetic.nigeria_like_pars(n_agents=int(args.agents), n_nodes=args.nodes, seed=args.seed)
    prev = np.zeros(args.nodes, np.int64)
    prev[rng.choice(args.nodes, size=2, replace=False)] = 10
    pars.update({"init_immun": list(np.asarray(immun, float)), "init_prev": list(prev), "age_pyramid_path": None})
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim = lp.SEIR_ABM(lp.PropertySet(pars))
    sim.components = [lp.VitalDynamics_ABM, lp.DiseaseState_ABM, lp.RI_ABM, lp.SIA_ABM, lp.Transmission_ABM]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    sim.run()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    births = sim.results.births.sum(axis=1).astype(np.int64)
    cnt = int(np.sum(pars["init_pop"])) + np.cumsum(births)
    at = float(cnt[1 : sim.t].sum())
    out = {"value": at / (t2 - t0), "unit": "agent-ticks/s", "ticks": int(sim.t) - 1, "agents": int(cnt[0]),
           "capacity": int(sim.people.capacity), "seconds": t2 - t0,
           "phases_s": {"construct": t1 - t0, "run": t2 - t1},
           "path": "SEIR_ABM(pars); sim.components = [...]; sim.run(): agent table initialised on the device, "
                   "results copied to sim.results, columns left on the device",
           "new_exposed_total": int(sim.results.new_exposed.sum())}
    if sim._engine is not None:
        sim._engine.close()
    del sim
    return out


def continental_sim(args):
    """SEIR_ABM of the continental workload with the five components (agent
    table initialised on the device), its agent and node counts."""
    import laser_polio_gb300 as lp
    from laser_polio_gb300 import synthetic

    agents, nodes = int(args.agents), int(args.nodes)
    pars, immun, rng = synthetic.continental_pars(n_agents=agents, n_nodes=nodes, dur=365, seed=args.seed)
    prev = np.zeros(nodes, np.int64)
    prev[rng.choice(nodes, size=2, replace=False)] = 10
    pars.update({"init_immun": list(np.asarray(immun, float)), "init_prev": list(prev), "age_pyramid_path": None})
    sim = lp.SEIR_ABM(lp.PropertySet(pars))
    sim.components = [lp.VitalDynamics_ABM, lp.DiseaseState_ABM, lp.RI_ABM, lp.SIA_ABM, lp.Transmission_ABM]
    return sim, agents, nodes


def desc_params(desc):
    """The fields of a simulation description the byte model reads."""
    return {"n_nodes": desc.n_nodes, "n_strains": desc.n_strains, "capacity": desc.capacity,
            "vd_step": desc.vd_step, "ri_enabled": desc.ri_enabled, "ri_step": desc.ri_step,
            "sia": [(desc.sia[i].tick,) for i in range(desc.n_sia)]}


def continental_arm(args):
    """The continental workload through the user's path: 4000 nodes, 1e9
    agents (capacity as the reference sizes it for the births of the run),
    node populations lognormal(ln 2.5e5, 0.9), dense gravity network over a
    5000 km square, RI and SIA as the Nigeria-scale workload, 365 ticks.
    SEIR_ABM(pars) with the five components (agent table initialised on the
    device), then the steps of run(): start (bind and layout), W untimed
    ticks, the remaining ticks between CUDA events on the engine's stream,
    results and columns copied into the sim.  value: agent-ticks/s of the
    timed ticks; e2e: all ticks over the wall time of construction, start,
    ticks and copy-back.  A second run of the same sim in profiling mode
    gives each kernel's share of the whole run and the top kernel's
    algorithmic bytes against the measured HBM peak."""
    import torch

    from laser_polio_gb300.model import _engine_of

    W = max(3, args.warmup)
    free0 = torch.cuda.mem_get_info()[0]
    with ClockSampler(0) as clocks:
        clocks.wait_ready()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim, agents, nodes = continental_sim(args)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        eng = _engine_of(sim)
        eng._ensure_started()
        h = eng.handle
        h.sync()
        t2 = time.perf_counter()
        used = free0 - torch.cuda.mem_get_info()[0]
        stream = torch.cuda.ExternalStream(h.cuda_stream())
        h.step(W)
        h.sync()
        n_rest = sim.nt - 1 - W
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = h.kernel_launches()
        t3 = time.perf_counter()
        e0.record(stream)
        h.step(n_rest)
        e1.record(stream)
        h.sync()
        t4 = time.perf_counter()
        launches = h.kernel_launches() - l0
        ms = e0.elapsed_time(e1)
        st = h.state(0)
        sim.t, sim.should_stop = st.t, bool(st.stopped)
        eng._finish()
        torch.cuda.synchronize()
        t5 = time.perf_counter()
    births = sim.results.births.sum(axis=1).astype(np.int64)
    cnt = int(eng.spec.desc.count) + np.cumsum(births)
    at_timed = float(cnt[W + 1 : W + 1 + n_rest].sum())
    at_all = float(cnt[1 : sim.nt].sum())
    new_exposed = int(sim.results.new_exposed.sum())
    capacity = int(sim.people.capacity)
    eng.close()
    del sim, eng
    torch.cuda.empty_cache()

    # profiling pass: the same run again, every kernel timed with events
    sim, _, _ = continental_sim(args)
    eng = _engine_of(sim)
    eng._ensure_started()
    h = eng.handle
    h.set_profiling(True)
    h.step(sim.nt - 1)
    h.sync()
    prof = merge_selection(h.profile())
    work = h.counters()
    res = result_arrays(desc_params(eng.spec.desc) | {"nt": sim.nt})
    h.read_results(0, res)
    params = desc_params(eng.spec.desc)
    eng.close()
    del sim, eng
    torch.cuda.empty_cache()
    ticks = np.arange(1, len(cnt))
    ne = int(res["new_exposed"][ticks].sum() - res["ri_protected"][ticks].sum() - res["sia_protected"][ticks].sum())
    alg = kernel_alg_bytes(params, ticks, cnt, work, ne, (res["I"] > 0).sum(axis=1))
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    tot = sum(v[0] for v in prof.values()) or 1.0
    kernels = {}
    for k, (k_ms, n) in prof.items():
        if not n:
            continue
        row = {"ms_per_launch": k_ms / n, "launches": n, "share": k_ms / tot}
        if k in alg and k_ms > 0:
            row["alg_bytes_per_launch"] = alg[k] / n
            row["achieved_gbs"] = alg[k] / (k_ms / 1e3) / 1e9
            row["frac"] = row["achieved_gbs"] / peak
        kernels[k] = row
    top = max(prof, key=lambda k: prof[k][0])
    roof = {"kernel": top, "bound": "hbm", "achieved": kernels[top].get("achieved_gbs"), "peak": peak,
            "unit": "GB/s", "frac": kernels[top].get("frac"), "traffic": None,
            "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
            "alg_bytes_per_launch": kernels[top].get("alg_bytes_per_launch"),
            "mean_launch_ms": kernels[top]["ms_per_launch"], "share_of_run": kernels[top]["share"],
            "work": work, "kernels": kernels,
            "window": "every tick of the run (profiling pass: events around every kernel)"}
    line = {
        "metric": f"agent-ticks/s ({nodes} nodes, {agents:.2g} agents, full agent step)",
        "value": at_timed / (ms / 1e3), "unit": "agent-ticks/s", "n_gpus": 1, "steps": n_rest, "warmup": W,
        "ms_per_step": ms / n_rest, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int8/int32 state, f64 node FOI",
        "data": "synthetic (seeded, the continental workload's distributions; agent table drawn on the device)",
        "config": {"workload": f"continental {nodes} nodes x {agents:.2g} agents, capacity {capacity:.3g}, "
                               f"ticks {W + 1}-{len(cnt) - 1} of a {len(cnt) - 1}-tick run",
                   "l2": "state columns far larger than L2 (no flush needed)"},
        "e2e": {"value": at_all / (t5 - t0), "unit": "agent-ticks/s", "ticks": len(cnt) - 1, "seconds": t5 - t0,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "phases_s": {"construct": t1 - t0, "start": t2 - t1, "untimed_ticks": t3 - t2,
                             "ticks": t4 - t3, "copy_back": t5 - t4},
                "path": "SEIR_ABM(pars); sim.components = [...]; the steps of run(), results and columns "
                        "into the sim on the device"},
        "roofline": roof,
        "device_bytes_after_start": used,
        "gpu_launches": launches,
        "new_exposed_total": new_exposed,
        "clocks": clocks.summary(),
    }
    if args.continental_reps > 1:
        line["replicates"] = continental_replicates(agents, nodes, args.continental_reps, args.seed, W)
    print(json.dumps(line), flush=True)
    if args.out:
        Path(args.out).write_text(json.dumps(line, indent=1))


def continental_replicates(agents, nodes, reps, seed, W):
    """R parameter sets over one continental agent table in one handle: the
    table (agents / R agents, the continental node layout, 365 ticks) is
    drawn once and bound R times, each replicate with its own R0 (every
    agent's infectivity scaled), seasonal amplitude and peak, gravity k and
    seed.  The configuration's R x 1e9 agents would need R x 68 GB of engine
    state (52 B per capacity slot) and do not fit in one GPU's memory, so the
    table is 1e9 / R agents and the batch 1e9 in all.  All ticks after W are
    timed between CUDA events, batched and then the replicates one after
    another."""
    import torch

    from laser_polio_gb300 import synthetic
    from laser_polio_gb300._lib import Handle
    from laser_polio_gb300.core import gravity, row_normalizer
    from laser_polio_gb300.engine import make_desc
    from laser_polio_gb300.utils import seasonality_table
    import datetime

    t0 = time.perf_counter()
    p0, cols = synthetic.bundle("continental", n_agents=agents // reps, n_nodes=nodes, dur=365, seed=seed)
    t_gen = time.perf_counter() - t0
    pops, dist, nt = p0["pop0"].astype(np.float64), p0["distances"], p0["nt"]
    dates = [datetime.date(2019, 1, 1) + datetime.timedelta(days=d) for d in range(nt)]
    sets = [(1.0, 0.4, 180, 0.5), (0.8, 0.3, 150, 0.3), (1.2, 0.5, 210, 0.8), (1.1, 0.2, 120, 0.6)]
    rng = np.random.default_rng(seed + 7)
    runs = []
    for r in range(reps):
        scale, amp, peak, k = sets[r % len(sets)]
        p = dict(p0, seed=seed + r, seasonality=seasonality_table(dates, amp, peak),
                 r0_scalars=p0["r0_scalars"] * rng.lognormal(0.0, 0.1, nodes),
                 network=row_normalizer(gravity(pops, dist, k, 1, 1, 2.0) / np.power(pops.sum(), 2.0), 0.2))
        c = cols if scale == 1.0 else dict(cols, daily_infectivity=(cols["daily_infectivity"] * np.float32(scale))
                                                                  .astype(np.float32))
        runs.append((p, c, make_desc(p)))

    def run(idx):
        h = Handle([runs[i][2][0] for i in idx])
        try:
            for j, i in enumerate(idx):
                h.bind_columns(j, runs[i][1])
            h.start()
            h.step(W)
            h.sync()
            stream = torch.cuda.ExternalStream(h.cuda_stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            h.step(nt - 1 - W)
            e1.record(stream)
            h.sync()
            ms = e0.elapsed_time(e1)
            at, ne = 0.0, 0
            for j, i in enumerate(idx):
                res = result_arrays(runs[i][0])
                h.read_results(j, res)
                at += float(counts_per_tick(runs[i][0], res["births"])[W + 1 : nt].sum())
                ne += int(res["new_exposed"].sum())
        finally:
            h.close()
        return ms, at, ne

    ms_b, at_b, ne_b = run(list(range(reps)))
    ms_s, at_s = 0.0, 0.0
    for i in range(reps):
        ms, at, _ = run([i])
        ms_s += ms
        at_s += at
    assert at_s == at_b
    return {"value": at_b / (ms_b / 1e3), "unit": "agent-ticks/s", "replicates": reps,
            "agents_each": int(p0["count"]), "agents": int(p0["count"]) * reps, "nodes_each": nodes,
            "ticks": f"{W + 1}-{nt - 1} of {nt - 1}", "ms_per_step": ms_b / (nt - 1 - W),
            "sequential": {"value": at_s / (ms_s / 1e3), "ms_total": ms_s}, "batched_ms_total": ms_b,
            "speedup_vs_sequential": ms_s / ms_b, "generation_s": t_gen, "new_exposed_total": ne_b,
            "parameter_sets": "(R0 scale, amp, peak, k) in " + str(sets[:reps]) + "; r0 scalars x lognormal(0, 0.1)"}


def tick_kind(params, t):
    """plain / vd / vd+ri / sia ... : the components that act on tick t
    besides the every-tick ones."""
    parts = []
    if t % params["vd_step"] == 0:
        parts.append("vd")
    if params["ri_enabled"] and t % params["ri_step"] == 0:
        parts.append("ri")
    if any(e[0] == t for e in params["sia"]):
        parts.append("sia")
    return "+".join(parts) or "plain"


def full_run(desc, cols, params, dev):
    """The whole run on the device: once replayed as the engine runs it
    (graphs of 8 ticks), timed between CUDA events on its stream; once tick by
    tick with an event pair per tick, for the mean time of each kind of tick.
    Returns (line entry, the handle's end-of-run results)."""
    import torch

    from laser_polio_gb300._lib import Handle

    n = params["nt"] - 1
    h = Handle([desc], device=dev)
    h.bind_columns(0, cols)
    h.start()
    h.sync()
    stream = torch.cuda.ExternalStream(h.cuda_stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    h.step(n)
    e1.record(stream)
    h.sync()
    ms_all = e0.elapsed_time(e1)
    res = result_arrays(params)
    h.read_results(0, res)
    h.close()
    cnt = counts_per_tick(params, res["births"])
    at = float(cnt[1 : n + 1].sum())

    h = Handle([desc], device=dev)
    h.bind_columns(0, cols)
    h.start()
    h.sync()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
    evs[0].record(stream := torch.cuda.ExternalStream(h.cuda_stream()))
    for t in range(1, n + 1):
        h.step(1)
        evs[t].record(stream)
    h.sync()
    per_tick = np.array([evs[t - 1].elapsed_time(evs[t]) for t in range(1, n + 1)])
    h.close()
    kinds = {}
    for t in range(1, n + 1):
        k = tick_kind(params, t)
        us, c = kinds.get(k, (0.0, 0))
        kinds[k] = (us + per_tick[t - 1] * 1e3, c + 1)
    by_kind = {k: {"ticks": c, "us_per_tick": us / c, "share": us / (per_tick.sum() * 1e3)}
               for k, (us, c) in sorted(kinds.items(), key=lambda kv: -kv[1][1])}
    return {"ticks": n, "value": at / (ms_all / 1e3), "unit": "agent-ticks/s", "ms_total": ms_all,
            "ms_per_tick": ms_all / n, "new_exposed_total": int(res["new_exposed"].sum()),
            "by_tick_kind": by_kind,
            "by_tick_kind_note": "one tick per launch sequence with an event pair per tick (no graphs), so the "
                                 "per-kind sum exceeds the replayed total"}


def batch_measure(n_reps, seed, W, K, profile=True):
    """R calibration replicates (node counts from {14, 44, 120, 300}, 1e6-2e7
    agents each, per-replicate R0 / seasonality / gravity k, 730 ticks): the
    same ticks timed once with all replicates in one handle (one launch
    sequence per tick) and once as R plain runs one after another.  Both
    time only the device ticks (CUDA events on the handle's stream).  A
    profiling pass of the batch gives the kernels' shares and the dominant
    kernel's modelled roofline."""
    import torch

    from laser_polio_gb300 import synthetic
    from laser_polio_gb300._lib import Handle
    from laser_polio_gb300.engine import make_desc

    t_gen = time.perf_counter()
    specs = synthetic.replicate_specs(n_reps, seed=seed, dur=730)
    bundles = [synthetic.bundle(**sp) for sp in specs]
    t_gen = time.perf_counter() - t_gen
    descs = [make_desc(p) for p, _ in bundles]
    nt = bundles[0][0]["nt"]
    K = max(1, min(K, nt - 1 - W))

    def run(idx, profiling=False):
        h = Handle([descs[i][0] for i in idx])
        for j, i in enumerate(idx):
            h.bind_columns(j, bundles[i][1])
        h.start()
        h.step(W)
        h.sync()
        if profiling:
            h.set_profiling(True)
        stream = torch.cuda.ExternalStream(h.cuda_stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        l0 = h.kernel_launches()
        e0.record(stream)
        h.step(K)
        e1.record(stream)
        h.sync()
        ms = e0.elapsed_time(e1)
        launches = h.kernel_launches() - l0
        at, cnts, ne, srcs = 0.0, [], 0, []
        for j, i in enumerate(idx):
            res = result_arrays(bundles[i][0])
            h.read_results(j, res)
            cnt = counts_per_tick(bundles[i][0], res["births"])
            cnts.append(cnt)
            srcs.append((res["I"] > 0).sum(axis=1))
            at += float(cnt[W + 1 : W + K + 1].sum())
            tk = slice(W + 1, W + K + 1)
            ne += int(res["new_exposed"][tk].sum() - res["ri_protected"][tk].sum() - res["sia_protected"][tk].sum())
        prof = merge_selection(h.profile()) if profiling else None
        work = h.counters() if profiling else None
        h.close()
        return ms, at, launches, prof, work, cnts, ne, srcs

    ms_b, at_b, launches_b = run(list(range(len(bundles))))[:3]
    ms_s, at_s = 0.0, 0.0
    for i in range(len(bundles)):
        ms, at = run([i])[:2]
        ms_s += ms
        at_s += at
    assert at_s == at_b
    out = {
        "value": at_b / (ms_b / 1e3), "unit": "agent-ticks/s", "replicates": len(bundles),
        "agents": int(sum(p["count"] for p, _ in bundles)), "nodes": [p["n_nodes"] for p, _ in bundles],
        "ticks": f"{W + 1}-{W + K} of 730", "ms_per_step": ms_b / K, "gpu_launches_per_tick": launches_b / K,
        "sequential": {"value": at_s / (ms_s / 1e3), "ms_total": ms_s},
        "batched_ms_total": ms_b, "speedup_vs_sequential": ms_s / ms_b, "generation_s": t_gen,
    }
    if profile:
        _, _, _, prof, work, cnts, ne, srcs = run(list(range(len(bundles))), profiling=True)
        ticks = np.arange(W + 1, W + K + 1)
        alg = kernel_alg_bytes([p for p, _ in bundles], ticks, cnts, work, ne, srcs)
        tot = sum(v[0] for v in prof.values())
        top = max(prof, key=lambda k: prof[k][0])
        t_ms, t_n = prof[top]
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        peak = float(peaks.get("hbm_gbs", 6800.0))
        ach = alg[top] / (t_ms / 1e3) / 1e9 if top in alg and t_ms > 0 else None
        out["kernels"] = {k: {"ms_per_launch": v[0] / max(1, v[1]), "share": v[0] / tot} for k, v in prof.items()}
        out["roofline"] = {"kernel": top, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                           "frac": ach / peak if ach is not None else None,
                           "alg_bytes_per_launch": alg.get(top, 0.0) / max(1, t_n),
                           "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}
    return out


def batch_arm(args):
    """The batch measurement alone, as its own line (see batch_measure)."""
    with ClockSampler(0) as clocks:
        clocks.wait_ready()
        b = batch_measure(args.batch, args.seed, args.warmup, args.steps)
    line = {
        "metric": f"agent-ticks/s, {b['replicates']}-replicate calibration batch",
        "value": b["value"], "unit": "agent-ticks/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": b["ms_per_step"], "higher_is_better": True,
        "data": "synthetic (seeded numpy, calibration-batch shapes)",
        "config": {"workload": f"{b['replicates']} replicates, nodes in {{14, 44, 120, 300}}, "
                               f"{b['agents']:.3g} agents in total, ticks {b['ticks']}"},
        "batch": b, "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    if args.out:
        Path(args.out).write_text(json.dumps(line, indent=1))


def replay_inputs(args, T, dev):
    """The expected-incidence map's inputs recorded by forward runs of the
    engine at the Nigeria scale (args.agents agents, args.nodes nodes,
    T ticks, births, RI and SIA on): one handle, two simulations of the same
    agent table.  Simulation 0 runs at the base parameters (R0 14, seasonal
    amplitude 0.4 peaking on day 180, gravity k 0.5) and records srisk,
    beta and pop per transmission tick and node (lpg_record_aggregates):
    these are the replayed aggregates.  Simulation 1 runs at perturbed
    parameters (every agent's infectivity x1.1, amplitude 0.35, peak day 170,
    k 0.6, r0 scalars x lognormal(0, 0.05)); its recorded expected exposures
    are the target curve.  Returns (map inputs at the base parameters,
    target [T, nodes], record of the runs), the record holding the largest
    difference between the map's lam on simulation 0's aggregates and the
    engine's own expected exposures, relative to the largest."""
    import datetime
    import torch

    from laser_polio_gb300 import ops, synthetic
    from laser_polio_gb300._lib import Handle
    from laser_polio_gb300.core import gravity, row_normalizer
    from laser_polio_gb300.engine import make_desc
    from laser_polio_gb300.utils import seasonality_table

    t0 = time.perf_counter()
    pa, cols = synthetic.bundle("nigeria", n_agents=int(args.agents), n_nodes=args.nodes, dur=T, seed=args.seed)
    G, ns, nt = pa["n_nodes"], pa["n_strains"], pa["nt"]
    pops, dist = pa["pop0"].astype(np.float64), pa["distances"]
    rng = np.random.default_rng(args.seed + 1)
    dates = [datetime.date(2019, 1, 1) + datetime.timedelta(days=d) for d in range(nt)]
    pb = dict(pa, seasonality=seasonality_table(dates, 0.35, 170),
              r0_scalars=pa["r0_scalars"] * rng.lognormal(0.0, 0.05, G),
              network=row_normalizer(gravity(pops, dist, 0.6, 1, 1, 2.0) / np.power(pops.sum(), 2.0), 0.2))
    cols_b = dict(cols, daily_infectivity=(cols["daily_infectivity"] * np.float32(1.1)).astype(np.float32))
    da, ka = make_desc(pa)
    db, kb = make_desc(pb)
    t_gen = time.perf_counter() - t0
    h = Handle([da, db], device=dev)
    try:
        h.record_aggregates(0)
        h.record_aggregates(1)
        h.bind_columns(0, cols)
        h.bind_columns(1, cols_b)
        h.start()
        h.sync()
        stream = torch.cuda.ExternalStream(h.cuda_stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.step(nt - 1)
        e1.record(stream)
        assert h.sync_statuses() == [0, 0]
        ms = e0.elapsed_time(e1)
        agg = h.read_aggregates(0, nt, G, ns)
        tgt = h.read_aggregates(1, nt, G, ns)["lam"]
    finally:
        h.close()
    del cols, cols_b
    ticks = slice(1, nt)  # no component runs on tick 0
    doy = np.array([d.timetuple().tm_yday for d in dates], np.float64)
    year = np.array([366.0 if (d.year % 4 == 0 and (d.year % 100 != 0 or d.year % 400 == 0)) else 365.0
                     for d in dates])
    inp = dict(srisk=agg["srisk"][ticks], beta=agg["beta"][ticks], pop=agg["pop"][ticks], doy=doy[ticks],
               year=year[ticks], r0s=pa["r0_scalars"], R=1.0, amp=0.4, peak=180.0, pops=pops, dist=dist,
               k=0.5, a=1.0, b=1.0, c=2.0, max_frac=0.2)
    lam, _ = ops.expected_incidence(inp)
    eng = agg["lam"][ticks]
    rec = {"source": "recorded by the engine's forward runs (lpg_record_aggregates)",
           "agents": int(pa["count"]), "nodes": G, "ticks": nt - 1, "simulations": 2,
           "forward_ms": ms, "generate_s": t_gen,
           "new_exposed_expected": float(eng.sum()), "target_expected": float(tgt[ticks].sum()),
           "map_vs_engine_max_rel": float(np.max(np.abs(lam - eng)) / max(np.max(np.abs(eng)), 1e-300))}
    return inp, tgt[ticks].copy(), rec


def incidence_arm(args):
    """Loss and gradient of the expected incidence over T ticks of replayed
    Nigeria-scale aggregates (774 nodes, 3 strains), against a target curve
    from perturbed parameters: L = sum (log1p(lam) - log1p(target))^2 and its
    gradient with respect to R, amp, peak, r0s and k, a, b, c.  With
    --incidence-data replay (the default) the aggregates and the target are
    recorded by forward runs of the engine (replay_inputs); with synthetic,
    seeded numpy aggregates of the same shapes stand in and the target is the
    map at perturbed parameters.  One step = one
    evaluation on a resident plan (lpg_incidence_plan_eval: parameters up,
    loss and gradients down).  value: K evaluations between CUDA events on
    the plan's stream.  e2e: wall time from host arrays, the plan's one-time
    upload of the aggregates and target included, over the same K
    evaluations.  roofline: the slower product's FP32 instructions over its
    mean launch time (profiling pass) against the nominal FP32 issue rate."""
    import torch

    from laser_polio_gb300 import ops, synthetic

    T = args.incidence
    replay = None
    if args.incidence_data == "replay" and not args.continental:
        inp, target, replay = replay_inputs(args, T, 0)
        G, S = inp["r0s"].shape[0], inp["beta"].shape[2]
    elif args.continental:
        # the continental shapes: two recording runs of 1.3e9-slot tables would hold
        # their host columns twice over, so seeded aggregates of those shapes stand in
        inp = synthetic.incidence_inputs(T=T, n_nodes=args.nodes, n_agents=args.agents, seed=args.seed,
                                         mu=np.log(2.5e5), sigma=0.9, side_km=5000.0)
        G, S = inp["r0s"].shape[0], inp["beta"].shape[2]
        rng = np.random.default_rng(args.seed + 1)
        pert = dict(inp, R=1.1, amp=0.35, peak=170.0, k=0.6, r0s=inp["r0s"] * rng.lognormal(0.0, 0.05, G))
        target, _ = ops.expected_incidence(pert)
    else:
        inp = synthetic.incidence_inputs(T=T, n_nodes=args.nodes, seed=args.seed)
        G, S = inp["r0s"].shape[0], inp["beta"].shape[2]
        rng = np.random.default_rng(args.seed + 1)
        pert = dict(inp, R=1.1, amp=0.35, peak=170.0, k=0.6, r0s=inp["r0s"] * rng.lognormal(0.0, 0.05, G))
        target, _ = ops.expected_incidence(pert)
    W, K = max(3, args.warmup), max(1, min(args.steps, 200))
    torch.cuda.synchronize()
    with ClockSampler(0) as clocks:
        clocks.wait_ready()
        t0 = time.perf_counter()
        plan = ops.IncidencePlan(inp, target)
        t_setup = time.perf_counter() - t0
        for _ in range(W):
            plan.evaluate(inp, network_grad=False)
        stream = torch.cuda.ExternalStream(plan.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e0.record(stream)
        for _ in range(K):
            res = plan.evaluate(inp, network_grad=False)
        e1.record(stream)
        torch.cuda.synchronize()
        t_eval = time.perf_counter() - t1
        dev_ms = e0.elapsed_time(e1) / K
    plan.set_profiling(True)
    for _ in range(K):
        plan.evaluate(inp, network_grad=False)
    prof = plan.profile()
    plan.close()
    tot = sum(ms for ms, _ in prof.values())
    kernels = {name: {"launches": n, "ms_per_eval": ms / K, "share": ms / tot if tot else None}
               for name, (ms, n) in prof.items()}
    # the products run in double-float on the FP32 pipe: 12 FP32 instructions per term
    # (Dekker product by FMA, two cross terms, Knuth TwoSum), T S G G terms per launch
    terms = float(T * S * G * G)
    top = max(prof, key=lambda n: prof[n][0])
    gemm = max(("k_inc_gemm_mix", "k_inc_gemm_flows"), key=lambda n: prof[n][0])
    ms_g = prof[gemm][0] / max(1, prof[gemm][1])
    fp32_peak = 152 * 128 * 2.07e9 / 1e12  # lane-instructions/s at the maximum SM clock (nominal)
    ach = 12.0 * terms / (ms_g / 1e3) / 1e12
    roof = {"kernel": gemm, "top_kernel": top, "bound": "fp32", "achieved": ach, "peak": fp32_peak,
            "unit": "T FP32 lane-instructions/s", "frac": ach / fp32_peak,
            "peak_kind": "nominal GB300 FP32 issue rate, 152 SMs x 128 lanes x 2.07 GHz (not measured)",
            "fp64_equivalent_tflops": 2.0 * terms / (ms_g / 1e3) / 1e12, "traffic": None,
            "instructions_per_launch": 12.0 * terms}
    h2d_setup = sum(inp[k].nbytes for k in ("srisk", "beta", "pop", "doy", "year", "pops", "dist")) + target.nbytes
    cpu = None
    if not args.no_cpu:
        from oracle import incidence as oracle_incidence

        n_cpu, t0 = 0, time.perf_counter()
        while n_cpu < 50 and (n_cpu == 0 or time.perf_counter() - t0 < 10.0):
            lam, _ = oracle_incidence.incidence(inp)
            resid = np.log1p(lam) - np.log1p(target)
            oracle_incidence.incidence(inp, 2.0 * resid / (1.0 + lam))
            n_cpu += 1
        cpu_s = (time.perf_counter() - t0) / n_cpu
        cpu = {"value": 1.0 / cpu_s, "unit": "evaluations/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n_cpu} loss and gradient evaluations, T={T}, numpy FP64 restatement "
                         "(products through BLAS on the host's threads)"}
    line = {
        "metric": "expected-incidence loss and gradient evaluations/s",
        "value": 1e3 / dev_ms,
        "unit": "evaluations/s",
        "n_gpus": 1,
        "steps": K,
        "warmup": W,
        "ms_per_step": dev_ms,
        "higher_is_better": True,
        "dtype": "f64",
        "data": ("synthetic agents (seeded numpy, Nigeria-scale shapes); aggregates and target recorded by "
                 "forward runs of the engine" if replay else "synthetic (seeded numpy, replayed-aggregate shapes)"),
        "config": {"workload": f"adjoint of expected incidence, {G} nodes, {T} ticks, {S} strains",
                   "loss": "sum (log1p(lam) - log1p(target))^2",
                   "l2": "working set (~40 MB) L2-resident by design; no flush"},
        "e2e": {"value": K / (t_setup + t_eval), "unit": "evaluations/s", "setup_ms": t_setup * 1e3,
                "ms_per_eval": t_eval / K * 1e3, "h2d_bytes_per_step": h2d_setup / K + 8 * G,
                "d2h_bytes_per_step": 8 * (8 + G)},
        "gpu_launches": 7 * K,  # per evaluation: network, mix, forward, backward + seasonal, flows, network_grad
        "kernels": kernels,
        "roofline": roof,
        "cpu_baseline": cpu,
        "loss": res["loss"],
        "grad": {k: res["grad"][k] for k in ("R", "amp", "peak", "k", "a", "b", "c")},
        "replay": replay,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    if args.out:
        Path(args.out).write_text(json.dumps(line, indent=1))


def export_arm(args):
    """save_sim_results' CSV (utils.py:689-786) of a 2556-tick x 774-node
    results table (1.98e6 rows, seeded synthetic counts): the native writer
    (lpg_write_results_csv, host threads) against a restatement of the same
    file with Python's csv module (the reference writes it with pandas, which
    is absent here).  Host only; rows/s over K writes after W warm-up writes."""
    import csv
    import datetime
    import tempfile
    import types

    from laser_polio_gb300.core import PropertySet
    from laser_polio_gb300.utils import RESULT_TABLE_COLUMNS, save_sim_results

    nt, nodes = 2556, args.nodes
    rng = np.random.default_rng(args.seed)
    sim = types.SimpleNamespace(
        nt=nt, nodes=np.arange(nodes),
        results=types.SimpleNamespace(**{a: rng.integers(0, 200_000, (nt, nodes)).astype(np.int32)
                                         for _, a in RESULT_TABLE_COLUMNS}),
        datevec=[datetime.date(2019, 1, 1) + datetime.timedelta(days=d) for d in range(nt)],
        pars=PropertySet({"node_lookup": {n: {"dot_name": f"AFRO:NIGERIA:STATE_{n % 37}:LGA_{n}"}
                                          for n in range(nodes)}}))
    rows = nt * nodes
    W, K = max(1, min(args.warmup, 3)), max(1, min(args.steps, 5))
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "results.csv"
        for _ in range(W):
            save_sim_results(sim, path)
        t0 = time.perf_counter()
        for _ in range(K):
            save_sim_results(sim, path)
        native_s = (time.perf_counter() - t0) / K
        size = path.stat().st_size
        native_bytes = path.read_bytes()
        ref = Path(d) / "ref.csv"
        t0 = time.perf_counter()
        names = [c for c, _ in RESULT_TABLE_COLUMNS]
        arrs = [getattr(sim.results, a) for _, a in RESULT_TABLE_COLUMNS]
        with open(ref, "w", newline="") as f:
            w = csv.writer(f, lineterminator="\n")
            w.writerow(["timestep", "date", "node", "dot_name", *names])
            lookup = sim.pars.node_lookup
            for t in range(nt):
                ds = str(sim.datevec[t])
                for n in range(nodes):
                    w.writerow([t, ds, n, lookup[n]["dot_name"], *[int(a[t, n]) for a in arrs]])
        py_s = time.perf_counter() - t0
        same = ref.read_bytes() == native_bytes
    line = {
        "metric": "results table rows/s written as CSV",
        "value": rows / native_s,
        "unit": "rows/s",
        "n_gpus": 0,
        "steps": K,
        "warmup": W,
        "ms_per_step": native_s * 1e3,
        "higher_is_better": True,
        "dtype": "int32",
        "data": "synthetic (seeded counts)",
        "config": {"workload": f"save_sim_results CSV, {nt} timesteps x {nodes} nodes = {rows} rows",
                   "bytes": size, "threads": os.cpu_count()},
        "cpu_baseline": {"value": rows / py_s, "unit": "rows/s", "cores": 1, "kind": "port",
                         "sample": "the same file with Python's csv module, one write"},
        "identical_bytes": same,
    }
    print(json.dumps(line), flush=True)
    if args.out:
        Path(args.out).write_text(json.dumps(line, indent=1))


def main():
    args = parse()
    if args.export:
        export_arm(args)
        return
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.batch:
        batch_arm(args)
        return
    if args.incidence:
        incidence_arm(args)
        return
    if args.continental:
        continental_arm(args)
        return
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = local
    from laser_polio_gb300._lib import Handle
    from laser_polio_gb300.engine import make_desc

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    params, cols = make_bundle(args, rank, pinned=True)
    desc, keep = make_desc(params)
    W, K = args.warmup, args.steps
    nt = params["nt"]
    if W + K > nt - 1:
        K = max(1, nt - 1 - W)
    col_bytes = sum(v.nbytes for v in cols.values())
    P = min(W + K, args.parity_ticks)  # ticks of the oracle's parity leg


    # ---- end to end through the C ABI from pinned host columns --------------
    e2e = None
    e2e_res = e2e_cols = None
    if not args.no_e2e:
        # output buffers page-locked like the input columns, allocated before the timed region
        res = result_arrays(params, pinned=True)
        out_cols = {k: pinned_empty(v.shape, v.dtype) for k, v in cols.items()}
        warm_up_api(args, dev)
        barrier()
        t0 = time.perf_counter()
        marks = [t0]
        h = Handle([desc], device=dev)
        marks.append(time.perf_counter())
        h.bind_columns(0, cols)
        h.sync()
        marks.append(time.perf_counter())
        h.start()
        marks.append(time.perf_counter())
        h.step(W + K)
        h.sync()
        marks.append(time.perf_counter())
        h.read_results(0, res)
        barrier()
        marks.append(time.perf_counter())
        dt = time.perf_counter() - t0
        # the agent table back on the host as well (not part of a run's
        # result: the user path reads columns only when it asks for them)
        h.read_columns(0, out_cols)
        barrier()
        marks.append(time.perf_counter())
        dt_cols = marks[-1] - t0
        phases = dict(zip(("create", "bind", "start", "ticks", "read_results", "read_columns"),
                          (b - a for a, b in zip(marks, marks[1:]))))
        e2e_count = h.state(0).count
        h.close()
        cnt = counts_per_tick(params, res["births"])
        at = float(cnt[1 : W + K + 1].sum())
        res_bytes = sum(v.nbytes for v in res.values())
        e2e = {"value": at / dt, "unit": "agent-ticks/s", "h2d_bytes_per_step": int(col_bytes // (W + K)),
               "d2h_bytes_per_step": int(res_bytes // (W + K)), "seconds": dt, "ticks": W + K,
               "timed": "create, bind (every column up), start, ticks, read_results (the run's result down)",
               "with_columns": {"value": at / dt_cols, "seconds": dt_cols,
                                "d2h_bytes_per_step": int((res_bytes + col_bytes) // (W + K))},
               "phases_s": phases}
        if P == W + K:
            e2e_res, e2e_cols = res, out_cols
        else:
            del out_cols

    # the clocks of the rest of the device phase (timed region, full run, user
    # path, batch, profiling); started after the end-to-end leg, whose large
    # host-to-device copies nvidia-smi's polling slows down
    clocks = ClockSampler(dev)
    clocks.__enter__()
    clocks.wait_ready()

    # ---- device-resident timed region ------------------------------------
    h = Handle([desc], device=dev)
    h.bind_columns(0, cols)
    h.start()
    h.step(W)
    h.sync()
    c0 = h.counters()
    stream = torch.cuda.ExternalStream(h.cuda_stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = h.kernel_launches()
    barrier()
    timed_from = len(clocks.lines)
    e0.record(stream)
    h.step(K)
    e1.record(stream)
    h.sync()
    barrier()
    timed_to = len(clocks.lines)
    ms = e0.elapsed_time(e1)
    launches = h.kernel_launches() - l0
    c1 = h.counters()
    work = {k: c1[k] - c0[k] for k in c1}
    res = result_arrays(params)
    h.read_results(0, res)
    st = h.state(0)
    h.close()
    cnt = counts_per_tick(params, res["births"])
    ticks = np.arange(W + 1, W + K + 1)
    agent_ticks = float(cnt[ticks].sum())
    ms_max, at_total = reduce_over_ranks(ms, agent_ticks, ws, "cuda")
    value = at_total / (ms_max / 1e3)

    # ---- the whole run, and the time of each kind of tick ------------------
    full = None
    if not args.no_full_run:
        full = full_run(desc, cols, params, dev)

    # ---- the user's path: construct (device initialisation) and run -------
    api = None
    if not args.no_api:
        api = api_run(args, dev)

    # ---- the calibration batch: 64 replicates in one handle vs one by one --
    batch = None
    if not args.no_batch and ws == 1:
        batch = batch_measure(args.batch_reps, args.seed, W, K)

    # ---- per-kernel times (profiling mode, same ticks) --------------------
    roof = None
    prof = None
    if not args.no_profile:
        h = Handle([desc], device=dev)
        h.bind_columns(0, cols)
        h.start()
        h.step(W)
        h.sync()
        h.set_profiling(True)
        h.step(K)
        h.sync()
        prof = merge_selection(h.profile())
        h.close()
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        peak = float(peaks.get("hbm_gbs", 6800.0))
        which = "measured" if "hbm_gbs" in peaks else "fallback"
        share = {k: v[0] / sum(x[0] for x in prof.values()) for k, v in prof.items()}
        # agents exposed by transmission: new exposures less the RI and SIA protections counted with them
        new_exposed = int(res["new_exposed"][ticks].sum() - res["ri_protected"][ticks].sum()
                          - res["sia_protected"][ticks].sum())
        alg = kernel_alg_bytes(params, ticks, cnt, work, new_exposed, (res["I"] > 0).sum(axis=1))
        per_kernel = {}
        for k, (tot_ms, nl) in prof.items():
            row = {"ms_per_launch": tot_ms / max(1, nl), "launches": nl, "share": share[k]}
            if k in alg:
                row["alg_bytes_per_launch"] = alg[k] / max(1, nl)
                row["achieved_gbs"] = alg[k] / (tot_ms / 1e3) / 1e9 if tot_ms > 0 else None
                row["frac"] = row["achieved_gbs"] / peak if row["achieved_gbs"] is not None else None
            per_kernel[k] = row
        top = max(prof, key=lambda k: prof[k][0])
        t_ms, t_n = prof[top]
        per_launch_ms = t_ms / max(1, t_n)
        t_alg = alg.get(top)
        achieved = t_alg / (t_ms / 1e3) / 1e9 if t_alg is not None else None
        traffic = None
        if top in NCU_TRAFFIC_PER_UNIT:
            unit, per_unit, fixed = NCU_TRAFFIC_PER_UNIT[top]
            traffic = (per_unit * work[unit] + fixed * t_n) / max(1, t_n)
        col = sum(tick_bytes(params, t) * cnt[t] for t in ticks) / K
        roof = {
            "kernel": top,
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak if achieved is not None else None,
            "traffic": traffic,
            "traffic_source": NCU_TRAFFIC_SOURCE.get(top),
            "peak_source": which,
            "alg_bytes_per_launch": t_alg / max(1, t_n) if t_alg is not None else None,
            "mean_launch_ms": per_launch_ms,
            "share_of_tick": share[top],
            "work": work,
            "reference_column_bytes_per_tick": col,
            "reference_column_equiv_gbs": col / (ms / K / 1e3) / 1e9,
            "kernels": per_kernel,
        }

    # the parity leg's own device run when the e2e run covered other ticks
    if rank == 0 and not args.no_cpu and e2e_res is None:
        h = Handle([desc], device=dev)
        h.bind_columns(0, cols)
        h.start()
        h.step(P)
        h.sync()
        e2e_res = result_arrays(params)
        h.read_results(0, e2e_res)
        e2e_count = h.state(0).count
        e2e_cols = {k: np.empty(v.shape, v.dtype) for k, v in cols.items()}
        h.read_columns(0, e2e_cols)
        h.close()
    clocks.__exit__(None, None, None)

    # ---- CPU baseline and parity: the oracle over the same ticks -----------
    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        del h
        cpu_res = oracle_leg(params, cols, min(W, P - 1), P - min(W, P - 1))
        o = cpu_res.pop("oracle")
        if o.state().t - 1 != P or e2e_count != o.state().count:
            parity = {"bit_exact": False, "mismatches": [f"state: oracle at tick {o.state().t} with "
                                                         f"{o.state().count} agents, GPU {e2e_count}"]}
        else:
            parity = compare_with_oracle(o, e2e_res, lambda name, dtype: e2e_cols[name], params, e2e_count)
        parity = {"ticks": P, "agents": params["count"], **parity}
        o.close()
        w0 = min(W, P - 1)
        cpu = {"value": cpu_res["value"], "unit": "agent-ticks/s", "cores": cpu_res["cores"], "kind": "port",
               "sample": f"oracle, ticks {w0 + 1}-{P} after {w0} untimed of the same population "
                         f"({cpu_res['seconds']:.1f} s)"}

    if rank == 0:
        summ = clocks.summary()
        summ["samples_in_timed_region"] = timed_to - timed_from
        summ["window"] = "nvidia-smi every 100 ms from the timed region to the end of the device phase " \
                         "(timed region, full run, user path, batch, profiling)"
        line = {
            "metric": "agent-ticks/s (774 nodes, 2.2e8 agents, full agent step)",
            "value": value,
            "unit": "agent-ticks/s",
            "n_gpus": ws,
            "steps": K,
            "warmup": W,
            "ms_per_step": ms_max / K,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "int8/int32 state, f64 node FOI",
            "data": "synthetic (seeded numpy, Nigeria-scale shapes)",
            "config": workload_config(params, W, K, ws),
            "e2e": e2e,
            "roofline": roof,
            "cpu_baseline": cpu,
            "parity": parity,
            "full_run": full,
            "e2e_api": api,
            "batch": batch,
            "clocks": summ,
            "gpu_launches": launches,
            "work_counters": work,
            "final_tick": st.t,
            "new_exposed_total": int(res["new_exposed"].sum()),
        }
        print(json.dumps(line), flush=True)
        if args.out:
            Path(args.out).write_text(json.dumps(line, indent=1))
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
