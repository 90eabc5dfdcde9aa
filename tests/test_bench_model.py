"""The benchmark's host-side pieces, on the CPU: the continental workload's
synthetic shapes, the parameters the byte model reads from a simulation
description, and the byte model's mixing term (bench.kernel_alg_bytes)."""

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

import bench  # noqa: E402
from laser_polio_gb300 import synthetic  # noqa: E402
from laser_polio_gb300.core import gravity, row_normalizer  # noqa: E402
from laser_polio_gb300.engine import make_desc  # noqa: E402


def test_continental_bundle_has_the_workloads_shapes():
    """4000 nodes whose populations sum to the agents asked for, a dense
    network from the distances returned beside it (gravity k 0.5, a = b = 1,
    c = 2, max export fraction 0.2), RI, an SIA every 180 days, 3 strains."""
    p, cols = synthetic.bundle("continental", n_agents=400_000, dur=200, seed=3)
    assert p["n_nodes"] == 4000 and p["count"] == 400_000 and p["nt"] == 201 and p["n_strains"] == 3
    assert p["pop0"].sum() == 400_000 and p["pop0"].min() >= 1
    d = p["distances"]
    assert d.shape == (4000, 4000) and np.all(np.diag(d) == 0) and d.max() <= 5000.0 * np.sqrt(2)
    pops = p["pop0"].astype(np.float64)
    want = row_normalizer(gravity(pops, d, 0.5, 1, 1, 2.0) / np.power(pops.sum(), 2.0), 0.2)
    np.testing.assert_array_equal(p["network"], want)
    assert p["ri_enabled"] and [e[0] for e in p["sia"]] == [180]
    assert len(cols["node_id"]) == p["capacity"] and int((cols["node_id"][: p["count"]] >= 0).sum()) == 400_000


def test_continental_and_nigeria_parameters_share_one_recipe():
    """continental_pars is the Nigeria-scale recipe with the continental
    node populations and square; the Nigeria-scale defaults are unchanged."""
    a, immun_a, _ = synthetic.nigeria_like_pars(n_agents=1_000_000, n_nodes=50, dur=30, seed=5)
    b, immun_b, _ = synthetic.nigeria_like_pars(n_agents=1_000_000, n_nodes=50, dur=30, seed=5,
                                                mu=np.log(2.8e5), sigma=0.7, side_km=1000.0)
    np.testing.assert_array_equal(a["init_pop"], b["init_pop"])
    np.testing.assert_array_equal(a["distances"], b["distances"])
    np.testing.assert_array_equal(immun_a, immun_b)
    c, _, _ = synthetic.continental_pars(n_agents=1_000_000, n_nodes=50, dur=30, seed=5)
    assert int(np.sum(c["init_pop"])) == 1_000_000 and c["distances"].max() > 1000.0 * np.sqrt(2)


def test_desc_params_reads_the_fields_the_byte_model_uses():
    p, _ = synthetic.bundle("nigeria", n_agents=50_000, n_nodes=20, dur=400, seed=2)
    desc, _keep = make_desc(p)
    q = bench.desc_params(desc)
    assert (q["n_nodes"], q["n_strains"], q["capacity"]) == (20, 3, p["capacity"])
    assert (q["vd_step"], q["ri_enabled"], q["ri_step"]) == (p["vd_step"], p["ri_enabled"], p["ri_step"])
    assert [t for (t,) in q["sia"]] == [e[0] for e in p["sia"]]


def test_mixing_bytes_count_only_sources_with_infected_agents():
    """k_node_mix reads, per tick, 16 B of network for each (node, source
    with infected agents), 8 B per node and strain of infectivity totals and
    20 B per chunk; sources without infectivity cost nothing."""
    p = {"n_nodes": 10, "n_strains": 3, "capacity": 4096, "vd_step": 7, "ri_enabled": 0, "ri_step": 14, "sia": []}
    ticks = np.arange(1, 4)
    cnt = np.full(5, 1000)
    work = dict.fromkeys(("sweep_index", "sweep_due", "sweep_evt_due", "sweep_dod_due", "queue_ds", "queue_rs",
                          "sel_targets", "ri_index", "ri_due"), 0)
    none = bench.kernel_alg_bytes(p, ticks, cnt, work, 0, np.zeros(5, int))["k_node_mix"]
    some = bench.kernel_alg_bytes(p, ticks, cnt, work, 0, np.array([0, 2, 2, 2, 0]))["k_node_mix"]
    chunks = 3 * bench.NODE_TX_CHUNK_B * 4096 / 2048
    assert none == 3 * 10 * 3 * 8.0 + chunks
    assert some - none == 3 * 10 * 2 * bench.NODE_TX_NET_B
