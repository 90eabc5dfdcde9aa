"""Expected incidence and its vector-Jacobian product (lpg_expected_incidence).

CPU: the numpy restatement (oracle/incidence.py) is pinned to the package's
network and seasonality builders (the ones the engine runs on) and its
reverse pass to fourth-order central finite differences of its own forward
pass, with and without capped network rows.  GPU: the CUDA path against the
oracle on the same inputs; FP64 elementwise work, double-float products
(about 2^-45 of the summed terms) and atomically reduced sums, so agreement
is to a relative 1e-9, not bit for bit."""

import datetime

import numpy as np
import pytest

from laser_polio_gb300 import ops
from laser_polio_gb300.core import gravity, row_normalizer
from laser_polio_gb300.utils import seasonality_table
from oracle import incidence as I

SCALARS = ("R", "amp", "peak", "k", "a", "b", "c")
FD_RTOL = 1e-6


def _loss(inp, g, **mod):
    x = dict(inp)
    x.update(mod)
    return float((g * I.incidence(x)[0]).sum())


def _fd(f, x0, h):
    return (-f(x0 + 2 * h) + 8 * f(x0 + h) - 8 * f(x0 - h) + f(x0 - 2 * h)) / (12 * h)


def _case(max_frac):
    inp = I.random_inputs(10, 8, 2, seed=3)
    inp["max_frac"] = max_frac
    g = np.random.default_rng(2).normal(size=(10, 8))
    return inp, g


@pytest.mark.parametrize("max_frac", [0.2, 3.5e-6], ids=["uncapped", "capped"])
def test_oracle_vjp_matches_finite_differences(max_frac):
    inp, g = _case(max_frac)
    _, _, rs, capped = I.network(inp["pops"], inp["dist"], inp["k"], inp["a"], inp["b"], inp["c"], max_frac)
    if max_frac < 1e-3:
        assert 0 < capped.sum() < len(capped)
        # keep every row sum away from the cap under the steps below
        assert np.min(np.abs(rs / max_frac - 1.0)) > 0.05
    else:
        assert not capped.any()
    _, gr = I.incidence(inp, g)
    for name in SCALARS:
        h = 1e-3 * max(1.0, abs(inp[name]))
        fd = _fd(lambda v: _loss(inp, g, **{name: v}), inp[name], h)
        # L is ~1e4 and moves by ~1e-4 per unit of k, a, b, c: cancellation
        # limits those differences to ~1e-4 here; the chain check below is tight
        tol = FD_RTOL if name in ("R", "amp", "peak") else 5e-4
        assert abs(gr[name] - fd) <= tol * abs(fd), (name, gr[name], fd)
    # k, a, b, c through the network alone: d/dtheta sum(dL/dN * N(theta))
    W = gr["network"]
    par = {n: inp[n] for n in ("k", "a", "b", "c")}
    for name in par:
        def f(v, name=name):
            q = dict(par, **{name: v})
            return float((W * I.network(inp["pops"], inp["dist"], q["k"], q["a"], q["b"], q["c"], max_frac)[0]).sum())
        fd = _fd(f, par[name], 1e-3 * max(1.0, abs(par[name])))
        assert abs(gr[name] - fd) <= FD_RTOL * abs(fd), ("chain", name, gr[name], fd)
    for j in (0, 5):
        def f(v, j=j):
            r = inp["r0s"].copy()
            r[j] = v
            return _loss(inp, g, r0s=r)
        fd = _fd(f, inp["r0s"][j], 1e-3)
        assert abs(gr["r0s"][j] - fd) <= FD_RTOL * abs(fd), ("r0s", j)
    # dL/dN: perturb the normalised network directly
    N = I.network(inp["pops"], inp["dist"], inp["k"], inp["a"], inp["b"], inp["c"], max_frac)[0]
    args = [inp[n] for n in ("srisk", "beta", "pop", "doy", "year", "r0s", "R", "amp", "peak")]
    for a, b in ((2, 5), (7, 0)):
        def f(v, a=a, b=b):
            M = N.copy()
            M[a, b] = v
            return float((g * I.forward(*args, M)[0]).sum())
        fd = _fd(f, N[a, b], 1e-4)
        assert abs(gr["network"][a, b] - fd) <= FD_RTOL * abs(fd) + 1e-12, ("network", a, b)
    assert np.all(np.diag(gr["network"]) == 0.0)


def test_oracle_network_is_the_engines_network():
    inp = I.random_inputs(2, 40, 1, seed=7)
    for max_frac in (0.2, 1e-5):
        N = I.network(inp["pops"], inp["dist"], 0.5, 1.0, 1.0, 2.0, max_frac)[0]
        want = row_normalizer(gravity(inp["pops"], inp["dist"], 0.5, 1.0, 1.0, 2.0)
                              / np.power(inp["pops"].sum(), 2.0), max_frac)
        np.testing.assert_allclose(N, want, rtol=1e-14, atol=0)


def test_oracle_seasonality_is_the_engines_seasonality():
    dates = [datetime.date(2019, 1, 1) + datetime.timedelta(days=d) for d in range(800)]  # 2020 is a leap year
    doy = np.array([d.timetuple().tm_yday for d in dates], np.float64)
    year = np.array([366.0 if d.year == 2020 else 365.0 for d in dates])
    inp = I.random_inputs(len(dates), 3, 1, seed=1)
    inp.update(doy=doy, year=year, amp=0.3, peak=200.0)
    N = I.network(inp["pops"], inp["dist"], inp["k"], inp["a"], inp["b"], inp["c"], inp["max_frac"])[0]
    _, mid = I.forward(*[inp[n] for n in ("srisk", "beta", "pop", "doy", "year", "r0s", "R", "amp", "peak")], N)
    np.testing.assert_allclose(mid["seas"], seasonality_table(dates, 0.3, 200.0), rtol=1e-14, atol=0)


def test_wrapper_rejects_bad_shapes_before_any_device_call():
    inp = I.random_inputs(4, 5, 2, seed=0)
    bad = dict(inp, pop=inp["pop"][:, :3])
    with pytest.raises(ValueError, match="pop"):
        ops.expected_incidence(bad)
    with pytest.raises(ValueError, match="g has shape"):
        ops.expected_incidence(inp, np.zeros((4, 4)))


def _close(got, want, rtol, what):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = np.max(np.abs(want)) if want.size else 0.0
    err = np.max(np.abs(got - want)) if want.size else 0.0
    assert err <= rtol * max(scale, 1e-300), (what, err, scale)


@pytest.mark.gpu
@pytest.mark.parametrize(
    "T,G,S,max_frac,seed",
    [(1, 1, 1, 0.2, 0), (10, 8, 2, 3.5e-6, 3), (37, 33, 3, 0.2, 5), (365, 100, 1, 1e-5, 11), (30, 774, 4, 0.2, 2)],
)
def test_gpu_incidence_and_vjp_match_oracle(T, G, S, max_frac, seed):
    """Relative 1e-9 of each output's largest magnitude (the GPU sums in
    another order, with atomics and double-float products)."""
    inp = I.random_inputs(T, G, S, seed=seed)
    inp["max_frac"] = max_frac
    g = np.random.default_rng(seed + 100).normal(size=(T, G))
    want_lam, want = I.incidence(inp, g)
    lam0, none = ops.expected_incidence(inp)
    assert none is None
    lam, got = ops.expected_incidence(inp, g)
    _close(lam0, want_lam, 1e-12, "lam")
    _close(lam, want_lam, 1e-12, "lam with g")
    for name in SCALARS:
        _close(got[name], want[name], 1e-9, name)
    _close(got["r0s"], want["r0s"], 1e-9, "r0s")
    _close(got["network"], want["network"], 1e-9, "network")
    assert np.all(np.diag(got["network"]) == 0.0)


def test_plan_without_gpu_reports_cuda_error():
    import torch

    from laser_polio_gb300 import _lib

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_lib.LpgError):
        ops.IncidencePlan(I.random_inputs(3, 4, 1, seed=0))


def _oracle_loss_grad(inp, target):
    lam, _ = I.incidence(inp)
    r = np.log1p(lam) - np.log1p(target)
    _, grads = I.incidence(inp, 2.0 * r / (1.0 + lam))
    return lam, float((r * r).sum()), grads


@pytest.mark.gpu
@pytest.mark.parametrize("T,G,S,max_frac", [(20, 16, 3, 0.2), (60, 120, 2, 1e-5)])
def test_gpu_plan_target_loss_and_gradient_match_oracle(T, G, S, max_frac):
    """A plan with a target curve: the loss and its gradient at several
    parameter sets against the oracle (relative 1e-9; loss 1e-11), the
    aggregates uploaded once."""
    inp = I.random_inputs(T, G, S, seed=9)
    inp["max_frac"] = max_frac
    rng = np.random.default_rng(4)
    target = I.incidence(dict(inp, R=1.3, amp=0.3, r0s=inp["r0s"] * rng.lognormal(0, 0.1, G)))[0]
    plan = ops.IncidencePlan(inp, target)
    plan.set_profiling(True)
    try:
        for R, amp, peak, k in ((1.1, 0.4, 180.0, 0.5), (0.9, 0.25, 30.0, 0.8), (1.1, 0.4, 180.0, 0.5)):
            x = dict(inp, R=R, amp=amp, peak=peak, k=k)
            want_lam, want_loss, want = _oracle_loss_grad(x, target)
            got = plan.evaluate(x, lam=True)
            _close(got["lam"], want_lam, 1e-12, "lam")
            assert abs(got["loss"] - want_loss) <= 1e-11 * want_loss, (got["loss"], want_loss)
            for name in SCALARS:
                _close(got["grad"][name], want[name], 1e-9, name)
            _close(got["grad"]["r0s"], want["r0s"], 1e-9, "r0s")
            _close(got["grad"]["network"], want["network"], 1e-9, "network")
        # an explicit g overrides the target loss's dL/dlam
        g = rng.normal(size=(T, G))
        got = plan.evaluate(inp, g, network_grad=False)
        _, want = I.incidence(inp, g)
        assert "network" not in got["grad"]
        for name in SCALARS:
            _close(got["grad"][name], want[name], 1e-9, name)
        prof = plan.profile()
        assert list(prof) == ["k_inc_network", "k_inc_gemm_mix", "k_inc_forward", "k_inc_backward",
                              "k_inc_gemm_flows", "k_inc_network_grad"]
        assert all(ms > 0 and n >= 4 for ms, n in prof.values())
    finally:
        plan.close()


@pytest.mark.gpu
def test_gpu_engine_records_the_aggregates_its_exposures_come_from():
    """A forward run of the engine records, per transmission tick, the
    aggregates the adjoint replays (lpg_record_aggregates); the expected-
    incidence map on them reproduces the engine's own expected exposures
    (relative 1e-9 of the largest: the engine mixes in exact integers and
    uses expm1, the map in double-float and 1 - exp, as model.py does)."""
    from laser_polio_gb300 import synthetic
    from laser_polio_gb300._lib import Handle
    from laser_polio_gb300.engine import make_desc

    params, cols = synthetic.bundle(kind="nigeria", n_agents=300_000, n_nodes=30, dur=150, seed=7)
    G, ns, nt = params["n_nodes"], params["n_strains"], params["nt"]
    rng = np.random.default_rng(1)
    xy = rng.uniform(0, 300, (G, 2))
    dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(dist, 0.0)
    pops = params["pop0"].astype(np.float64)
    net = dict(k=1.2e4, a=1.0, b=1.0, c=2.0, max_frac=0.05)  # 16 of 30 rows capped
    params["network"] = row_normalizer(gravity(pops, dist, net["k"], net["a"], net["b"], net["c"])
                                       / np.power(pops.sum(), net["c"]), net["max_frac"])
    assert 0 < (params["network"].sum(1) >= net["max_frac"] * (1 - 1e-12)).sum() < G  # capped and uncapped rows
    desc, _keep = make_desc(params)
    h = Handle([desc])
    try:
        h.record_aggregates(0)
        h.bind_columns(0, cols)
        h.start()
        h.step(nt - 1)
        h.sync()
        agg = h.read_aggregates(0, nt, G, ns)
    finally:
        h.close()
    dates = [datetime.date(2019, 1, 1) + datetime.timedelta(days=d) for d in range(nt)]
    np.testing.assert_array_equal(seasonality_table(dates, 0.4, 180), params["seasonality"])
    doy = np.array([d.timetuple().tm_yday for d in dates], np.float64)
    year = np.array([366.0 if d.year % 4 == 0 else 365.0 for d in dates])
    ticks = slice(1, nt)  # no component runs on tick 0
    assert np.all(agg["pop"][ticks] > 0) and agg["lam"][ticks].sum() > 0
    inp = dict(srisk=agg["srisk"][ticks], beta=agg["beta"][ticks], pop=agg["pop"][ticks], doy=doy[ticks],
               year=year[ticks], r0s=params["r0_scalars"], R=1.0, amp=0.4, peak=180.0, pops=pops, dist=dist, **net)
    lam, _ = ops.expected_incidence(inp)
    _close(lam, agg["lam"][ticks], 1e-9, "engine exposures")


@pytest.mark.gpu
def test_gpu_replayed_nigeria_like_runs_give_the_adjoints_inputs_and_target():
    """The adjoint's replay as the bench runs it (bench.replay_inputs), on a
    small Nigeria-like population: two simulations of one agent table in one
    handle, base and perturbed parameters, both recording.  The map on the
    base run's aggregates reproduces its exposures within 1e-9 of the
    largest; the target (the perturbed run's exposures) differs from them;
    the plan's loss equals the oracle's on the same inputs and target, and
    its R gradient is negative (the target has 10% more infectivity)."""
    import types
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench

    args = types.SimpleNamespace(agents=4e5, nodes=40, seed=11)
    inp, target, rec = bench.replay_inputs(args, 120, 0)
    assert inp["srisk"].shape == (120, 40) and inp["beta"].shape == (120, 40, 3) and target.shape == (120, 40)
    assert rec["map_vs_engine_max_rel"] < 1e-9 and rec["new_exposed_expected"] > 0
    assert rec["target_expected"] > 0 and not np.array_equal(target, inp["srisk"])
    plan = ops.IncidencePlan(inp, target)
    try:
        res = plan.evaluate(inp)
    finally:
        plan.close()
    lam_o, _ = I.incidence(inp)
    resid = np.log1p(lam_o) - np.log1p(target)
    loss_o = float((resid**2).sum())
    assert abs(res["loss"] - loss_o) <= 1e-11 * abs(loss_o)
    assert res["grad"]["R"] < 0


def test_plan_rejects_bad_arguments_before_any_device_call():
    """lpg_incidence_plan_create checks sizes and inputs on the host first
    (LPG_ERR_ARG -> ValueError), with or without a GPU."""
    inp = I.random_inputs(4, 5, 2, seed=0)
    with pytest.raises(ValueError, match="pops"):
        ops.IncidencePlan(dict(inp, pops=-inp["pops"]))
    dist = inp["dist"].copy()
    dist[1, 3] = -1.0
    with pytest.raises(ValueError, match="dist"):
        ops.IncidencePlan(dict(inp, dist=dist))
    with pytest.raises(ValueError, match="total population"):
        ops.IncidencePlan(dict(inp, pops=np.zeros_like(inp["pops"])))
    beta5 = np.zeros((4, 5, 5))
    with pytest.raises(ValueError, match="bad sizes"):
        ops.IncidencePlan(dict(inp, beta=beta5))


def _recording_bundle(n_agents, n_nodes, dur, seed, capped_rows):
    """A synthetic run with its own gravity network (distances kept), k set
    so that about ``capped_rows`` rows reach max_frac."""
    from laser_polio_gb300 import synthetic

    params, cols = synthetic.bundle(kind="nigeria", n_agents=n_agents, n_nodes=n_nodes, dur=dur, seed=seed)
    G = params["n_nodes"]
    rng = np.random.default_rng(seed + 1)
    xy = rng.uniform(0, 300, (G, 2))
    dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(dist, 0.0)
    pops = params["pop0"].astype(np.float64)
    raw = (gravity(pops, dist, 1.0, 1.0, 1.0, 2.0) / pops.sum() ** 2).sum(1)
    k = float("%.2g" % (0.05 / np.sort(raw)[::-1][capped_rows - 1] * 0.99))
    net = dict(k=k, a=1.0, b=1.0, c=2.0, max_frac=0.05)
    params["network"] = row_normalizer(gravity(pops, dist, k, 1.0, 1.0, 2.0) / pops.sum() ** 2, 0.05)
    return params, cols, pops, dist, net


def _replay_inputs(params, agg, pops, dist, net):
    nt = params["nt"]
    dates = [datetime.date(2019, 1, 1) + datetime.timedelta(days=d) for d in range(nt)]
    np.testing.assert_array_equal(seasonality_table(dates, 0.4, 180), params["seasonality"])
    doy = np.array([d.timetuple().tm_yday for d in dates], np.float64)
    year = np.array([366.0 if d.year % 4 == 0 else 365.0 for d in dates])
    ticks = slice(1, nt)  # no component runs on tick 0
    return dict(srisk=agg["srisk"][ticks], beta=agg["beta"][ticks], pop=agg["pop"][ticks], doy=doy[ticks],
                year=year[ticks], r0s=params["r0_scalars"], R=1.0, amp=0.4, peak=180.0, pops=pops, dist=dist, **net)


def test_oracle_map_reproduces_the_oracles_transmission_exposures():
    """The CPU oracle of the agent step (pinned to the reference's tests)
    records, per transmission tick, the aggregates it mixes and its expected
    exposures (model.py:1315-1363); the numpy expected-incidence map on those
    aggregates reproduces them (relative 1e-12 of the largest; measured 5e-15:
    the oracle mixes in exact integers and uses expm1, the map 1 - exp as
    model.py does), and recording leaves the run's results unchanged."""
    from laser_polio_gb300.engine import make_desc
    from oracle.oracle import OracleSim

    params, cols, pops, dist, net = _recording_bundle(60_000, 12, 90, seed=5, capped_rows=5)
    N = row_normalizer(gravity(pops, dist, net["k"], 1.0, 1.0, 2.0) / pops.sum() ** 2, 0.05)
    assert 0 < (N.sum(1) >= 0.05 * (1 - 1e-12)).sum() < len(pops)
    desc, keep = make_desc(params)
    runs = []
    for record in (True, False):
        o = OracleSim(desc, keepalive=keep)
        if record:
            o.record_aggregates()
        o.bind_columns({k: v.copy() for k, v in cols.items()})
        o.start()
        o.step(params["nt"] - 1)
        res = _results_like(params)
        o.read_results(res)
        agg = o.read_aggregates() if record else None
        o.close()
        runs.append((res, agg))
    for name in runs[0][0]:
        np.testing.assert_array_equal(runs[0][0][name], runs[1][0][name], err_msg=name)
    agg = runs[0][1]
    assert agg["lam"][1:].sum() > 0 and np.all(agg["pop"][1:] > 0)
    np.testing.assert_array_equal(agg["pop"][1:], runs[0][0]["pop"][1:])  # nothing is recorded on tick 0
    lam, _ = I.incidence(_replay_inputs(params, agg, pops, dist, net))
    _close(lam, agg["lam"][1:], 1e-12, "oracle exposures")


def _results_like(params):
    from laser_polio_gb300 import _abi

    nt, n, ns = params["nt"], params["n_nodes"], params["n_strains"]
    return {name: np.zeros((nt, n, ns) if wide else (nt, n), np.int32) for name, wide in _abi.RESULT_FIELDS}


class _OraclePlan:
    """IncidencePlan's evaluate() restated by the numpy oracle (CPU)."""

    def __init__(self, inp, target):
        self.inp, self.target, self.calls = inp, target, 0

    def evaluate(self, params, g=None, *, lam=False, loss=None, grad=True, network_grad=True):
        self.calls += 1
        x = dict(self.inp, **{k: params[k] for k in ("R", "amp", "peak", "k", "a", "b", "c", "max_frac")},
                 r0s=params["r0s"])
        lam_v, _ = I.incidence(x)
        out = {"lam": lam_v} if lam else {}
        r = None if self.target is None else np.log1p(lam_v) - np.log1p(self.target)
        if self.target is not None if loss is None else loss:
            out["loss"] = float((r * r).sum())
        if grad:
            out["grad"] = I.incidence(x, 2.0 * r / (1.0 + lam_v) if g is None else g)[1]
        return out


def test_fit_incidence_recovers_the_parameters_of_the_target():
    """Gradient-based calibration (calibrate.fit_incidence, L-BFGS-B on the
    adjoint's loss and gradient) recovers R, amp and peak of a target curve,
    and then the per-node r0 scalars as well."""
    from laser_polio_gb300.calibrate import fit_incidence

    inp = I.random_inputs(60, 10, 2, seed=21)
    truth = dict(R=1.25, amp=0.3, peak=150.0, k=0.5)
    target = I.incidence(dict(inp, **truth))[0]
    plan = _OraclePlan(inp, target)
    start = dict(inp, R=1.0, amp=0.45, peak=175.0)
    fit, res = fit_incidence(plan, start, free=("R", "amp", "peak"), bounds={"amp": (0.0, 1.0)})
    assert res.success, res.message
    for name in ("R", "amp", "peak"):
        assert abs(fit[name] - truth[name]) <= 1e-5 * max(1.0, abs(truth[name])), (name, fit[name])
    # the per-node r0 scalars too, with R held at its fitted value (R and r0s are not separable)
    r0_true = inp["r0s"].copy()
    target2 = I.incidence(dict(inp, **truth))[0]
    plan2 = _OraclePlan(inp, target2)
    fit2, res2 = fit_incidence(plan2, dict(fit, r0s=r0_true * 1.1), free=(), fit_r0s=True)
    assert res2.success, res2.message
    np.testing.assert_allclose(fit2["r0s"], r0_true, rtol=1e-5)
    with pytest.raises(ValueError, match="unknown"):
        fit_incidence(plan, start, free=("R0",))


def test_torch_autograd_function_gives_the_adjoints_gradient():
    """ops.ExpectedIncidence (a torch.autograd.Function over a plan): the
    calibration loss written in torch and backpropagated gives the oracle's
    gradient (relative 1e-12), and torch.autograd.gradcheck passes.  Every
    node-tick gets some local infectivity: where only mixing reaches a node,
    the rate is ~1e-10 and 1 - exp(-r) (the reference's form) cancels to
    ~1e-6 relative, which gradcheck's numerical Jacobian would inherit."""
    import torch

    inp = I.random_inputs(6, 5, 2, seed=13)
    inp["beta"] = inp["beta"] + 1.0
    target = I.incidence(dict(inp, R=1.2, amp=0.3))[0]
    plan = _OraclePlan(inp, target)
    params = {n: torch.tensor(float(inp[n]), dtype=torch.float64, requires_grad=True) for n in SCALARS}
    params["r0s"] = torch.tensor(inp["r0s"], dtype=torch.float64, requires_grad=True)
    params["max_frac"] = inp["max_frac"]
    lam = ops.expected_incidence_torch(plan, params)
    loss = ((torch.log1p(lam) - torch.log1p(torch.as_tensor(target))) ** 2).sum()
    loss.backward()
    _, want_loss, want = _oracle_loss_grad(inp, target)
    assert abs(loss.item() - want_loss) <= 1e-12 * want_loss
    for n in SCALARS:
        _close(params[n].grad.item(), want[n], 1e-12, n)
    _close(params["r0s"].grad.numpy(), want["r0s"], 1e-12, "r0s")

    def f(R, amp, r0s):
        return ops.expected_incidence_torch(plan, dict(params, R=R, amp=amp, r0s=r0s))

    args = (torch.tensor(1.1, dtype=torch.float64, requires_grad=True),
            torch.tensor(0.35, dtype=torch.float64, requires_grad=True),
            torch.tensor(inp["r0s"], dtype=torch.float64, requires_grad=True))
    # eps 1e-4: at 1e-6 the central differences carry ~1e-5 of rounding noise
    assert torch.autograd.gradcheck(f, args, eps=1e-4, atol=1e-6, rtol=1e-5)


@pytest.mark.gpu
def test_gpu_torch_autograd_function_on_a_plan():
    """ExpectedIncidence over a device plan: a torch loss backpropagated
    through it gives the oracle's gradient (relative 1e-9)."""
    import torch

    inp = I.random_inputs(30, 40, 3, seed=17)
    target = I.incidence(dict(inp, R=1.2, amp=0.3))[0]
    plan = ops.IncidencePlan(inp)
    try:
        params = {n: torch.tensor(float(inp[n]), dtype=torch.float64, requires_grad=True) for n in SCALARS}
        params["r0s"] = torch.tensor(inp["r0s"], dtype=torch.float64, requires_grad=True)
        params["max_frac"] = inp["max_frac"]
        lam = ops.expected_incidence_torch(plan, params)
        loss = ((torch.log1p(lam) - torch.log1p(torch.as_tensor(target))) ** 2).sum()
        loss.backward()
    finally:
        plan.close()
    _, want_loss, want = _oracle_loss_grad(inp, target)
    assert abs(loss.item() - want_loss) <= 1e-11 * want_loss
    for n in SCALARS:
        _close(params[n].grad.item(), want[n], 1e-9, n)
    _close(params["r0s"].grad.numpy(), want["r0s"], 1e-9, "r0s")


def test_oracle_recording_must_be_asked_before_start():
    """lpo_record_aggregates after the start is refused, and reading
    aggregates that were not recorded raises (as the engine's calls)."""
    from laser_polio_gb300 import synthetic
    from laser_polio_gb300.engine import make_desc
    from oracle.oracle import OracleSim

    params, cols = synthetic.bundle(kind="zamfara", n_agents=5_000, dur=5, seed=1)
    desc, keep = make_desc(params)
    o = OracleSim(desc, keepalive=keep)
    o.bind_columns(cols)
    o.start()
    with pytest.raises(RuntimeError, match="after start"):
        o.record_aggregates()
    with pytest.raises(RuntimeError, match="not recorded"):
        o.read_aggregates()
    o.close()
