"""count_SEIRP (laser_polio/model.py:869-929) as a standalone op.

CPU: the numpy restatement in the oracle agrees with the counts the C oracle
logs for Transmission_ABM.log (model.py:1461-1483) after a run.  GPU: the
CUDA entry point lpg_count_seirp equals the restatement on seeded columns,
including dead slots, unaligned column views (slot-by-slot path), ragged
tails, empty input, invalid node ids and strains, and the node limit.
"""

import ctypes as C

import numpy as np
import pytest

from laser_polio_gb300 import synthetic
from oracle.oracle import count_seirp
from oracle_backend import run_spec_oracle
from oracle_backend import snapshot

NAMES = ("S", "E", "I", "R", "E_by_strain", "I_by_strain", "potentially_paralyzed", "paralyzed")


def random_columns(n, G, ns, seed, p_dead=0.1, bad_nodes=0, bad_strains=0):
    rng = np.random.default_rng(seed)
    node = np.sort(rng.integers(0, G, n)).astype(np.int16)  # the reference's node-contiguous layout
    if n:
        node[rng.integers(0, n, min(n, 2000))] = rng.integers(0, G, min(n, 2000))  # births appended out of order
    ds = rng.choice(np.array([-1, 0, 1, 2, 3], np.int8), n, p=[p_dead, 0.5 - p_dead, 0.1, 0.1, 0.3])
    st = rng.integers(0, ns, n).astype(np.int8)
    pp = rng.choice(np.array([-1, 0, 1], np.int8), n, p=[0.8, 0.1, 0.1])
    pa = (rng.random(n) < 0.05).astype(np.int8)
    if bad_nodes:
        i = rng.integers(0, n, bad_nodes)
        node[i] = np.where(rng.random(bad_nodes) < 0.5, -3, G + 5).astype(np.int16)
    if bad_strains:
        i = rng.integers(0, n, bad_strains)
        ds[i] = 2
        st[i] = ns
    return node, ds, st, pp, pa


def test_restatement_matches_oracle_log():
    sim = synthetic.zamfara_like(n_agents=60_000, dur=40, seed=7)
    spec, cols, res = snapshot(sim)
    st = run_spec_oracle(spec, cols, res, 40)
    t = st.t - 1
    G = res["S"].shape[1]
    ns = res["E_by_strain"].shape[2]
    got = count_seirp(cols["node_id"], cols["disease_state"], cols["strain"], cols["potentially_paralyzed"],
                      cols["paralyzed"], G, ns, st.count)
    assert got[-1] == 0
    for name, a in zip(NAMES, got[:-1]):
        np.testing.assert_array_equal(a, res[name][t], err_msg=name)


def _gpu_count(entry, cols, G, ns, n, offset=0):
    import torch

    from laser_polio_gb300 import _lib

    lib = _lib.load()
    dev = [torch.from_numpy(np.concatenate([np.zeros(offset, c.dtype), c])).cuda()[offset:] for c in cols]
    outs = [torch.full((G,), -7, dtype=torch.int32, device="cuda") for _ in range(4)]
    ebs = torch.full((G, ns), -7, dtype=torch.int32, device="cuda")
    ibs = torch.full((G, ns), -7, dtype=torch.int32, device="cuda")
    potp = torch.full((G,), -7, dtype=torch.int32, device="cuda")
    par = torch.full((G,), -7, dtype=torch.int32, device="cuda")
    bad = torch.full((1,), -7, dtype=torch.int64, device="cuda")
    S, E, I, R = outs
    stream = torch.cuda.current_stream().cuda_stream
    rc = getattr(lib, entry)(*[c.data_ptr() for c in dev], G, ns, n, S.data_ptr(), E.data_ptr(), I.data_ptr(),
                             R.data_ptr(), ebs.data_ptr(), ibs.data_ptr(), potp.data_ptr(), par.data_ptr(),
                             bad.data_ptr(), C.c_void_p(stream))
    assert rc == 0, lib.lpg_op_last_error()
    torch.cuda.synchronize()
    return tuple(t.cpu().numpy() for t in (S, E, I, R, ebs, ibs, potp, par)) + (int(bad.item()),)


def _check(cols, G, ns, n, offset=0, entry="lpg_count_seirp"):
    want = count_seirp(*cols, G, ns, n)
    got = _gpu_count(entry, cols, G, ns, n, offset)
    for name, a, b in zip(NAMES + ("n_invalid",), want, got):
        np.testing.assert_array_equal(b, a, err_msg=name)
    return got


@pytest.mark.gpu
@pytest.mark.parametrize(
    "n,G,ns,offset",
    [
        (0, 5, 3, 0),
        (1, 1, 1, 0),
        (15, 3, 2, 0),
        (4097 * 16 + 7, 14, 3, 0),
        (1_000_003, 774, 3, 0),
        (1_000_003, 774, 3, 1),  # unaligned views: the slot-by-slot path
        (2_000_000, 4096, 4, 0),  # the node limit, largest histogram
        (300_000, 44, 1, 3),
    ],
)
def test_gpu_count_matches_restatement(n, G, ns, offset):
    cols = random_columns(n, G, ns, seed=n + G)
    _check(cols, G, ns, n, offset)


@pytest.mark.gpu
def test_gpu_count_invalid_slots_and_prefix():
    n, G, ns = 500_000, 60, 3
    cols = random_columns(n, G, ns, seed=11, bad_nodes=123, bad_strains=45)
    got = _check(cols, G, ns, n)
    assert got[-1] > 0
    _check(cols, G, ns, n - 12345)  # only the active prefix [0, n_people) counts


@pytest.mark.gpu
def test_gpu_count_large():
    n, G, ns = 40_000_003, 774, 3
    cols = random_columns(n, G, ns, seed=2)
    _check(cols, G, ns, n)


@pytest.mark.gpu
def test_gpu_wrapper_and_errors():
    import torch

    from laser_polio_gb300.ops import count_SEIRP

    n, G, ns = 100_000, 20, 3
    cols = random_columns(n, G, ns, seed=4)
    want = count_seirp(*cols, G, ns, n)
    got = count_SEIRP(*cols, G, ns, n)
    for name, a, b in zip(NAMES, want, got):
        np.testing.assert_array_equal(b, a, err_msg=name)
    tcols = [torch.from_numpy(c).cuda() for c in cols]
    got_t = count_SEIRP(*tcols, G, ns, n)
    assert got_t[0].is_cuda
    np.testing.assert_array_equal(got_t[0].cpu().numpy(), want[0])
    with pytest.raises(ValueError, match="n_nodes"):
        count_SEIRP(*cols, 5000, ns, n)
    with pytest.raises(ValueError, match="n_strains"):
        count_SEIRP(*cols, G, 5, n)
