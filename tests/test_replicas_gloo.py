"""The N-GPU bench runs N independent replicas (the per-tick path has no
exchange step): its whole-job figures are the slowest rank's time and the
sum of every rank's agent-ticks.  Checked here with two gloo ranks on the
CPU."""

import ast
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = [12.5, 20.0][rank]
    agent_ticks = [3.0e9, 5.0e9][rank]
    got = bench.reduce_over_ranks(ms, agent_ticks, ws, "cpu")
    Path(outdir, f"rank{rank}").write_text(repr(got))
    assert bench.dist_env() == (ws, rank, 0)
    dist.destroy_process_group()


def test_two_replicas_reduce_to_slowest_time_and_total_work(tmp_path):
    ws, port = 2, _free_port()
    mp.spawn(_rank, args=(ws, port, str(tmp_path)), nprocs=ws, join=True)  # spawn: no fork
    got = [ast.literal_eval((tmp_path / f"rank{r}").read_text()) for r in range(ws)]
    assert got[0] == got[1] == (20.0, 8.0e9)


def test_single_rank_is_unchanged():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reduce_over_ranks(7.0, 1.5e9, 1, "cpu") == (7.0, 1.5e9)
