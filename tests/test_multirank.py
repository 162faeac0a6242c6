"""The multi-GPU path's host logic on CPU: two gloo ranks shard a batch of
chambers with no overlap and combine their results the way bench.py does
(sum of work over the slowest rank's time)."""
import importlib.util
import json
import os
import socket

import pytest

import helpers as H

torch = pytest.importorskip("torch")

_spec = importlib.util.spec_from_file_location(
    "multirank", os.path.join(H.ROOT, "astrophage-microscope_gb300", "multirank.py"))
MR = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(MR)


def test_lpt_shards_cover_and_balance():
    costs = [float(c) for c in (9, 1, 7, 3, 3, 8, 2, 5, 6, 4)]
    shards = MR.lpt_shards(costs, 3)
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(costs)
    assert MR.lpt_shards(costs, 3) == shards               # deterministic
    assert MR.lpt_shards(costs, 1) == [list(range(len(costs)))]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world_size, port, costs, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        mine = MR.lpt_shards(costs, world_size)[rank]
        units = sum(costs[i] for i in mine)               # work this rank did
        seconds = 1.0 + rank                              # the slower rank sets the job's time
        total = MR.reduce_sum(dist, units)
        slowest = MR.reduce_max(dist, seconds)
        rate = MR.job_rate(dist, units, seconds)
        dist.barrier()
        with open(out_path % rank, "w") as fh:
            json.dump([sorted(mine), total, slowest, rate], fh)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce(tmp_path):
    costs = [5.0, 3.0, 8.0, 1.0, 4.0, 2.0, 7.0]
    port = _free_port()
    out = str(tmp_path / "rank%d.txt")
    torch.multiprocessing.spawn(_rank_main, args=(2, port, costs, out), nprocs=2, join=True)
    got = []
    for r in range(2):
        with open(out % r) as fh:
            mine, total, slowest, rate = json.load(fh)
        got.append(mine)
        assert total == sum(costs)
        assert slowest == 2.0
        assert rate == sum(costs) / 2.0
    assert sorted(got[0] + got[1]) == list(range(len(costs)))
    assert not set(got[0]) & set(got[1])
