"""Multi-rank host logic of bench.py on CPU: two gloo ranks (no GPU).

The path shards by queries: every rank builds its own replica and answers its own full-size
query set, with no collective on the data path; the only collectives are the barrier and the
max-over-ranks reduction of the step time, and the job value is all ranks' queries over the
slowest rank's time (weak scaling)."""
import json
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    Q = np.arange(3 * 64, dtype=np.float32).reshape(64, 3)
    near = np.arange(64) % 2 == 0
    q, m = bench.rank_queries(Q, near, rank)
    t = bench.max_over_ranks(dist, 0.5 + rank)  # this rank's "step time"
    choice = bench.rank0_choice(dist, (8 + 4 * rank, 2, 128, rank))  # each rank "tuned" its own
    bench.barrier(dist)
    res = {"max_t": t, "choice": choice, "sum": float(q.sum()), "first": q[0].tolist(),
           "near_ok": bool(np.all(m == (q[:, 0] % 6 == 0))),
           "value": bench.job_value(len(q), world, t)}
    (Path(outdir) / f"r{rank}.json").write_text(json.dumps(res))
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    mp.spawn(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    r = [json.loads((tmp_path / f"r{i}.json").read_text()) for i in range(world)]
    # max over ranks reaches every rank
    assert r[0]["max_t"] == r[1]["max_t"] == 1.5
    # every rank runs rank 0's tuning choice
    assert r[0]["choice"] == r[1]["choice"] == [8, 2, 128, 0]
    # each rank holds a full query set of the same points (weak scaling), in its own order
    assert r[0]["sum"] == r[1]["sum"]
    assert r[0]["first"] != r[1]["first"]
    assert r[0]["near_ok"] and r[1]["near_ok"]  # masks follow their points
    assert r[0]["value"] == pytest.approx(2 * 64 / 1.5)
